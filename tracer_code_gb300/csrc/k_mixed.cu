// k_mixed.cu -- FP32 multigrid of the mixed-precision solve and the bridges
// between it and the FP64 streamfunction.
//
// The mixed solve runs the reference's W-cycle (multigrid,
// iterative_solver.f90:79-173) as defect correction.  Level 1 keeps the
// streamfunction psi, its RHS, the 13 folded coefficient planes and the
// residual in FP64.  Each level-1 visit smooths the correction equation
// L e = r in FP32 from e = 0 with r = RHS - L psi rounded to FP32
// (k_residual_to32), then adds e to psi in FP64 (k_update64) and the FP64
// residual of the new psi takes the reference's convergence test.  Levels
// 2..grids-1 hold FP32 corrections exactly as the reference holds FP64 ones
// (same sweeps, restriction, prolongation), the coarsest direct solve
// applies the FP64 inverse to the FP32 RHS, and the last prolongation adds
// the FP32 correction of level 2 to psi in FP64 (k_prolong_into64).  Since
// the smoother is linear, an exact-arithmetic run of this sequence produces
// the same iterates as the reference's; rounding enters only through the
// corrections, which the FP64 residual of every cycle measures.
//
// Sizes and traffic: a level-l FP32 sweep moves 13 coefficient + RHS + dt +
// psi-in + psi-out floats = 68 B per point (half the FP64 sweep's 136 B);
// at 1024x256 the level-1 FP32 working set (17.8 MB) stays in L2.
#include "tc_device.cuh"

namespace {

__global__ void k_to_f32(const double* __restrict__ in, float* __restrict__ out, size_t n) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t st = (size_t)gridDim.x * blockDim.x;
    for (; t < n; t += st) out[t] = (float)in[t];
}
void to_f32(cudaStream_t s, const double* in, float* out, size_t n) {
    int nb = (int)((n + 255) / 256);
    if (nb > 2432) nb = 2432;
    k_to_f32<<<nb, 256, 0, s>>>(in, out, n); tc_note_launch();
}

__global__ void __launch_bounds__(256, 1) k_sweep32(Lay L, Range2 r, const float* Sin,
                                                   float* Sout, const float* __restrict__ coef, const float* rhs,
                          const float* __restrict__ dts, const float* __restrict__ cA, const float* __restrict__ cB,
                          float c_uniform, int per_point, float temp, int Vbc) {
    RANGE_IK_DYN(r);
    const size_t x = inr ? IX(L, i, k) : 0;
    // coefficients, dt and Chebyshev denominators do not change within a solve
    float cf[TC_NCOEF], dt = 0.f, ca = 1.f, cb = 0.f;
    if (inr) {
        fold_coefs<float>(L, coef, x, cf);
        dt = __ldg(dts + x);
        if (per_point) {
            ca = __ldg(cA + x);
            cb = __ldg(cB + x);
        }
    }
    pdl_entry();
    if (!inr) return;
    const float res = fold_apply<float>(L, Sin, x, cf, ld_state(rhs + x));
    const float c = per_point ? 2.0f / (ca + cb * temp) : c_uniform;
    const float v = fmaf(c * dt, res, ld_state(Sin + x));
    store_stream<float>(L, Sout, i, k, v, Vbc);
    pdl_done();
}

// Level-1 FP32 sweep that forms its 13 coefficients from the five viscosity
// fields in registers (42 multiply-adds per point, the structural zeros of
// the stencil skipped) instead of reading 13 coefficient planes: 24 B of
// coefficient and dt data per point where the folded planes take 56 B.
// Two points per thread (rows k, k+1) share their vertical taps; the taps
// and their order are k_sweep_x2's, so only the coefficients' rounding
// differs from the folded FP32 sweep (FP32 sums of FP32-rounded fields
// instead of FP32 roundings of FP64 sums).
__global__ void __launch_bounds__(256, 1) k_sweep_g32(Lay L, Range2 r, FoldG32 F, const float* Sin, float* Sout,
                                                      const float* __restrict__ g, const float* rhs,
                                                      const float* __restrict__ dts, const float* __restrict__ cA,
                                                      const float* __restrict__ cB, float c_uniform, int per_point,
                                                      float temp, int Vbc) {
    const int i = r.i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = r.k0 + 2 * (int)(blockIdx.y * blockDim.y + threadIdx.y);
    bool act[2];
    act[0] = (i <= r.i1) && (k <= r.k1);
    act[1] = act[0] && (k + 1 <= r.k1);
    const size_t ld = (size_t)L.ld, pl = L.plane;
    const size_t x = act[0] ? IX(L, i, k) : 0;
    float cf[2][TC_NCOEF], dt[2], ca[2], cb[2];
#pragma unroll
    for (int p = 0; p < 2; p++) {
        const size_t xp = act[p] ? x + p * ld : x;
        float G[5];
#pragma unroll
        for (int j = 0; j < 5; j++) G[j] = act[p] ? __ldg(g + xp + j * pl) : 0.f;
        fold_from_fields(F, G, cf[p]);
        dt[p] = act[p] ? __ldg(dts + xp) : 0.f;
        ca[p] = (act[p] && per_point) ? __ldg(cA + xp) : 1.f;
        cb[p] = (act[p] && per_point) ? __ldg(cB + xp) : 0.f;
    }
    pdl_entry();
    if (!act[0]) return;
    // centre column rows k-2..k+3, columns i+-1 rows k-1..k+2, i+-2 rows k..k+1
    const float* s = Sin + x;
    float v0[6], vm1[4], vp1[4], vm2[2], vp2[2], rh[2];
#pragma unroll
    for (int q = 0; q < 6; q++) v0[q] = ld_state(s + (ptrdiff_t)(q - 2) * (ptrdiff_t)ld);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        vm1[q] = ld_state(s + (ptrdiff_t)(q - 1) * (ptrdiff_t)ld - 1);
        vp1[q] = ld_state(s + (ptrdiff_t)(q - 1) * (ptrdiff_t)ld + 1);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        vm2[q] = ld_state(s + (ptrdiff_t)q * (ptrdiff_t)ld - 2);
        vp2[q] = ld_state(s + (ptrdiff_t)q * (ptrdiff_t)ld + 2);
        rh[q] = act[q] ? ld_state(rhs + x + q * ld) : 0.f;
    }
    // the folded operator's tap order (fold_apply)
    float acc[2];
#pragma unroll
    for (int p = 0; p < 2; p++) {
        float a = fmaf(cf[p][0], v0[p + 2], rh[p]);
        a = fmaf(cf[p][1], vm1[p + 1], a);
        a = fmaf(cf[p][2], vp1[p + 1], a);
        a = fmaf(cf[p][3], vm2[p], a);
        a = fmaf(cf[p][4], vp2[p], a);
        a = fmaf(cf[p][5], v0[p + 1], a);
        a = fmaf(cf[p][6], v0[p + 3], a);
        a = fmaf(cf[p][7], v0[p], a);
        a = fmaf(cf[p][8], v0[p + 4], a);
        a = fmaf(cf[p][9], vm1[p], a);
        a = fmaf(cf[p][10], vp1[p], a);
        a = fmaf(cf[p][11], vm1[p + 2], a);
        acc[p] = fmaf(cf[p][12], vp1[p + 2], a);
    }
#pragma unroll
    for (int p = 0; p < 2; p++) {
        if (!act[p]) continue;
        const float c = per_point ? 2.0f / (ca[p] + cb[p] * temp) : c_uniform;
        store_stream<float>(L, Sout, i, k + p, fmaf(c * dt[p], acc[p], v0[p + 2]), Vbc);
    }
    pdl_done();
}

// the five fields G of k_sweep_g32 at the interior points, rounded to FP32
__global__ void k_level_g32(Lay L, Range2 r, const double* __restrict__ V, const double* __restrict__ vx,
                            const double* __restrict__ vz, const double* __restrict__ vxx,
                            const double* __restrict__ vzz, const double* __restrict__ vxz, float* __restrict__ g) {
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(L, i, k), pl = L.plane;
    g[x] = (float)(vxx[x] - vzz[x]);
    g[x + pl] = (float)V[x];
    g[x + 2 * pl] = (float)vxz[x];
    g[x + 3 * pl] = (float)vx[x];
    g[x + 4 * pl] = (float)vz[x];
}

__global__ void __launch_bounds__(256, 1) k_residual32(Lay L, Range2 r, const float* S, const float* __restrict__ coef,
                             const float* rhs, float* res) {
    RANGE_IK(r);
    const size_t x = inr ? IX(L, i, k) : 0;
    float cf[TC_NCOEF];
    if (inr) fold_coefs<float>(L, coef, x, cf);
    pdl_entry();
    if (!inr) return;
    res[x] = fold_apply<float>(L, S, x, cf, ld_state(rhs + x));
    pdl_done();
}

// zero[0..zn) = 0 over the whole launch (grid-stride), so a correction plane
// can be cleared in the same kernel that writes its level's RHS
template <typename T>
__device__ __forceinline__ void zero_plane(T* __restrict__ z, size_t zn) {
    if (z == nullptr) return;
    const size_t nt = (size_t)gridDim.x * gridDim.y * blockDim.x * blockDim.y;
    const size_t t0 = ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x * blockDim.y +
                      (size_t)threadIdx.y * blockDim.x + threadIdx.x;
    for (size_t t = t0; t < zn; t += nt) z[t] = T(0);
}

template <typename Tin>
__global__ void k_restrict_to32(Lay C, Lay F, Range2 r, const Tin* rf, float* rc,
                                float* zero, size_t zn) {
    pdl_entry();
    zero_plane(zero, zn);
    RANGE_IK(r);
    if (!inr) return;
    rc[IX(C, i, k)] = (float)restrict9<Tin>(rf, F, 2 * i, 2 * k);
    pdl_done();
}

// bilinear prolongation value of the coarse correction at fine (i,k)
template <typename T>
__device__ __forceinline__ T prolong_value(const Lay& C, const float* __restrict__ ec, int i, int k) {
    const bool ie = (i % 2) == 0, ke = (k % 2) == 0;
    if (ie && ke) return (T)ld_state(ec + IX(C, i / 2, k / 2));
    if (ie) return ((T)ld_state(ec + IX(C, i / 2, (k - 1) / 2)) + (T)ld_state(ec + IX(C, i / 2, (k + 1) / 2))) / T(2);
    if (ke) return ((T)ld_state(ec + IX(C, (i - 1) / 2, k / 2)) + (T)ld_state(ec + IX(C, (i + 1) / 2, k / 2))) / T(2);
    return ((T)ld_state(ec + IX(C, (i - 1) / 2, (k - 1) / 2)) + (T)ld_state(ec + IX(C, (i + 1) / 2, (k - 1) / 2)) +
            (T)ld_state(ec + IX(C, (i + 1) / 2, (k + 1) / 2)) + (T)ld_state(ec + IX(C, (i - 1) / 2, (k + 1) / 2))) / T(4);
}

template <typename T>
__global__ void k_prolong_add(Lay C, Lay F, Range2 r, const float* ec, T* ef, int Vbc) {
    pdl_entry();
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(F, i, k);
    store_stream<T>(F, ef, i, k, ld_state(ef + x) + prolong_value<T>(C, ec, i, k), Vbc);
    pdl_done();
}

// FP64 residual of psi, rounded to FP32 as the RHS of the level-1 correction
__global__ void __launch_bounds__(256, 1) k_residual_to32(Lay L, Range2 r, const double* S, const double* __restrict__ coef,
                                const double* rhs, float* rhs32,
                                float* zero, size_t zn) {
    pdl_entry();
    zero_plane(zero, zn);
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(L, i, k);
    rhs32[x] = (float)folded_residual<double>(L, S, coef, ld_state(rhs + x), x);
    pdl_done();
}

// psi += e in FP64, ghosts from the new interior value
__global__ void k_update64(Lay L, Range2 r, double* S, const float* e, int Vbc) {
    pdl_entry();
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(L, i, k);
    store_stream<double>(L, S, i, k, ld_state(S + x) + (double)ld_state(e + x), Vbc);
    pdl_done();
}

// coarsest level: x = A^-1 (RowB .* rhs) in FP64 from the FP32 RHS, stored as FP32
// (one warp per interior unknown; cq/cx list the interior unknowns)
__global__ void k_coarse_apply32(Lay L, const double* __restrict__ Ainv, const double* __restrict__ rowb,
                                 const float* rhs, int n, const int* __restrict__ cq, const int* __restrict__ cx,
                                 int m, float* err, int Vbc) {
    pdl_entry();
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= m) return;
    const int pw = __ldg(cq + w), N = L.b + 1;
    const double* row = Ainv + (size_t)pw * n;
    double acc = 0.0;
    for (int e = lane; e < m; e += 32) {
        const int q = __ldg(cq + e);
        acc = fma(__ldg(row + q), (double)ld_state(rhs + __ldg(cx + e)) * __ldg(rowb + q), acc);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) store_stream<float>(L, err, pw / N, pw % N, (float)acc, Vbc);
    pdl_done();
}

Range2 interior(const Lay& L) { return Range2{1, L.a - 1, 1, L.b - 1}; }

}  // namespace

void launch_level_to_f32(cudaStream_t s, const Level& lv, int cheb) {
    to_f32(s, lv.coef, lv.coef32, (size_t)TC_NCOEF * lv.L.plane);
    to_f32(s, lv.dt_stream, lv.dts32, lv.L.plane);
    if (cheb) {
        to_f32(s, lv.cA, lv.cA32, lv.L.plane);
        to_f32(s, lv.cB, lv.cB32, lv.L.plane);
    }
}

// Weights of k_sweep_g32 from the level's FP64 fold basis: g = (G0, G1, 2 G1,
// 4 G2, 2 G3, 2 G4) in k_level_coefs, so w = (f0, f1 + 2 f2, 4 f3, 2 f4, 2 f5)
// (formed in FP64, then rounded).  False when an entry outside the mask is
// not exactly zero.
bool fold_g32_weights(const LevConst& c, FoldG32* out) {
    const unsigned mask[TC_NCOEF] = TC_FOLD_G32_MASK;
    for (int d = 0; d < TC_NCOEF; d++) {
        const double* f = c.fold[d];
        const double w[5] = {f[0], f[1] + 2.0 * f[2], 4.0 * f[3], 2.0 * f[4], 2.0 * f[5]};
        for (int j = 0; j < 5; j++) {
            if (!((mask[d] >> j) & 1u) && w[j] != 0.0) return false;
            out->w[d][j] = (float)w[j];
        }
    }
    return true;
}

void launch_level_g32(cudaStream_t s, const Level& lv, const double* vis) {
    const Range2 r = interior(lv.L);
    k_level_g32<<<grid_for(r), dim3(BX, BY), 0, s>>>(lv.L, r, vis, lv.vx, lv.vz, lv.vxx, lv.vzz, lv.vxz, lv.g32);
    tc_note_launch();
}

static constexpr bool kSweep32Pairs = true;  // k_sweep_x2 (two points per thread) for the per-sweep FP32 smoother
void launch_sweep32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, float c_uniform, int per_point,
                    float temp, int Vbc) {
    const Range2 r = interior(lv.L);
    if (lv.g32 != nullptr && lv.use_g32) {
        dim3 g = grid_for_shape(r, lv.sweep_bx, 2 * lv.sweep_by);
        launch_pdl(k_sweep_g32, g, dim3(lv.sweep_bx, lv.sweep_by), 0, s, lv.L, r, lv.gw, Sin, Sout,
                   (const float*)lv.g32, (const float*)lv.rhs32, (const float*)lv.dts32, (const float*)lv.cA32,
                   (const float*)lv.cB32, c_uniform, per_point, temp, Vbc);
    } else if (kSweep32Pairs) {
        dim3 g = grid_for_shape(r, lv.sweep_bx, 2 * lv.sweep_by);
        launch_pdl(k_sweep_x2<float>, g, dim3(lv.sweep_bx, lv.sweep_by), 0, s, lv.L, r, Sin, Sout, lv.coef32, lv.rhs32,
                   lv.dts32, lv.cA32, lv.cB32, c_uniform, per_point, temp, Vbc);
    } else {
        launch_pdl(k_sweep32, grid_for_shape(r, lv.sweep_bx, lv.sweep_by), dim3(lv.sweep_bx, lv.sweep_by), 0, s, lv.L,
                   r, Sin, Sout, lv.coef32, lv.rhs32, lv.dts32, lv.cA32, lv.cB32, c_uniform, per_point, temp, Vbc);
    }
    tc_note_launch();
}

void launch_residual32(cudaStream_t s, const Level& lv, const float* S) {
    const Range2 r = interior(lv.L);
    launch_pdl(k_residual32, grid_for(r), dim3(BX, BY), 0, s, lv.L, r, S, lv.coef32, lv.rhs32, lv.res32); tc_note_launch();
}

void launch_restrict32(cudaStream_t s, const Level& coarse, const Level& fine, const float* rf, float* rhs_c,
                       float* zero) {
    const Range2 r = interior(coarse.L);
    launch_pdl(k_restrict_to32<float>, grid_for(r), dim3(BX, BY), 0, s, coarse.L, fine.L, r, rf, rhs_c, zero,
               zero ? coarse.L.plane : (size_t)0);
    tc_note_launch();
}

void launch_restrict64to32(cudaStream_t s, const Level& coarse, const Level& fine, const double* rf, float* rhs_c,
                           float* zero) {
    const Range2 r = interior(coarse.L);
    launch_pdl(k_restrict_to32<double>, grid_for(r), dim3(BX, BY), 0, s, coarse.L, fine.L, r, rf, rhs_c, zero,
               zero ? coarse.L.plane : (size_t)0);
    tc_note_launch();
}

void launch_prolong32(cudaStream_t s, const Level& coarse, const Level& fine, const float* ec, float* ef, int Vbc) {
    const Range2 r = interior(fine.L);
    launch_pdl(k_prolong_add<float>, grid_for(r), dim3(BX, BY), 0, s, coarse.L, fine.L, r, ec, ef, Vbc); tc_note_launch();
}

void launch_prolong_into64(cudaStream_t s, const Level& coarse, const Level& fine, const float* ec, double* S,
                           int Vbc) {
    const Range2 r = interior(fine.L);
    launch_pdl(k_prolong_add<double>, grid_for(r), dim3(BX, BY), 0, s, coarse.L, fine.L, r, ec, S, Vbc); tc_note_launch();
}

void launch_residual_to32(cudaStream_t s, const Level& lv, const double* S, float* rhs32, float* zero) {
    const Range2 r = interior(lv.L);
    launch_pdl(k_residual_to32, grid_for(r), dim3(BX, BY), 0, s, lv.L, r, S, lv.coef, lv.rhs, rhs32, zero,
               zero ? lv.L.plane : (size_t)0);
    tc_note_launch();
}

void launch_update64(cudaStream_t s, const Level& lv, double* S, const float* e, int Vbc) {
    const Range2 r = interior(lv.L);
    launch_pdl(k_update64, grid_for(r), dim3(BX, BY), 0, s, lv.L, r, S, e, Vbc); tc_note_launch();
}

void launch_coarse_apply32(cudaStream_t s, const Level& lv, const double* Ainv, const double* rowb, int n,
                           const int* cq, const int* cx, int m, float* err, int Vbc) {
    const int threads = 256;
    const unsigned nb = (unsigned)((m * 32 + threads - 1) / threads);
    launch_pdl(k_coarse_apply32, nb, threads, 0, s, lv.L, Ainv, rowb, lv.rhs32, n, cq, cx, m, err, Vbc); tc_note_launch();
}
