// k_subcycle.cu -- the bottom of the W-cycle as a precomputed matrix.
//
// In the reference's W-cycles (multigrid_cycle.f90:9-92) every descent into
// level S = grids-1 runs, until the cycle returns to level S-1:
//
//     k times: smooth S (Nmulti sweeps, Chebyshev going down), residual,
//              restrict into the coarsest level G, direct solve on G,
//              prolong the coarse correction and add it to S's correction;
//     then:    smooth S (Nmulti sweeps, Richardson going up)
//
// with k = 1 or 2 (grids = 6: "5 6 5" and "5 6 5 6 5").  When a level's
// correction restarts from zero at every new restricted residual
// (mg_zero_coarse = 1) and the operators are fixed for the solve (Newtonian
// rheology), this is a fixed linear map e_S = M_k r_S of the restricted
// residual r_S: the sweeps, the residual, the transfers and the direct solve
// are all linear.  M_k (n_S x n_S, n_S the interior unknowns of S) is built
// once per multigrid call by running the sub-cycle on the n_S unit vectors,
// one CTA per column, with the per-point arithmetic of the solver's smoother
// kernels (k_sweep, k_residual, restrict9, k_coarse_apply, k_prolong; FP64,
// or in the mixed solve FP32 from its FP32 operator with the coarsest solve
// in FP64) in shared memory; each descent then costs one matrix-vector
// product instead of (2k+1) x Nmulti latency-bound sweeps and k coarse
// solves.  In exact arithmetic the cycle is unchanged; only the
// summation order of the bottom correction differs.  This is the same step
// the coarsest level takes already (an explicit inverse of the banded
// matrix instead of DGBTRS per visit, iterative_solver.f90:138-142).
#include "tc_device.cuh"

namespace {

constexpr int kMaxS = 1024;  // interior points of level S at most
// build CTA: FP32 one point per thread on 1024 threads (32 warps to hide the
// sweeps' latencies); FP64 two points per thread on 512 (its registers)
template <typename T>
struct BuildShape {
    static constexpr int threads = sizeof(T) == sizeof(float) ? 1024 : 512;
    static constexpr int ppt = kMaxS / threads;
};

template <typename T>
struct SubArgs {
    Lay LS, LG;
    const T* coef;  // level S folded operator (TC_NCOEF planes), pseudo-time step, Chebyshev denominators
    const T* dts;
    const T* cA;
    const T* cB;
    const T* tab;  // [4][nsweeps]: c and temp of the sweeps of a downward visit, then of an upward one
    const T* ctab; // per-point Chebyshev factors 2/(cA + cB temp_n) of a downward visit, [nsweeps][nS]
    int nsweeps, per_point_down;
    const double* Ainv;  // coarsest level: explicit inverse, row scaling, interior unknown lists
    const double* rowb;
    const int* cq;
    const int* cx;
    int n, m;
    int Vbc, kmax, nS;
    T* M[4];  // outputs for k = 1..4 (null: not needed)
};

// shared-memory versions of the stencil helpers (same terms in the same order)
template <typename T>
__device__ __forceinline__ T sm_restrict9(const T* in, const Lay& F, int ii, int kk) {
    T corners = (in[IX(F, ii - 1, kk - 1)] + in[IX(F, ii - 1, kk + 1)] + in[IX(F, ii + 1, kk + 1)] +
                 in[IX(F, ii - 1, kk + 1)]) / T(16);
    T sides = (in[IX(F, ii - 1, kk)] + in[IX(F, ii, kk - 1)] + in[IX(F, ii + 1, kk)] + in[IX(F, ii, kk + 1)]) / T(8);
    T centre = in[IX(F, ii, kk)] / T(4);
    return corners + sides + centre;
}

template <typename T>
__device__ __forceinline__ T sm_prolong(const Lay& C, const T* ec, int i, int k) {
    const bool ie = (i % 2) == 0, ke = (k % 2) == 0;
    if (ie && ke) return ec[IX(C, i / 2, k / 2)];
    if (ie) return (ec[IX(C, i / 2, (k - 1) / 2)] + ec[IX(C, i / 2, (k + 1) / 2)]) / T(2);
    if (ke) return (ec[IX(C, (i - 1) / 2, k / 2)] + ec[IX(C, (i + 1) / 2, k / 2)]) / T(2);
    return (ec[IX(C, (i - 1) / 2, (k - 1) / 2)] + ec[IX(C, (i + 1) / 2, (k - 1) / 2)] +
            ec[IX(C, (i + 1) / 2, (k + 1) / 2)] + ec[IX(C, (i - 1) / 2, (k + 1) / 2)]) / T(4);
}

// rhs - L S at x, the 13 taps in folded_residual's order
template <typename T>
__device__ __forceinline__ T sm_apply(const Lay& L, const T* S, size_t x, const T* c, T rhs) {
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    T acc = rhs;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) acc = fma(-c[d], S[(ptrdiff_t)x + off[d]], acc);
    return acc;
}

// The ghost copies store_stream writes for interior point (i, k) besides the
// point itself (at most three when a, b >= 2 SP + 1): their plane offsets and
// signs, in store_stream's order, so that a sweep of the build writes
// v, then sg[g] * v at idx[g] -- the same values, without re-deriving them.
template <typename T>
__device__ __forceinline__ int ghost_targets(const Lay& L, int i, int k, int Vbc, int* idx, T* sg) {
    const int a = L.a, b = L.b;
    int gi[2] = {i, 0};
    T si[2] = {T(1), T(-1)};
    int ng = 1;
    if (i <= SP) gi[ng++] = -i;
    else if (i >= a - SP) gi[ng++] = 2 * a - i;
    int gk[2] = {k, 0};
    const T zsgn = (Vbc == 1) ? T(1) : T(-1);
    T sk[2] = {T(1), zsgn};
    int nk = 1;
    if (k <= SP) gk[nk++] = -k;
    else if (k >= b - SP) gk[nk++] = 2 * b - k;
    int n = 0;
    for (int u = 0; u < nk; u++)
        for (int t = 0; t < ng; t++) {
            if (u == 0 && t == 0) continue;
            idx[n] = (int)IX(L, gi[t], gk[u]);
            sg[n] = si[t] * sk[u];
            n++;
        }
    return n;
}

template <typename T>
__global__ void __launch_bounds__(BuildShape<T>::threads, 1) k_subcycle_build(SubArgs<T> A) {
    constexpr int kThreads = BuildShape<T>::threads, kPPT = BuildShape<T>::ppt;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* P0 = reinterpret_cast<T*>(smem_raw);
    T* P1 = P0 + A.LS.plane;
    T* P2 = P1 + A.LS.plane;
    T* R = P2 + A.LS.plane;
    T* RG = R + A.LS.plane;
    T* EG = RG + A.LG.plane;
    const int tid = threadIdx.x;
    const int nS = A.nS;
    const int a1 = A.LS.a - 1;
    const int j = blockIdx.x;  // column: interior point j of level S (i fastest)
    const size_t total = 4 * A.LS.plane + 2 * A.LG.plane;
    for (size_t t = tid; t < total; t += blockDim.x) P0[t] = T(0);
    // this thread's points of level S, their operator, dt, ghost copies and
    // RHS (the unit vector of column j) in registers
    int pi[kPPT], pk[kPPT];
    size_t px[kPPT];
    bool pa[kPPT];
    T cf[kPPT][TC_NCOEF], dt[kPPT], rq[kPPT];
    int gn[kPPT], gidx[kPPT][3];
    T gsg[kPPT][3];
    // threads in rows of rpad slots (a1 rounded up to whole warps) when
    // that many fit, so that no warp's taps straddle two rows (which puts
    // two lanes on one shared-memory bank); else a1 slots per row
    const int b1 = A.LS.b - 1;
    const int rpad = (((a1 + 31) & ~31) * b1 <= kThreads * kPPT) ? ((a1 + 31) & ~31) : a1;
    int pidx[kPPT];  // interior point index (i fastest over a1), the matrix's row order
#pragma unroll
    for (int q = 0; q < kPPT; q++) {
        const int slot = tid + q * kThreads, si = slot % rpad, sk = slot / rpad;
        pa[q] = si < a1 && sk < b1;
        pi[q] = pa[q] ? 1 + si : 1;
        pk[q] = pa[q] ? 1 + sk : 1;
        pidx[q] = pa[q] ? sk * a1 + si : 0;
        const int p = pidx[q];
        px[q] = IX(A.LS, pi[q], pk[q]);
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[q][d] = pa[q] ? __ldg(A.coef + px[q] + d * A.LS.plane) : T(0);
        dt[q] = pa[q] ? __ldg(A.dts + px[q]) : T(0);
        rq[q] = (pa[q] && p == j) ? T(1) : T(0);
        gn[q] = pa[q] ? ghost_targets<T>(A.LS, pi[q], pk[q], A.Vbc, gidx[q], gsg[q]) : 0;
    }
    __syncthreads();
    if (tid == 0) R[IX(A.LS, 1 + j % a1, 1 + j / a1)] = T(1);
    __syncthreads();
    // store_stream of v at this thread's point q into S
    auto put = [&](T* S, int q, T v) {
        S[px[q]] = v;
        for (int g = 0; g < gn[q]; g++) S[gidx[q][g]] = gsg[q][g] * v;
    };
    // one visit of Nmulti sweeps from Sa (ping-pong with Sb); returns the plane holding the result
    auto visit = [&](T* Sa, T* Sb, int up) -> T* {
        const T* cv = A.tab + (up ? 2 : 0) * A.nsweeps;
        const bool pp = !up && A.per_point_down;
        // the sweep's factors are loaded one sweep ahead (their latency is
        // not on the sweep-to-sweep path)
        T cnext[kPPT];
        T cunext = __ldg(cv);
#pragma unroll
        for (int q = 0; q < kPPT; q++) cnext[q] = (pp && pa[q]) ? __ldg(A.ctab + pidx[q]) : T(0);
        for (int n = 0; n < A.nsweeps; n++) {
            const T cu = cunext;
            T cpp[kPPT];
#pragma unroll
            for (int q = 0; q < kPPT; q++) cpp[q] = cnext[q];
            if (n + 1 < A.nsweeps) {
                cunext = __ldg(cv + n + 1);
#pragma unroll
                for (int q = 0; q < kPPT; q++)
                    if (pp && pa[q]) cnext[q] = __ldg(A.ctab + (size_t)(n + 1) * nS + pidx[q]);
            }
#pragma unroll
            for (int q = 0; q < kPPT; q++) {
                if (!pa[q]) continue;
                const T res = sm_apply(A.LS, Sa, px[q], cf[q], rq[q]);
                // the per-point factor from the table (the same correctly rounded
                // division as k_sweep's, done once per solve)
                const T c = pp ? cpp[q] : cu;
                put(Sb, q, fma(c * dt[q], res, Sa[px[q]]));
            }
            __syncthreads();
            T* t = Sa;
            Sa = Sb;
            Sb = t;
        }
        return Sa;
    };
    const int lane = tid & 31, warp = tid >> 5, nwarps = kThreads / 32;
    const int NG = A.LG.b + 1;
    for (int blk = 1; blk <= A.kmax; blk++) {
        // smooth S going down; the result back in P0
        T* e = visit(P0, P1, 0);
        if (e != P0) {
            for (size_t t = tid; t < A.LS.plane; t += blockDim.x) P0[t] = e[t];
            __syncthreads();
        }
        // residual into P1, restricted into the coarsest RHS
#pragma unroll
        for (int q = 0; q < kPPT; q++)
            if (pa[q]) P1[px[q]] = sm_apply(A.LS, P0, px[q], cf[q], rq[q]);
        __syncthreads();
        for (int c = tid; c < (A.LG.a - 1) * (A.LG.b - 1); c += blockDim.x) {
            const int ic = 1 + c % (A.LG.a - 1), kc = 1 + c / (A.LG.a - 1);
            RG[IX(A.LG, ic, kc)] = sm_restrict9(P1, A.LS, 2 * ic, 2 * kc);
        }
        __syncthreads();
        // direct solve x = A^-1 (RowB .* rhs): one warp per unknown, lane-strided sum and shuffle tree
        for (int w = warp; w < A.m; w += nwarps) {
            const int pw = __ldg(A.cq + w);
            const double* row = A.Ainv + (size_t)pw * A.n;
            double acc = 0.0;
            for (int e2 = lane; e2 < A.m; e2 += 32) {
                const int q = __ldg(A.cq + e2);
                acc = fma(__ldg(row + q), (double)RG[__ldg(A.cx + e2)] * __ldg(A.rowb + q), acc);
            }
            for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
            if (lane == 0) store_stream<T>(A.LG, EG, pw / NG, pw % NG, (T)acc, A.Vbc);
        }
        __syncthreads();
        // prolong the coarse correction and add it to S's
#pragma unroll
        for (int q = 0; q < kPPT; q++)
            if (pa[q]) put(P0, q, P0[px[q]] + sm_prolong<T>(A.LG, EG, pi[q], pk[q]));
        __syncthreads();
        T* out = A.M[blk - 1];
        if (out != nullptr) {
            // this pattern ends here: smooth S going up from a copy, column j of M_blk
            for (size_t t = tid; t < A.LS.plane; t += blockDim.x) P1[t] = P0[t];
            __syncthreads();
            T* f = visit(P1, P2, 1);
            for (int p = tid; p < nS; p += blockDim.x)
                out[(size_t)p * nS + j] = f[IX(A.LS, 1 + p % a1, 1 + p / a1)];
            __syncthreads();
        }
    }
}

// ---- FP32 build, four columns per CTA --------------------------------------------
// The mixed solve's build (k_subcycle_build<float>'s arithmetic per column)
// on four unit vectors at once: every shared-memory plane holds the four
// columns' values of a point in one float4, so a sweep's 13 tap loads serve
// four columns, and the coefficients, ghost targets and factors are shared.
// The coarsest solve uses the compact FP32 inverse Ac (Ac[e][e2] = A^-1 at
// the interior unknowns cq[e], cq[e2], times the row scale rowb[cq[e2]]):
// the matrix is stored in FP32 anyway, and an FP64 solve of 945 x 2
// right-hand sides costs about 150 us of the FP64 pipe per build.
__device__ __forceinline__ float4 f4_fma(float c, float4 v, float4 a) {
    return make_float4(fmaf(c, v.x, a.x), fmaf(c, v.y, a.y), fmaf(c, v.z, a.z), fmaf(c, v.w, a.w));
}
__device__ __forceinline__ float4 f4_scale(float c, float4 v) { return make_float4(c * v.x, c * v.y, c * v.z, c * v.w); }
__device__ __forceinline__ float4 f4_add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 f4_div(float4 a, float d) { return make_float4(a.x / d, a.y / d, a.z / d, a.w / d); }

// sm_restrict9 per component (same terms, same order)
__device__ __forceinline__ float4 sm_restrict9_4(const float4* in, const Lay& F, int ii, int kk) {
    const float4 c0 = in[IX(F, ii - 1, kk - 1)], c1 = in[IX(F, ii - 1, kk + 1)], c2 = in[IX(F, ii + 1, kk + 1)],
                 c3 = in[IX(F, ii - 1, kk + 1)];
    const float4 s0 = in[IX(F, ii - 1, kk)], s1 = in[IX(F, ii, kk - 1)], s2 = in[IX(F, ii + 1, kk)],
                 s3 = in[IX(F, ii, kk + 1)];
    const float4 cc = in[IX(F, ii, kk)];
    const float4 corners = f4_div(f4_add(f4_add(f4_add(c0, c1), c2), c3), 16.f);
    const float4 sides = f4_div(f4_add(f4_add(f4_add(s0, s1), s2), s3), 8.f);
    const float4 centre = f4_div(cc, 4.f);
    return f4_add(f4_add(corners, sides), centre);
}
// sm_prolong per component
__device__ __forceinline__ float4 sm_prolong4(const Lay& C, const float4* ec, int i, int k) {
    const bool ie = (i % 2) == 0, ke = (k % 2) == 0;
    if (ie && ke) return ec[IX(C, i / 2, k / 2)];
    if (ie) return f4_div(f4_add(ec[IX(C, i / 2, (k - 1) / 2)], ec[IX(C, i / 2, (k + 1) / 2)]), 2.f);
    if (ke) return f4_div(f4_add(ec[IX(C, (i - 1) / 2, k / 2)], ec[IX(C, (i + 1) / 2, k / 2)]), 2.f);
    return f4_div(f4_add(f4_add(f4_add(ec[IX(C, (i - 1) / 2, (k - 1) / 2)], ec[IX(C, (i + 1) / 2, (k - 1) / 2)]),
                                ec[IX(C, (i + 1) / 2, (k + 1) / 2)]),
                         ec[IX(C, (i - 1) / 2, (k + 1) / 2)]),
                  4.f);
}
// store_stream per component
__device__ __forceinline__ void store_stream4(const Lay& L, float4* S, int i, int k, float4 v, int Vbc) {
    int idx[3];
    float sg[3];
    const int n = ghost_targets<float>(L, i, k, Vbc, idx, sg);
    S[IX(L, i, k)] = v;
    for (int g = 0; g < n; g++) S[idx[g]] = f4_scale(sg[g], v);
}

__global__ void __launch_bounds__(1024, 1) k_subcycle_build4(SubArgs<float> A, const float* __restrict__ Ac) {
    constexpr int kThreads = 1024;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* P0 = reinterpret_cast<float4*>(smem_raw);
    float4* P1 = P0 + A.LS.plane;
    float4* P2 = P1 + A.LS.plane;
    float4* RG = P2 + A.LS.plane;
    float4* EG = RG + A.LG.plane;
    const int tid = threadIdx.x;
    const int nS = A.nS;
    const int a1 = A.LS.a - 1, b1 = A.LS.b - 1;
    const int j0 = blockIdx.x * 4;  // columns j0 .. j0 + 3 (those below nS)
    const size_t total = 3 * A.LS.plane + 2 * A.LG.plane;
    for (size_t t = tid; t < total; t += blockDim.x) P0[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int rpad = (((a1 + 31) & ~31) * b1 <= kThreads) ? ((a1 + 31) & ~31) : a1;
    const int si = tid % rpad, sk = tid / rpad;
    const bool pa = si < a1 && sk < b1;
    const int pi = pa ? 1 + si : 1, pk = pa ? 1 + sk : 1;
    const int pidx = pa ? sk * a1 + si : 0;
    const size_t px = IX(A.LS, pi, pk);
    float cf[TC_NCOEF], dt;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) cf[d] = pa ? __ldg(A.coef + px + d * A.LS.plane) : 0.f;
    dt = pa ? __ldg(A.dts + px) : 0.f;
    const float4 rq = make_float4(pa && pidx == j0 ? 1.f : 0.f, pa && pidx == j0 + 1 ? 1.f : 0.f,
                                  pa && pidx == j0 + 2 ? 1.f : 0.f, pa && pidx == j0 + 3 ? 1.f : 0.f);
    int gidx[3];
    float gsg[3];
    const int gn = pa ? ghost_targets<float>(A.LS, pi, pk, A.Vbc, gidx, gsg) : 0;
    __syncthreads();
    auto put = [&](float4* S, float4 v) {
        S[px] = v;
        for (int g = 0; g < gn; g++) S[gidx[g]] = f4_scale(gsg[g], v);
    };
    const ptrdiff_t ld = (ptrdiff_t)A.LS.ld;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    // rhs - L S at this thread's point, per column (sm_apply's order)
    auto apply = [&](const float4* S, float4 rhs) {
        float4 acc = rhs;
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) acc = f4_fma(-cf[d], S[(ptrdiff_t)px + off[d]], acc);
        return acc;
    };
    auto visit = [&](float4* Sa, float4* Sb, int up) -> float4* {
        const float* cv = A.tab + (up ? 2 : 0) * A.nsweeps;
        const bool pp = !up && A.per_point_down;
        float cunext = __ldg(cv);
        float cnext = (pp && pa) ? __ldg(A.ctab + pidx) : 0.f;
        for (int n = 0; n < A.nsweeps; n++) {
            const float cu = cunext, cpp = cnext;
            if (n + 1 < A.nsweeps) {
                cunext = __ldg(cv + n + 1);
                if (pp && pa) cnext = __ldg(A.ctab + (size_t)(n + 1) * nS + pidx);
            }
            if (pa) {
                const float4 res = apply(Sa, rq);
                const float c = pp ? cpp : cu;
                const float cd = c * dt;
                const float4 s0 = Sa[px];
                put(Sb, make_float4(fmaf(cd, res.x, s0.x), fmaf(cd, res.y, s0.y), fmaf(cd, res.z, s0.z),
                                    fmaf(cd, res.w, s0.w)));
            }
            __syncthreads();
            float4* t = Sa;
            Sa = Sb;
            Sb = t;
        }
        return Sa;
    };
    const int lane = tid & 31, warp = tid >> 5, nwarps = kThreads / 32;
    const int NG = A.LG.b + 1;
    for (int blk = 1; blk <= A.kmax; blk++) {
        float4* e = visit(P0, P1, 0);
        if (e != P0) {
            for (size_t t = tid; t < A.LS.plane; t += blockDim.x) P0[t] = e[t];
            __syncthreads();
        }
        if (pa) P1[px] = apply(P0, rq);
        __syncthreads();
        for (int c = tid; c < (A.LG.a - 1) * (A.LG.b - 1); c += blockDim.x) {
            const int ic = 1 + c % (A.LG.a - 1), kc = 1 + c / (A.LG.a - 1);
            RG[IX(A.LG, ic, kc)] = sm_restrict9_4(P1, A.LS, 2 * ic, 2 * kc);
        }
        __syncthreads();
        // coarsest solve x = Ac RG (one warp per unknown, lane-strided, shuffle tree)
        for (int w = warp; w < A.m; w += nwarps) {
            const int pw = __ldg(A.cq + w);
            const float* row = Ac + (size_t)w * A.m;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int e2 = lane; e2 < A.m; e2 += 32) acc = f4_fma(__ldg(row + e2), RG[__ldg(A.cx + e2)], acc);
            for (int o = 16; o > 0; o >>= 1) {
                acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
                acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
                acc.z += __shfl_down_sync(0xffffffffu, acc.z, o);
                acc.w += __shfl_down_sync(0xffffffffu, acc.w, o);
            }
            if (lane == 0) store_stream4(A.LG, EG, pw / NG, pw % NG, acc, A.Vbc);
        }
        __syncthreads();
        if (pa) put(P0, f4_add(P0[px], sm_prolong4(A.LG, EG, pi, pk)));
        __syncthreads();
        float* out = A.M[blk - 1];
        if (out != nullptr) {
            for (size_t t = tid; t < A.LS.plane; t += blockDim.x) P1[t] = P0[t];
            __syncthreads();
            const float4* f = visit(P1, P2, 1);
            for (int p = tid; p < nS; p += blockDim.x) {
                const float4 v = f[IX(A.LS, 1 + p % a1, 1 + p / a1)];
                float* o = out + (size_t)p * nS + j0;
                o[0] = v.x;
                if (j0 + 1 < nS) o[1] = v.y;
                if (j0 + 2 < nS) o[2] = v.z;
                if (j0 + 3 < nS) o[3] = v.w;
            }
            __syncthreads();
        }
    }
}

// Ac[e][e2] = Ainv[cq[e] * n + cq[e2]] * rowb[cq[e2]], rounded to FP32
__global__ void k_coarse_compact32(const double* __restrict__ Ainv, const double* __restrict__ rowb,
                                   const int* __restrict__ cq, int m, int n, float* __restrict__ Ac) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m * m) return;
    const int e = t / m, e2 = t % m;
    const int q = cq[e2];
    Ac[t] = (float)(Ainv[(size_t)cq[e] * n + q] * rowb[q]);
}

// e_S = M r_S: one warp per interior unknown p of level S (lane-strided sum
// in FP64, shuffle tree), written with the stream BCs' ghost copies.  The
// product cancels strongly (the sum of the terms' magnitudes is far above
// the result), so it is summed in FP64 whatever the entries' type: FP64
// entries in the FP64 solve (the level-1 correction after one W-cycle within
// 5e-13 of the sweep path's), FP32 entries built from the FP32 operator in
// the mixed solve (after one W-cycle 3.7e-5 from the FP64 cycle's, where the
// FP32 sweeps give 1.9e-4).  The mixed
// solve's FP32 RHS and correction are converted at the load and the store.
//
// The matrix is fixed for the solve, so each warp loads its row into
// registers before waiting for the previous kernel; the RHS is then staged
// once per block in shared memory as FP64 (one conversion and one index
// computation per entry and block, not per entry and row).
template <typename TM, typename TV>
__global__ void __launch_bounds__(256) k_subcycle_apply(Lay L, const TM* __restrict__ M, const TV* rhs, TV* err,
                                                        int nS, int Vbc) {
    constexpr int kPerLane = kMaxS / 32;  // nS <= kMaxS
    __shared__ double r[kMaxS];
    const int lane = threadIdx.x & 31;
    const int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int a1 = L.a - 1;
    TM m[kPerLane];
    {
        const TM* row = M + (size_t)(p < nS ? p : 0) * nS;
#pragma unroll
        for (int q = 0; q < kPerLane; q++) {
            const int jj = lane + 32 * q;
            m[q] = (p < nS && jj < nS) ? __ldg(row + jj) : TM(0);
        }
    }
    pdl_entry();
    for (int jj = threadIdx.x; jj < nS; jj += blockDim.x)
        r[jj] = (double)ld_state(rhs + IX(L, 1 + jj % a1, 1 + jj / a1));
    __syncthreads();
    if (p >= nS) return;
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < kPerLane; q++) {
        const int jj = lane + 32 * q;
        if (jj < nS) acc = fma((double)m[q], r[jj], acc);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) store_stream<TV>(L, err, 1 + p % a1, 1 + p / a1, (TV)acc, Vbc);
    pdl_done();
}

template <typename T>
size_t build_smem(const Lay& LS, const Lay& LG) {
    return sizeof(T) * (4 * LS.plane + 2 * LG.plane);
}

int launch_build4(cudaStream_t s, const SubArgs<float>& A, float* Ac) {
    const size_t smem = sizeof(float4) * (3 * A.LS.plane + 2 * A.LG.plane);
    if (A.nS > kMaxS || smem > 200 * 1024 || Ac == nullptr) return -1;
    const int mm = A.m * A.m;
    k_coarse_compact32<<<(mm + 255) / 256, 256, 0, s>>>(A.Ainv, A.rowb, A.cq, A.m, A.n, Ac);
    tc_note_launch();
    if (cudaFuncSetAttribute(k_subcycle_build4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    k_subcycle_build4<<<(A.nS + 3) / 4, 1024, smem, s>>>(A, Ac);
    tc_note_launch();
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename T>
int launch_build(cudaStream_t s, const SubArgs<T>& A) {
    const size_t smem = build_smem<T>(A.LS, A.LG);
    if (A.nS > kMaxS || smem > 200 * 1024) return -1;
    if (cudaFuncSetAttribute(k_subcycle_build<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return -1;
    k_subcycle_build<T><<<A.nS, BuildShape<T>::threads, smem, s>>>(A);
    tc_note_launch();
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

int subcycle_fits(const Lay& LS, const Lay& LG) {
    if (LS.a < 2 * SP + 1 || LS.b < 2 * SP + 1) return 0;  // at most one mirror per direction (ghost_targets)
    const int nS = (LS.a - 1) * (LS.b - 1);
    return (nS <= kMaxS && build_smem<double>(LS, LG) <= 200 * 1024) ? 1 : 0;
}

// fp32 = 0: the matrices in FP64 from the level's FP64 operator (tab, ctab
// and M FP64).  fp32 = 1 (the mixed solve): in FP32 from its FP32 operator,
// the arithmetic of its FP32 smoother (tab, ctab and M FP32; the coarsest
// solve FP64 as in k_coarse_apply32).
int launch_subcycle_build(cudaStream_t s, const Level& S, const Level& G, int fp32, const void* tab,
                          const void* ctab, int nsweeps, int per_point_down, const double* Ainv, const double* rowb,
                          const int* cq, const int* cx, int n, int m, int Vbc, int kmax, void* const* M, float* Ac) {
    if (per_point_down && ctab == nullptr) return -1;
    if (kmax < 1 || kmax > 4) return -1;
    if (fp32) {
        SubArgs<float> A{};
        A.LS = S.L; A.LG = G.L;
        A.coef = S.coef32; A.dts = S.dts32; A.cA = S.cA32; A.cB = S.cB32;
        A.tab = (const float*)tab; A.ctab = (const float*)ctab; A.nsweeps = nsweeps;
        A.per_point_down = per_point_down;
        A.Ainv = Ainv; A.rowb = rowb; A.cq = cq; A.cx = cx; A.n = n; A.m = m;
        A.Vbc = Vbc; A.kmax = kmax; A.nS = (S.L.a - 1) * (S.L.b - 1);
        for (int k = 0; k < 4; k++) A.M[k] = (float*)M[k];
        if (Ac != nullptr) return launch_build4(s, A, Ac);
        return launch_build(s, A);
    }
    SubArgs<double> A{};
    A.LS = S.L; A.LG = G.L;
    A.coef = S.coef; A.dts = S.dt_stream; A.cA = S.cA; A.cB = S.cB;
    A.tab = (const double*)tab; A.ctab = (const double*)ctab; A.nsweeps = nsweeps;
    A.per_point_down = per_point_down;
    A.Ainv = Ainv; A.rowb = rowb; A.cq = cq; A.cx = cx; A.n = n; A.m = m;
    A.Vbc = Vbc; A.kmax = kmax; A.nS = (S.L.a - 1) * (S.L.b - 1);
    for (int k = 0; k < 4; k++) A.M[k] = (double*)M[k];
    return launch_build(s, A);
}

// e_S = M r_S in the solver's precision (fp32: FP32 RHS and correction);
// m32: the matrix is FP32; the products are summed in FP64 either way
void launch_subcycle_apply(cudaStream_t s, const Level& S, const void* M, int fp32, int m32, void* err, int Vbc) {
    const int nS = (S.L.a - 1) * (S.L.b - 1);
    const unsigned nb = (unsigned)((nS * 32 + 255) / 256);
    if (fp32 && m32)
        launch_pdl(k_subcycle_apply<float, float>, nb, 256, 0, s, S.L, (const float*)M, (const float*)S.rhs32,
                   (float*)err, nS, Vbc);
    else if (fp32)
        launch_pdl(k_subcycle_apply<double, float>, nb, 256, 0, s, S.L, (const double*)M, (const float*)S.rhs32,
                   (float*)err, nS, Vbc);
    else
        launch_pdl(k_subcycle_apply<double, double>, nb, 256, 0, s, S.L, (const double*)M, (const double*)S.rhs,
                   (double*)err, nS, Vbc);
    tc_note_launch();
}
