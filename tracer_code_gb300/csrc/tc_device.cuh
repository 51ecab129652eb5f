// tc_device.cuh -- device helpers shared by the kernel files.
//
// All kernels are compiled with --fmad=false: plain a*b+c in this code is a
// rounded multiply followed by a rounded add, exactly as in the reference's
// x86-64 gfortran build, so the kernels that the tests compare bit-for-bit
// with the CPU restatement (velocities, Taylor interpolation, RK updates,
// histograms, smoothers) reproduce its rounding.  Where bit-equality is not
// required (the folded multigrid operator) fma() is written explicitly.
#pragma once

#include "tc_internal.h"

#include <math.h>

#define BX 32
#define BY 8

struct Range2 {
    int i0, i1, k0, k1;  // inclusive
};

// metric array a at fine node n (Metric in tc_internal.h)
__device__ __forceinline__ double mt(const double* a, int n) { return a[n + TC_MPAD]; }

// The streamfunction operator of iterative_solver.f90 stream_space on a
// stretched grid, given the computational derivatives q = (Sr, Srr, Srrr,
// Srrrr, Ss, Sss, Ssss, Sssss, Srs, Srrs, Srss, Srrss) at a node whose
// metrics are x1..x4 (xr..xrrrr), x13 = xr**3, x14 = xr**4 and likewise for z,
// and whose viscosity and its x/z derivatives are v, vx, vz, vxx, vzz, vxz;
// the reference's expressions in its order.
__device__ __forceinline__ double stream_op_metric(const double* q, double x1, double x2, double x3, double x4,
                                                   double x13, double x14, double z1, double z2, double z3,
                                                   double z4, double z13, double z14, double v, double vx, double vz,
                                                   double vxx, double vzz, double vxz) {
    const double Sr = q[0], Srr = q[1], Srrr = q[2], Srrrr = q[3], Ss = q[4], Sss = q[5], Ssss = q[6],
                 Sssss = q[7], Srs = q[8], Srrs = q[9], Srss = q[10], Srrss = q[11];
    const double Sx = Sr / x1, Sz = Ss / z1;
    const double Sxx = (Srr - Sx * x2) / (x1 * x1);
    const double Szz = (Sss - Sz * z2) / (z1 * z1);
    const double Sxxx = (Srrr - 3.0 * Sxx * x1 * x2 - Sx * x3) / x13;
    const double Szzz = (Ssss - 3.0 * Szz * z1 * z2 - Sz * z3) / z13;
    const double Sxxxx = (Srrrr - 6.0 * Sxxx * x2 * (x1 * x1) - (3.0 * (x2 * x2) + 4.0 * x1 * x3) * Sxx - Sx * x4) / x14;
    const double Szzzz = (Sssss - 6.0 * Szzz * z2 * (z1 * z1) - (3.0 * (z2 * z2) + 4.0 * z1 * z3) * Szz - Sz * z4) / z14;
    const double Sxz = Srs / x1 / z1;
    const double Sxxz = (Srrs - Sxz * z1 * x2) / z1 / (x1 * x1);
    const double Sxzz = (Srss - Sxz * x1 * z2) / x1 / (z1 * z1);
    const double Sxxzz =
        (Srrss - Sxzz * x2 * (z1 * z1) - Sxxz * z2 * (x1 * x1) - Sxz * x2 * z2) / ((x1 * z1) * (x1 * z1));
    const double t1 = (vxx - vzz) * (Sxx - Szz);
    const double t2 = v * (Sxxxx + Szzzz);
    const double t3 = 2.0 * v * Sxxzz;
    const double t4 = 4.0 * vxz * Sxz;
    const double t5 = 2.0 * vx * (Sxxx + Sxzz);
    const double t6 = 2.0 * vz * (Szzz + Sxxz);
    return t1 + t2 + t3 + t4 + t5 + t6;
}

inline dim3 grid_for(const Range2& r) {
    int ni = r.i1 - r.i0 + 1, nk = r.k1 - r.k0 + 1;
    if (ni < 1) ni = 1;
    if (nk < 1) nk = 1;
    return dim3((unsigned)((ni + BX - 1) / BX), (unsigned)((nk + BY - 1) / BY), 1);
}
inline int nblocks_of(const Range2& r) {
    dim3 g = grid_for(r);
    return (int)(g.x * g.y);
}

#define RANGE_IK(r)                                    \
    const int i = (r).i0 + (int)(blockIdx.x * BX + threadIdx.x); \
    const int k = (r).k0 + (int)(blockIdx.y * BY + threadIdx.y); \
    const bool inr = (i <= (r).i1) && (k <= (r).k1);
// the same for kernels launched with a tuned block shape (blockDim.x x blockDim.y)
#define RANGE_IK_DYN(r)                                \
    const int i = (r).i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x); \
    const int k = (r).k0 + (int)(blockIdx.y * blockDim.y + threadIdx.y); \
    const bool inr = (i <= (r).i1) && (k <= (r).k1);
inline dim3 grid_for_shape(const Range2& r, int bx, int by) {
    int ni = r.i1 - r.i0 + 1, nk = r.k1 - r.k0 + 1;
    if (ni < 1) ni = 1;
    if (nk < 1) nk = 1;
    return dim3((unsigned)((ni + bx - 1) / bx), (unsigned)((nk + by - 1) / by), 1);
}

enum { RED_SUM = 0, RED_MIN = 1, RED_MAX = 2 };

__device__ __forceinline__ double red_apply(int op, double a, double b) {
    if (op == RED_SUM) return a + b;
    if (op == RED_MIN) return fmin(a, b);
    return fmax(a, b);
}
__device__ __forceinline__ double red_identity(int op) {
    if (op == RED_SUM) return 0.0;
    if (op == RED_MIN) return INFINITY;
    return -INFINITY;
}

// Block-level reduction of v (one value per thread, any 1-D/2-D block of at
// most 1024 threads) followed by a deterministic grid-level finish: each
// block stores its partial; the last block to arrive (counter) folds the
// partials in block order and writes *out, then re-arms the counter.
// Every thread of every block must call this exactly once.
__device__ __forceinline__ void reduce_to(int op, double v, double* part, unsigned int* count, double* out,
                                          double scale_div1 = 1.0, double scale_div2 = 1.0) {
    __shared__ double sh[32];
    __shared__ bool last;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nth = blockDim.x * blockDim.y;
    const int bid = blockIdx.x + blockIdx.y * gridDim.x;
    const int nb = gridDim.x * gridDim.y;
    for (int off = 16; off > 0; off >>= 1) v = red_apply(op, v, __shfl_down_sync(0xffffffffu, v, off));
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        double x = (tid < ((nth + 31) >> 5)) ? sh[tid] : red_identity(op);
        for (int off = 16; off > 0; off >>= 1) x = red_apply(op, x, __shfl_down_sync(0xffffffffu, x, off));
        if (tid == 0) {
            part[bid] = x;
            __threadfence();
            unsigned int t = atomicAdd(count, 1u);
            last = (t == (unsigned int)(nb - 1));
        }
    }
    __syncthreads();
    if (last) {
        __threadfence();
        if (tid < 32) {
            double x = red_identity(op);
            // lane-strided partial folds in fixed order, then a fixed tree;
            // eight loads in flight per lane (the fold order is unchanged)
            int b = tid;
            for (; b + 32 * 7 < nb; b += 32 * 8) {
                double t[8];
#pragma unroll
                for (int u = 0; u < 8; u++) t[u] = __ldcg(part + b + 32 * u);
#pragma unroll
                for (int u = 0; u < 8; u++) x = red_apply(op, x, t[u]);
            }
            for (; b < nb; b += 32) x = red_apply(op, x, __ldcg(part + b));
            for (int off = 16; off > 0; off >>= 1) x = red_apply(op, x, __shfl_down_sync(0xffffffffu, x, off));
            if (tid == 0) {
                if (op == RED_SUM) x = x / scale_div1 / scale_div2;
                *out = x;
                *count = 0u;
            }
        }
    }
}

// Host-side count of kernels this library enqueues (tc_kernel_launches).
void tc_note_launch(long long n = 1);

struct CPtrs {
    const double* p[TC_MAX_TYPES];
};
struct CPtrsW {
    double* p[TC_MAX_TYPES];
};

// ---------------------------------------------------------------------------
// Stencil helpers shared by the FP64 kernels (reference arithmetic) and their
// FP32 instances in the mixed-precision solve.
// ---------------------------------------------------------------------------

// full-weighting restriction at fine point (ii,kk); the corner term repeats
// (ii-1,kk+1) and omits (ii+1,kk-1), as iterative_solver.f90:607
// Loads of data that an earlier kernel of the stream wrote (streamfunction
// corrections, RHS, residuals) go to L2 only (ld.global.cg).  With
// programmatic dependent launch a kernel's CTAs can run on SMs whose L1 still
// holds lines of the same buffer from two launches back (ping-pong buffers),
// and a plain or non-coherent load could return such a stale line; the
// solve-constant coefficients keep __ldg.
template <typename T>
__device__ __forceinline__ T ld_state(const T* p) { return __ldcg(p); }

template <typename T>
__device__ __forceinline__ T restrict9(const T* in, const Lay& F, int ii, int kk) {
    T corners = (ld_state(in + IX(F, ii - 1, kk - 1)) + ld_state(in + IX(F, ii - 1, kk + 1)) +
                 ld_state(in + IX(F, ii + 1, kk + 1)) + ld_state(in + IX(F, ii - 1, kk + 1))) / T(16);
    T sides = (ld_state(in + IX(F, ii - 1, kk)) + ld_state(in + IX(F, ii, kk - 1)) + ld_state(in + IX(F, ii + 1, kk)) +
               ld_state(in + IX(F, ii, kk + 1))) / T(8);
    T centre = ld_state(in + IX(F, ii, kk)) / T(4);
    return corners + sides + centre;
}

// rhs - L S at x with the 13 folded coefficient planes (stream_space with
// the Database=2 order-2 stencil, iterative_solver.f90:456-561)
// All 26 loads are issued before the first multiply-add (independent loads
// in flight together instead of one L2 round trip per term); the sum keeps
// the tap order below, so the result does not depend on the load schedule.
template <typename T>
__device__ __forceinline__ T folded_residual(const Lay& L, const T* S, const T* __restrict__ coef, T rhs,
                                             size_t x) {
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const size_t pl = L.plane;
    const T* cf = coef + x;
    const T* s = S + x;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    T c[TC_NCOEF], v[TC_NCOEF];
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) {
        c[d] = __ldg(cf + d * pl);
        v[d] = ld_state(s + off[d]);
    }
    T acc = rhs;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) acc = fma(-c[d], v[d], acc);
    return acc;
}

// folded_residual in two phases, so that a kernel can load the coefficient
// planes (written once per multigrid call) before it waits for the previous
// kernel of the stream, and the stencil values and RHS after: same terms,
// same order, same result
template <typename T>
__device__ __forceinline__ void fold_coefs(const Lay& L, const T* __restrict__ coef, size_t x, T* c) {
    const size_t pl = L.plane;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) c[d] = __ldg(coef + x + d * pl);
}
template <typename T>
__device__ __forceinline__ T fold_apply(const Lay& L, const T* S, size_t x, const T* c, T rhs) {
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const T* s = S + x;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    T v[TC_NCOEF];
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) v[d] = ld_state(s + off[d]);
    T acc = rhs;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) acc = fma(-c[d], v[d], acc);
    return acc;
}

// the 13 folded FP32 coefficients, negated, from the five viscosity fields G
// (eta_xx - eta_zz, eta, eta_xz, eta_x, eta_z) and the weights of FoldG32:
// per tap the masked fields in order, first a product, then multiply-adds
__device__ __forceinline__ void fold_from_fields(const FoldG32& F, const float* G, float* cf) {
    constexpr unsigned kMask[TC_NCOEF] = TC_FOLD_G32_MASK;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) {
        float c = 0.f;
        bool first = true;
#pragma unroll
        for (int j = 0; j < 5; j++) {
            if (!((kMask[d] >> j) & 1u)) continue;
            c = first ? G[j] * F.w[d][j] : fmaf(G[j], F.w[d][j], c);
            first = false;
        }
        cf[d] = -c;
    }
}

// writes v at interior (i,k) and the ghost/mirror copies enforceBCs_stream
// derives from it (Vbc=0: antisymmetric rows; Vbc=1: symmetric rows)
template <typename T>
__device__ __forceinline__ void store_stream(const Lay& L, T* S, int i, int k, T v, int Vbc) {
    const int a = L.a, b = L.b;
    int gi[3] = {i, 0, 0};
    T si[3] = {T(1), T(-1), T(-1)};
    int ng = 1;
    if (i <= SP) gi[ng++] = -i;
    if (i >= a - SP) gi[ng++] = 2 * a - i;
    int gk[3] = {k, 0, 0};
    const T zsgn = (Vbc == 1) ? T(1) : T(-1);
    T sk[3] = {T(1), zsgn, zsgn};
    int nk = 1;
    if (k <= SP) gk[nk++] = -k;
    if (k >= b - SP) gk[nk++] = 2 * b - k;
    for (int u = 0; u < nk; u++)
        for (int t = 0; t < ng; t++) S[IX(L, gi[t], gk[u])] = (si[t] * sk[u]) * v;
}

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  Kernels of the multigrid cycle start with
// pdl_entry(), which waits until the previous kernel of the stream has
// completed and its writes are visible (griddepcontrol.wait), and end with
// pdl_done(), which lets the next kernel be scheduled while this one drains
// (griddepcontrol.launch_dependents; a thread that returns early counts as
// done).  launch_pdl() launches with the attribute that allows the early
// scheduling; without it both calls cost nothing.
// ---------------------------------------------------------------------------
//
// A kernel that uses them must not declare __restrict__ on a pointer whose
// memory an earlier kernel writes and which it reads or writes after
// pdl_entry(): the compiler may move accesses through such a pointer across
// the wait (it assumes nothing else touches that memory).  Solve-constant
// data (operator coefficients, dt, Chebyshev tables) may keep it.
__device__ __forceinline__ void pdl_entry() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_done() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<Args&&>(args)...);
}

// One smoother sweep (k_sweep / k_sweep32) for two vertically adjacent
// points per thread (rows k, k+1):
// the 18 stencil values of the pair are loaded once (13 per point alone),
// and the two multiply-add chains interleave.  Same taps in the same order
// per point as folded_residual, so the result equals the one-point kernels'.
template <typename T>
__global__ void __launch_bounds__(256, 1) k_sweep_x2(Lay L, Range2 r, const T* Sin, T* Sout, const T* __restrict__ coef,
                                                    const T* rhs, const T* __restrict__ dts,
                                                    const T* __restrict__ cA, const T* __restrict__ cB, T c_uniform,
                                                    int per_point, T temp, int Vbc) {
    const int i = r.i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = r.k0 + 2 * (int)(blockIdx.y * blockDim.y + threadIdx.y);
    bool act[2];
    act[0] = (i <= r.i1) && (k <= r.k1);
    act[1] = act[0] && (k + 1 <= r.k1);
    const size_t ld = (size_t)L.ld, pl = L.plane;
    const size_t x = act[0] ? IX(L, i, k) : 0;
    T cf[2][TC_NCOEF], dt[2], ca[2], cb[2];
#pragma unroll
    for (int p = 0; p < 2; p++) {
        const size_t xp = act[p] ? x + p * ld : x;
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[p][d] = act[p] ? -__ldg(coef + xp + d * pl) : T(0);
        dt[p] = act[p] ? __ldg(dts + xp) : T(0);
        ca[p] = (act[p] && per_point) ? __ldg(cA + xp) : T(1);
        cb[p] = (act[p] && per_point) ? __ldg(cB + xp) : T(0);
    }
    pdl_entry();
    if (!act[0]) return;
    // centre column rows k-2..k+3, columns i+-1 rows k-1..k+2, i+-2 rows k..k+1
    const T* s = Sin + x;
    T v0[6], vm1[4], vp1[4], vm2[2], vp2[2], rh[2];
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
        rh[q] = act[q] ? ld_state(rhs + x + q * ld) : T(0);
    }
    T acc[2];
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][0], v0[p + 2], rh[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][1], vm1[p + 1], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][2], vp1[p + 1], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][3], vm2[p], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][4], vp2[p], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][5], v0[p + 1], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][6], v0[p + 3], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][7], v0[p], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][8], v0[p + 4], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][9], vm1[p], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][10], vp1[p], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][11], vm1[p + 2], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) acc[p] = fma(cf[p][12], vp1[p + 2], acc[p]);
#pragma unroll
    for (int p = 0; p < 2; p++) {
        if (!act[p]) continue;
        const T c = per_point ? T(2) / (ca[p] + cb[p] * temp) : c_uniform;
        store_stream<T>(L, Sout, i, k + p, fma(c * dt[p], acc[p], v0[p + 2]), Vbc);
    }
    pdl_done();
}
