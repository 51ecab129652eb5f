// k_visit.cu -- one whole smoother visit of a small multigrid level
// (iterate_stream, iterative_solver.f90:860-963: Nmulti Richardson/Chebyshev
// sweeps with enforceBCs_stream after each, then compute_residual) in ONE
// launch of a thread-block cluster.
//
// Why: below 16K points a sweep is latency bound (about 6.5 us per launch
// whatever the size), and a W-cycle at 6 levels makes 24 visits x 70 sweeps
// to the two smallest smoothed levels.  Here each CTA of a cluster (up to
// 16) keeps a band of rows of the level in shared memory (two ping-pong
// buffers with two halo rows on each side), every thread owns one point and
// holds that point's 13 operator coefficients, RHS and pseudo-time step in
// registers for the whole visit, stores the values its neighbours need as
// halo directly into their shared memory (distributed shared memory, the
// addresses resolved once before the first sweep), and the cluster meets at
// one hardware barrier per sweep.  The per-point Chebyshev factor of the
// level with finite eigenvalue ratios comes from a table built once per
// multigrid call (k_cheb_table), so no FP64 division sits in the sweep.
// The arithmetic per point is the same as k_sweep / k_residual (same folded
// operator, same order, the same correctly rounded division for the table),
// so the level ends in the same state bit for bit.
#include "tc_device.cuh"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#define VISIT_MAX_SWEEPS 128
#define VISIT_THREADS 256
#define VISIT_MAX_CLUSTER 16
#define VISIT_SMEM_MAX (96 * 1024)

template <typename T>
struct VisitParams {
    Lay L;
    int nsweeps, per_point, Vbc, nrows_max;
    T c[VISIT_MAX_SWEEPS];
};

template <typename T>
struct ChebTemps {
    int nsweeps;
    T temp[VISIT_MAX_SWEEPS];
};

// rows k0..k1 of CTA `rank` out of C (interior rows 1..b-1 split evenly)
__device__ __forceinline__ void band_of(int rank, int C, int b, int& k0, int& k1) {
    const int nr = b - 1, base = nr / C, rem = nr % C;
    k0 = 1 + rank * base + min(rank, rem);
    k1 = k0 + base + (rank < rem ? 1 : 0) - 1;
}

// c(n, point) = 2 / (cA + cB*temp(n)) for the per-point Chebyshev level,
// the expression k_sweep evaluates, stored as tab[n*(a-1)(b-1) + (i-1) + (k-1)(a-1)].
template <typename T>
__global__ void k_cheb_table(Lay L, ChebTemps<T> Q, const T* __restrict__ cA, const T* __restrict__ cB,
                             T* __restrict__ tab) {
    const int a = L.a, b = L.b, npts = (a - 1) * (b - 1);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npts; p += gridDim.x * blockDim.x) {
        const int i = 1 + p % (a - 1), k = 1 + p / (a - 1);
        const size_t x = IX(L, i, k);
        const T A = __ldg(cA + x), B = __ldg(cB + x);
        for (int n = 0; n < Q.nsweeps; n++) tab[(size_t)n * npts + p] = T(2) / (A + B * Q.temp[n]);
    }
}

// One visit; T = double reproduces the reference arithmetic, T = float is the
// smoother of the mixed-precision solve.  NT threads per CTA, one point each.
template <typename T, int NT>
__global__ void __launch_bounds__(NT) k_visit_cluster(VisitParams<T> P, T* __restrict__ Sg, const T* __restrict__ coef,
                                                      const T* __restrict__ rhs, const T* __restrict__ dts,
                                                      const T* __restrict__ ctab, T* __restrict__ res) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), me = (int)cl.block_rank();
    const Lay& L = P.L;
    const int a = L.a, b = L.b, W = a + 1 + 2 * SP;  // shared row: columns -SP..a+SP
    int k0, k1;
    band_of(me, C, b, k0, k1);
    const int cnt = k1 - k0 + 1, R = P.nrows_max + 4;  // rows k0-2..k1+2 (buffer sized for the largest band)
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T* buf0 = reinterpret_cast<T*>(sm_raw);
    T* buf1 = buf0 + (size_t)R * W;
    const int tid = threadIdx.x, nth = blockDim.x;
    const T zsgn = (P.Vbc == 1) ? T(1) : T(-1);
    // load rows k0-2..k1+2 (ghosts and walls included) into both buffers
    for (int t = tid; t < (cnt + 4) * W; t += nth) {
        const int r = t / W, c = t % W;
        const int k = k0 - 2 + r, i = c - SP;
        T v = T(0);
        if (k >= -SP && k <= b + SP) v = Sg[IX(L, i, k)];
        buf0[(size_t)r * W + c] = v;
        buf1[(size_t)r * W + c] = v;
    }
    // this thread's point (the launcher guarantees one point per thread at most)
    const bool act = tid < cnt * (a - 1);
    const int i = act ? 1 + tid % (a - 1) : 1, k = act ? k0 + tid / (a - 1) : k0;
    const int r = k - k0 + 2;
    const int xs = r * W + i + SP;
    const size_t xg = IX(L, i, k);
    const int npl = (a - 1) * (b - 1), gp = (i - 1) + (k - 1) * (a - 1);
    T cf[TC_NCOEF];
    T rh = T(0), dt = T(0);
    if (act) {
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[d] = -__ldg(coef + xg + (size_t)d * L.plane);
        rh = __ldg(rhs + xg);
        dt = __ldg(dts + xg);
    } else {
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[d] = T(0);
    }
    // local mirror targets: side ghost column (enforceBCs_stream antisymmetric
    // walls) and the ghost row -1 / b+1 held as halo by the first / last CTA
    const int side = (i <= SP) ? r * W + (-i + SP) : (i >= a - SP) ? r * W + (2 * a - i + SP) : -1;
    const int grow = (k == 1) ? (r - 2) * W + i + SP : (k == b - 1) ? (r + 2) * W + i + SP : -1;
    // halo rows of the neighbouring CTAs (at most two on each side)
    // (slot j serves the CTA at offset d = -2, -1, +1, +2; null = not a halo row there)
    T* rem0[4];
    T* rem1[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int d = (j < 2) ? j - 2 : j - 1, o = me + d;
        rem0[j] = nullptr;
        rem1[j] = nullptr;
        if (o < 0 || o >= C || !act) continue;
        int ok0, ok1;
        band_of(o, C, b, ok0, ok1);
        if ((k >= ok0 - 2 && k <= ok0 - 1) || (k >= ok1 + 1 && k <= ok1 + 2)) {
            const int off = (k - ok0 + 2) * W + i + SP;
            rem0[j] = cl.map_shared_rank(buf0, o) + off;
            rem1[j] = cl.map_shared_rank(buf1, o) + off;
        }
    }
    cl.sync();
    for (int n = 0; n < P.nsweeps; n++) {
        const T* cur = (n & 1) ? buf1 : buf0;
        T* nxt = (n & 1) ? buf0 : buf1;
        if (act) {
            const T c = P.per_point ? __ldg(ctab + (size_t)n * npl + gp) : P.c[n];
            // identical term order to folded_residual
            T acc = rh;
            acc = fma(cf[0], cur[xs], acc);
            acc = fma(cf[1], cur[xs - 1], acc);
            acc = fma(cf[2], cur[xs + 1], acc);
            acc = fma(cf[3], cur[xs - 2], acc);
            acc = fma(cf[4], cur[xs + 2], acc);
            acc = fma(cf[5], cur[xs - W], acc);
            acc = fma(cf[6], cur[xs + W], acc);
            acc = fma(cf[7], cur[xs - 2 * W], acc);
            acc = fma(cf[8], cur[xs + 2 * W], acc);
            acc = fma(cf[9], cur[xs - 1 - W], acc);
            acc = fma(cf[10], cur[xs + 1 - W], acc);
            acc = fma(cf[11], cur[xs - 1 + W], acc);
            acc = fma(cf[12], cur[xs + 1 + W], acc);
            const T v = fma(c * dt, acc, cur[xs]);
            nxt[xs] = v;
            if (side >= 0) nxt[side] = -v;
            if (grow >= 0) nxt[grow] = zsgn * v;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                T* q = (n & 1) ? rem0[j] : rem1[j];
                if (q) *q = v;
            }
        }
        if (C == 1) __syncthreads();
        else cl.sync();
    }
    // final state: owned rows (with side ghosts) to global, then ghost rows
    const T* fin = (P.nsweeps & 1) ? buf1 : buf0;
    for (int t = tid; t < cnt * W; t += nth) {
        const int rr = 2 + t / W, c = t % W;
        Sg[IX(L, c - SP, k0 - 2 + rr)] = fin[(size_t)rr * W + c];
    }
    // residual on owned points (halos are current after the last barrier)
    if (act && res != nullptr) {
        T acc = rh;
        acc = fma(cf[0], fin[xs], acc);
        acc = fma(cf[1], fin[xs - 1], acc);
        acc = fma(cf[2], fin[xs + 1], acc);
        acc = fma(cf[3], fin[xs - 2], acc);
        acc = fma(cf[4], fin[xs + 2], acc);
        acc = fma(cf[5], fin[xs - W], acc);
        acc = fma(cf[6], fin[xs + W], acc);
        acc = fma(cf[7], fin[xs - 2 * W], acc);
        acc = fma(cf[8], fin[xs + 2 * W], acc);
        acc = fma(cf[9], fin[xs - 1 - W], acc);
        acc = fma(cf[10], fin[xs + 1 - W], acc);
        acc = fma(cf[11], fin[xs - 1 + W], acc);
        acc = fma(cf[12], fin[xs + 1 + W], acc);
        res[xg] = acc;
    }
    __threadfence();
    cl.sync();  // global rows written; no CTA leaves while others may touch its shared memory
    // top/bottom ghost rows from the (now global) interior rows
    if (me == 0 || me == C - 1) {
        for (int t = tid; t < 2 * W; t += nth) {
            const int g = 1 + t / W, c = t % W, ii = c - SP;
            if (me == 0) {
                const T v = Sg[IX(L, ii, g)];
                Sg[IX(L, ii, -g)] = zsgn * v;
            }
            if (me == C - 1) {
                const T v = Sg[IX(L, ii, b - g)];
                Sg[IX(L, ii, b + g)] = zsgn * v;
            }
        }
    }
}

template <typename T, int NT>
static bool visit_attrs() {
    if (cudaFuncSetAttribute(k_visit_cluster<T, NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return false;
    return cudaFuncSetAttribute(k_visit_cluster<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                VISIT_SMEM_MAX) == cudaSuccess;
}

// Kernel attributes for clusters of up to 16 CTAs and 96 KB of shared memory;
// returns how many 16-CTA clusters with that much shared memory can be
// resident (0 = the fused visit is unavailable, callers use per-sweep launches).
int visit_cluster_setup() {
    if (!visit_attrs<double, 256>() || !visit_attrs<float, 256>() || !visit_attrs<float, 1024>()) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(VISIT_MAX_CLUSTER, 1, 1);
    cfg.blockDim = dim3(1024, 1, 1);
    cfg.dynamicSmemBytes = VISIT_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = VISIT_MAX_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_visit_cluster<float, 1024>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Cluster size, threads per CTA and shared memory for a level, or 0 if the
// level is not fused (more points than threads, too many sweeps or too
// little shared memory).  FP64 uses 256 threads per CTA (13 coefficients in
// registers need more than the 64 a 1024-thread CTA allows); FP32 takes 256
// when that covers the level and 1024 otherwise.
static int visit_shape(const Lay& L, int nsweeps, size_t esize, int* nt, int* rows_max, size_t* smem) {
    const int a = L.a, b = L.b;
    if (nsweeps > VISIT_MAX_SWEEPS || b - 1 < 2 || a - 1 < 1) return 0;
    // as many CTAs as rows up to 16: fewer, fuller CTAs measured slower (the
    // sweep is bound by shared-memory loads per CTA, not by the barrier)
    const int C = (b - 1 < VISIT_MAX_CLUSTER) ? (b - 1) : VISIT_MAX_CLUSTER;
    const int nr = b - 1, rm = nr / C + (nr % C ? 1 : 0);
    int threads = 256;
    if (rm * (a - 1) > threads) {
        if (esize == sizeof(double)) return 0;
        threads = 1024;
        if (rm * (a - 1) > threads) return 0;
    }
    const size_t sm = esize * 2 * (size_t)(rm + 4) * (size_t)(a + 1 + 2 * SP);
    if (sm > VISIT_SMEM_MAX) return 0;
    *nt = threads;
    *rows_max = rm;
    *smem = sm;
    return C;
}

int visit_cluster_fits(const Lay& L, int nsweeps, int fp32) {
    int nt, rm;
    size_t sm;
    return visit_shape(L, nsweeps, fp32 ? sizeof(float) : sizeof(double), &nt, &rm, &sm) > 0;
}

template <typename T>
static void cheb_table_t(cudaStream_t s, const Lay& L, const double* tvals, int nsweeps, const T* cA, const T* cB,
                         T* tab) {
    ChebTemps<T> Q;
    Q.nsweeps = nsweeps;
    for (int n = 0; n < nsweeps; n++) Q.temp[n] = (T)tvals[n];
    const int npts = (L.a - 1) * (L.b - 1);
    k_cheb_table<T><<<(npts + 255) / 256, 256, 0, s>>>(L, Q, cA, cB, tab); tc_note_launch();
}
void launch_cheb_table(cudaStream_t s, const Level& lv, const double* tvals, int nsweeps, double* tab) {
    cheb_table_t<double>(s, lv.L, tvals, nsweeps, lv.cA, lv.cB, tab);
}
void launch_cheb_table32(cudaStream_t s, const Level& lv, const double* tvals, int nsweeps, float* tab) {
    cheb_table_t<float>(s, lv.L, tvals, nsweeps, lv.cA32, lv.cB32, tab);
}

template <typename T>
static int visit_t(cudaStream_t s, const Lay& L, T* S, const T* coef, const T* rhs, const T* dts, const T* ctab,
                   T* res, const double* cvals, int nsweeps, int per_point, int Vbc) {
    int nt, rows_max;
    size_t smem;
    const int C = visit_shape(L, nsweeps, sizeof(T), &nt, &rows_max, &smem);
    if (C == 0) return 1;
    if (per_point && ctab == nullptr) return 1;
    VisitParams<T> P;
    P.L = L;
    P.nsweeps = nsweeps;
    P.per_point = per_point;
    P.Vbc = Vbc;
    P.nrows_max = rows_max;
    for (int n = 0; n < nsweeps; n++) P.c[n] = (T)cvals[n];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C, 1, 1);
    cfg.blockDim = dim3((unsigned)nt, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (nt == 256) e = cudaLaunchKernelEx(&cfg, k_visit_cluster<T, 256>, P, S, coef, rhs, dts, ctab, res);
    else e = cudaLaunchKernelEx(&cfg, k_visit_cluster<T, 1024>, P, S, coef, rhs, dts, ctab, res);
    if (e != cudaSuccess) return 2;
    tc_note_launch();
    return 0;
}

// Returns 0 if the level was handled here (caller skips the per-sweep path).
int launch_visit_cluster(cudaStream_t s, const Level& lv, double* S, const double* cvals, const double* ctab,
                         int nsweeps, int per_point, int Vbc) {
    return visit_t<double>(s, lv.L, S, lv.coef, lv.rhs, lv.dt_stream, ctab, lv.res, cvals, nsweeps, per_point, Vbc);
}
int launch_visit_cluster32(cudaStream_t s, const Level& lv, float* S, const double* cvals, const float* ctab,
                           int nsweeps, int per_point, int Vbc) {
    return visit_t<float>(s, lv.L, S, lv.coef32, lv.rhs32, lv.dts32, ctab, lv.res32, cvals, nsweeps, per_point, Vbc);
}
