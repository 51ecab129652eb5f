// k_visit.cu -- one whole smoother visit of a small multigrid level
// (iterate_stream, iterative_solver.f90:860-963: Nmulti Richardson/Chebyshev
// sweeps with enforceBCs_stream after each, then compute_residual) in ONE
// launch of a thread-block cluster.
//
// Why: below 16K points a sweep is latency bound (about 6.5 us per launch
// whatever the size), and a W-cycle at 6 levels makes 24 visits x 70 sweeps
// to the two smallest smoothed levels.  Here each CTA of a cluster (up to
// 16) keeps a band of rows of the level in shared memory (two ping-pong
// buffers with two halo rows on each side), computes its rows, stores the
// rows its neighbours need as halo directly into their shared memory
// (distributed shared memory), and the cluster meets at one hardware
// barrier per sweep.  The arithmetic per point is the same as k_sweep /
// k_residual (same folded operator, same order), so the level ends in the
// same state bit for bit.
#include "tc_device.cuh"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#define VISIT_MAX_SWEEPS 128

struct VisitParams {
    Lay L;
    int nsweeps, per_point, Vbc, nrows_max;
    double c[VISIT_MAX_SWEEPS];
    double temp[VISIT_MAX_SWEEPS];
};

// rows k0..k1 of CTA `rank` out of C (interior rows 1..b-1 split evenly)
__device__ __forceinline__ void band_of(int rank, int C, int b, int& k0, int& k1) {
    const int nr = b - 1, base = nr / C, rem = nr % C;
    k0 = 1 + rank * base + min(rank, rem);
    k1 = k0 + base + (rank < rem ? 1 : 0) - 1;
}

__device__ __forceinline__ double stencil_res(const double* __restrict__ S, int W, size_t x,
                                              const double* __restrict__ cf, size_t pl, double rhs) {
    // identical term order to folded_residual (k_mg.cu); S has row stride W
    double acc = rhs;
    acc = fma(-__ldg(cf + 0 * pl), S[x], acc);
    acc = fma(-__ldg(cf + 1 * pl), S[x - 1], acc);
    acc = fma(-__ldg(cf + 2 * pl), S[x + 1], acc);
    acc = fma(-__ldg(cf + 3 * pl), S[x - 2], acc);
    acc = fma(-__ldg(cf + 4 * pl), S[x + 2], acc);
    acc = fma(-__ldg(cf + 5 * pl), S[x - W], acc);
    acc = fma(-__ldg(cf + 6 * pl), S[x + W], acc);
    acc = fma(-__ldg(cf + 7 * pl), S[x - 2 * W], acc);
    acc = fma(-__ldg(cf + 8 * pl), S[x + 2 * W], acc);
    acc = fma(-__ldg(cf + 9 * pl), S[x - 1 - W], acc);
    acc = fma(-__ldg(cf + 10 * pl), S[x + 1 - W], acc);
    acc = fma(-__ldg(cf + 11 * pl), S[x - 1 + W], acc);
    acc = fma(-__ldg(cf + 12 * pl), S[x + 1 + W], acc);
    return acc;
}

__global__ void __launch_bounds__(256) k_visit_cluster(VisitParams P, double* __restrict__ Sg,
                                                       const double* __restrict__ coef,
                                                       const double* __restrict__ rhs,
                                                       const double* __restrict__ dts,
                                                       const double* __restrict__ cA,
                                                       const double* __restrict__ cB, double* __restrict__ res) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), me = (int)cl.block_rank();
    const Lay& L = P.L;
    const int a = L.a, b = L.b, W = a + 1 + 2 * SP;  // shared row: columns -SP..a+SP
    int k0, k1;
    band_of(me, C, b, k0, k1);
    const int cnt = k1 - k0 + 1, R = P.nrows_max + 4;  // rows k0-2..k1+2 (buffer sized for the largest band)
    extern __shared__ double sm[];
    double* buf0 = sm;
    double* buf1 = sm + (size_t)R * W;
    const int tid = threadIdx.x, nth = blockDim.x;
    const double zsgn = (P.Vbc == 1) ? 1.0 : -1.0;
    // load rows k0-2..k1+2 (ghosts and walls included) into both buffers
    for (int t = tid; t < (cnt + 4) * W; t += nth) {
        const int r = t / W, c = t % W;
        const int k = k0 - 2 + r, i = c - SP;
        double v = 0.0;
        if (k >= -SP && k <= b + SP) v = Sg[IX(L, i, k)];
        buf0[(size_t)r * W + c] = v;
        buf1[(size_t)r * W + c] = v;
    }
    cl.sync();
    const int npts = cnt * (a - 1);
    for (int n = 0; n < P.nsweeps; n++) {
        const double* cur = (n & 1) ? buf1 : buf0;
        double* nxt = (n & 1) ? buf0 : buf1;
        const double cu = P.c[n], tn = P.temp[n];
        for (int pidx = tid; pidx < npts; pidx += nth) {
            const int k = k0 + pidx / (a - 1), i = 1 + pidx % (a - 1);
            const int r = k - k0 + 2;
            const size_t xs = (size_t)r * W + (size_t)(i + SP);
            const size_t xg = IX(L, i, k);
            const double rs = stencil_res(cur, W, xs, coef + xg, L.plane, __ldg(rhs + xg));
            const double c = P.per_point ? 2.0 / (__ldg(cA + xg) + __ldg(cB + xg) * tn) : cu;
            const double v = fma(c * __ldg(dts + xg), rs, cur[xs]);
            nxt[xs] = v;
            // side ghosts of this row (enforceBCs_stream: antisymmetric walls)
            if (i <= SP) nxt[(size_t)r * W + (size_t)(-i + SP)] = -v;
            if (i >= a - SP) nxt[(size_t)r * W + (size_t)(2 * a - i + SP)] = -v;
            // ghost rows -1 / b+1 are halo rows of the first / last CTA
            if (k == 1) nxt[(size_t)(r - 2) * W + (size_t)(i + SP)] = zsgn * v;  // row -1 (this CTA owns row 1)
            if (k == b - 1) nxt[(size_t)(r + 2) * W + (size_t)(i + SP)] = zsgn * v;  // row b+1
            // halo rows of the neighbouring CTAs
            for (int d = -2; d <= 2; d++) {
                const int o = me + d;
                if (d == 0 || o < 0 || o >= C) continue;
                int ok0, ok1;
                band_of(o, C, b, ok0, ok1);
                if ((k >= ok0 - 2 && k <= ok0 - 1) || (k >= ok1 + 1 && k <= ok1 + 2)) {
                    double* rb = cl.map_shared_rank(nxt, o);
                    rb[(size_t)(k - ok0 + 2) * W + (size_t)(i + SP)] = v;
                }
            }
        }
        cl.sync();
    }
    // final state: owned rows (with side ghosts) to global, then ghost rows
    const double* fin = (P.nsweeps & 1) ? buf1 : buf0;
    for (int t = tid; t < cnt * W; t += nth) {
        const int r = 2 + t / W, c = t % W;
        Sg[IX(L, c - SP, k0 - 2 + r)] = fin[(size_t)r * W + c];
    }
    // residual on owned points (halos are current after the last barrier)
    for (int pidx = tid; pidx < npts; pidx += nth) {
        const int k = k0 + pidx / (a - 1), i = 1 + pidx % (a - 1);
        const size_t xs = (size_t)(k - k0 + 2) * W + (size_t)(i + SP);
        const size_t xg = IX(L, i, k);
        res[xg] = stencil_res(fin, W, xs, coef + xg, L.plane, __ldg(rhs + xg));
    }
    __threadfence();
    cl.sync();  // global rows written; no CTA leaves while others may touch its shared memory
    // top/bottom ghost rows from the (now global) interior rows
    if (me == 0 || me == C - 1) {
        for (int t = tid; t < 2 * W; t += nth) {
            const int g = 1 + t / W, c = t % W, i = c - SP;
            if (me == 0) {
                const double v = Sg[IX(L, i, g)];
                Sg[IX(L, i, -g)] = zsgn * v;
            }
            if (me == C - 1) {
                const double v = Sg[IX(L, i, b - g)];
                Sg[IX(L, i, b + g)] = zsgn * v;
            }
        }
    }
}

// Kernel attributes for clusters of up to 16 CTAs and 96 KB of shared memory;
// returns how many 16-CTA clusters with that much shared memory can be
// resident (0 = the fused visit is unavailable, callers use per-sweep launches).
int visit_cluster_setup() {
    if (cudaFuncSetAttribute(k_visit_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(k_visit_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024) != cudaSuccess)
        return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16, 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = 96 * 1024;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_visit_cluster, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// Returns 0 if the level was handled here (caller skips the per-sweep path).
int launch_visit_cluster(cudaStream_t s, const Level& lv, double* S, const double* cvals, const double* tvals,
                         int nsweeps, int per_point, int Vbc) {
    const int a = lv.L.a, b = lv.L.b;
    if (nsweeps > VISIT_MAX_SWEEPS || (a - 1) * (b - 1) > 4096 || b - 1 < 2) return 1;
    const int C = (b - 1 < 16) ? (b - 1) : 16;
    const int nr = b - 1, rows_max = nr / C + (nr % C ? 1 : 0);
    if (rows_max < 1) return 1;
    const int W = a + 1 + 2 * SP;
    const size_t smem = sizeof(double) * 2 * (size_t)(rows_max + 4) * W;
    if (smem > 96 * 1024) return 1;
    VisitParams P;
    P.L = lv.L;
    P.nsweeps = nsweeps;
    P.per_point = per_point;
    P.Vbc = Vbc;
    P.nrows_max = rows_max;
    for (int n = 0; n < nsweeps; n++) { P.c[n] = cvals[n]; P.temp[n] = tvals[n]; }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C, 1, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_visit_cluster, P, S, (const double*)lv.coef, (const double*)lv.rhs,
                                       (const double*)lv.dt_stream, (const double*)lv.cA, (const double*)lv.cB,
                                       lv.res);
    if (e != cudaSuccess) return 2;
    tc_note_launch();
    return 0;
}
