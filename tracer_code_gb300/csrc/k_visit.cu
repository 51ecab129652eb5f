// k_visit.cu -- one whole smoother visit of a small multigrid level
// (iterate_stream, iterative_solver.f90:860-963: Nmulti Richardson/Chebyshev
// sweeps with enforceBCs_stream after each, then compute_residual) in ONE
// launch of a thread-block cluster.
//
// Why: below ~16K points a sweep is latency bound (several microseconds per
// launch whatever the size), and a W-cycle at 6 levels makes 30 visits of
// 70 sweeps to levels 3..5 alone.
//
// Layout.  The level's interior rows 1..b-1 are cut into bands of `rpc` rows,
// one band per CTA of a cluster (up to 16 CTAs).  Each CTA keeps its band
// plus two halo rows on each side in shared memory (ping-pong buffers; three
// when the cluster has more than one CTA, see below).  Each thread owns a
// vertical strip of P points of one column (rows r..r+P-1): it keeps their
// 13 folded operator coefficients, RHS and pseudo-time step in registers
// for the whole visit and loads the 5P+8 stencil values the strip needs
// once per sweep (instead of 13P), so a sweep costs few shared-memory loads.
//
// Exchange.  After computing a sweep, a thread stores the values of its
// points that are halo rows of a neighbouring CTA straight into that CTA's
// next buffer with st.async, which signals the receiver's mbarrier with the
// byte count; a CTA waits only for the bytes its own halo needs (no
// cluster-wide barrier per sweep).  A neighbour can run at most one sweep
// ahead (it needs this CTA's halo to start the next), so with three
// buffers it never writes a buffer this CTA is still reading.  Every wait
// is bounded: past the limit the kernel sets DevScalars.visit_timeout,
// leaves the sweep loop on all threads and returns normally.
//
// Arithmetic per point is that of k_sweep / k_residual (same folded
// operator taps in the same order, the Chebyshev factor from a table of the
// same correctly rounded division; FP32 divides in the sweep exactly as
// k_sweep32 does), so the level ends in the same state bit for bit as with
// one launch per sweep; the FP32 instance is the smoother of the mixed solve.
#include "tc_device.cuh"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#define VISIT_MAX_SWEEPS 128
#define VISIT_MAX_CLUSTER 16
#define VISIT_SMEM_MAX (96 * 1024)
#define VISIT_WAIT_LIMIT (1 << 20)
// polls of the timeout-path test's word (VisitParams.test_flag)
#define VISIT_TEST_WAIT_LIMIT (1 << 14)

template <typename T>
struct VisitParams {
    Lay L;
    int nsweeps, per_point, Vbc, rpc;
    T c[VISIT_MAX_SWEEPS];     // uniform Chebyshev/Richardson factor of sweep n
    T temp[VISIT_MAX_SWEEPS];  // Chebyshev node of sweep n (per-point factor, FP32)
    // optional transfers fused into the visit (nullptr: none)
    const T* ec;  // prolong: the coarser level's correction, added to the level's state first
    Lay Lc;
    T* rc;        // restrict: the final residual's full weighting into the coarser RHS
    Lay Lr;
    T* zc;        // with the restriction: the coarser correction set to zero (zn values)
    size_t zn;
    // timeout-path test (null in solves): before its first sweep the visit
    // waits, bounded, for this device word to become non-zero; nothing sets
    // it, so the wait runs out and the visit takes its timeout exit having
    // issued no remote write
    const int* test_flag;
};

// bilinear prolongation of the coarse correction at fine point (i,k): the
// value prolong (iterative_solver.f90:175-233) adds, in k_prolong's order
template <typename T>
__device__ __forceinline__ T prolong_at(const Lay& C, const T* ec, int i, int k) {
    const bool ie = (i % 2) == 0, ke = (k % 2) == 0;
    if (ie && ke) return ld_state(ec + IX(C, i / 2, k / 2));
    if (ie) return (ld_state(ec + IX(C, i / 2, (k - 1) / 2)) + ld_state(ec + IX(C, i / 2, (k + 1) / 2))) / T(2);
    if (ke) return (ld_state(ec + IX(C, (i - 1) / 2, k / 2)) + ld_state(ec + IX(C, (i + 1) / 2, k / 2))) / T(2);
    return (ld_state(ec + IX(C, (i - 1) / 2, (k - 1) / 2)) + ld_state(ec + IX(C, (i + 1) / 2, (k - 1) / 2)) +
            ld_state(ec + IX(C, (i + 1) / 2, (k + 1) / 2)) + ld_state(ec + IX(C, (i - 1) / 2, (k + 1) / 2))) /
           T(4);
}

// the level's state at (ii,kk) after the fused prolongation: interior points
// get psi + prolong, ghosts the mirrored interior value times the boundary
// signs (store_stream's rule), walls stay
template <typename T>
__device__ __forceinline__ T state_after_prolong(const Lay& L, const Lay& C, const T* S, const T* ec, int ii, int kk,
                                                 T zsgn) {
    const int a = L.a, b = L.b;
    int mi = ii, mk = kk;
    T si = T(1), sk = T(1);
    if (ii < 0) { mi = -ii; si = T(-1); }
    else if (ii > a) { mi = 2 * a - ii; si = T(-1); }
    if (kk < 0) { mk = -kk; sk = zsgn; }
    else if (kk > b) { mk = 2 * b - kk; sk = zsgn; }
    if (mi < 1 || mi > a - 1 || mk < 1 || mk > b - 1) return ld_state(S + IX(L, ii, kk));
    const T v = ld_state(S + IX(L, mi, mk)) + prolong_at(C, ec, mi, mk);
    return (si * sk) * v;
}

template <typename T>
struct ChebTemps {
    int nsweeps;
    T temp[VISIT_MAX_SWEEPS];
};

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

// ---- cluster shared-memory primitives ---------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t cluster_addr(uint32_t a, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_async(uint32_t raddr, float v, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(raddr),
                 "r"(__float_as_uint(v)), "r"(rbar)
                 : "memory");
}
__device__ __forceinline__ void st_async(uint32_t raddr, double v, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(raddr),
                 "l"(__double_as_longlong(v)), "r"(rbar)
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t a, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint32_t a, int bytes) {
    asm volatile("{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }" ::"r"(a), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t a, int parity) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// One visit.  NT threads per CTA; thread t owns column i = 1 + t % (a-1),
// strip j = t / (a-1) of its CTA's band (rows k0 + jP .. k0 + jP + P-1).
// W is the shared-memory row stride (>= a+5, a compile-time class so the
// stencil offsets fold into the load instructions).
template <typename T, int P, int NT, int W>
__global__ void __launch_bounds__(NT, 1) k_visit_cluster(VisitParams<T> Q, T* Sg,
                                                         const T* __restrict__ coef, const T* rhs,
                                                         const T* __restrict__ dts, const T* __restrict__ ctab,
                                                         const T* __restrict__ cA, const T* __restrict__ cB,
                                                         T* res, int* timeout_flag) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), me = (int)cl.block_rank();
    const Lay& L = Q.L;
    const int a = L.a, b = L.b;  // shared row: columns -SP..a+SP (W >= a + 1 + 2SP)
    const int rpc = Q.rpc;
    const int k0 = 1 + me * rpc, k1 = min(b - 1, k0 + rpc - 1);
    // rows k0-2 .. k0+rpcp+1 with the band rounded up to whole strips, so the
    // loads of a strip that runs past the band's last row stay inside the buffer
    const int R = ((rpc + P - 1) / P) * P + 4;
    const int nbuf = (C > 1) ? 3 : 2;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm_raw);  // 4 mbarriers (first 32 B)
    T* buf = reinterpret_cast<T*>(sm_raw + 32);
    const size_t bsz = (size_t)R * W;
    const int tid = threadIdx.x;
    const T zsgn = (Q.Vbc == 1) ? T(1) : T(-1);
    // this thread's strip
    const int cols = a - 1;
    const int i = 1 + tid % cols, strip = tid / cols;
    const int kr = k0 + strip * P;  // first row of the strip
    const int r0 = kr - k0 + 2;     // its buffer row
    const int cc = i + SP;          // buffer column
    const int npl = cols * (b - 1);
    bool act[P];
    T cf[P][TC_NCOEF], rh[P], dt[P];
    // FP32 evaluates the per-point Chebyshev factor 2/(cA + cB*temp) in the
    // sweep (as k_sweep32 does); FP64 reads it from the table (a division in
    // the sweep would dominate its FP64 pipe), prefetched two sweeps ahead
    constexpr bool kDivide = (sizeof(T) == sizeof(float));
    T ca[P], cbv[P];
    // per-thread flags: the column has a mirrored side ghost; the strip holds
    // row 1 or b-1 (ghost row -1 / b+1); the strip holds halo rows of another
    // CTA (bit 4+j of point p: CTA me-2, me-1, me+1, me+2 for j = 0..3)
    const bool has_side = (i <= SP || i >= a - SP);
    const int side = (i <= SP) ? SP - i : 2 * a - i + SP;
    bool has_grow = false;
    int remote = 0;  // bit (4p + j)
#pragma unroll
    for (int p = 0; p < P; p++) {
        const int k = kr + p;
        act[p] = (strip * P + p < rpc) && (tid < (NT / cols) * cols) && (k <= k1);
        const size_t xg = IX(L, i, act[p] ? k : k0);
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[p][d] = act[p] ? -__ldg(coef + xg + (size_t)d * L.plane) : T(0);
        rh[p] = T(0);
        dt[p] = act[p] ? __ldg(dts + xg) : T(0);
        ca[p] = (kDivide && Q.per_point && act[p]) ? __ldg(cA + xg) : T(1);
        cbv[p] = (kDivide && Q.per_point && act[p]) ? __ldg(cB + xg) : T(0);
        if (!act[p]) continue;
        if (k == 1 || k == b - 1) has_grow = true;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int o = me + ((j < 2) ? j - 2 : j - 1);
            if (o < 0 || o >= C) continue;
            const int ok0 = 1 + o * rpc, ok1 = min(b - 1, ok0 + rpc - 1);
            if ((k >= ok0 - 2 && k <= ok0 - 1) || (k >= ok1 + 1 && k <= ok1 + 2)) remote |= 1 << (4 * p + j);
        }
    }
    // everything above is fixed within a solve; the RHS and the level's state
    // come from earlier kernels of the stream
    pdl_entry();
#pragma unroll
    for (int p = 0; p < P; p++)
        if (act[p]) rh[p] = ld_state(rhs + IX(L, i, kr + p));
    // rows k0-2..k1+2 (ghosts, walls and halos) into every buffer; four
    // independent global loads in flight per thread
    {
        const int wa = a + 1 + 2 * SP, n_el = (k1 - k0 + 5) * wa;
        for (int t0 = tid; t0 < n_el; t0 += 4 * NT) {
            T v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int t = t0 + u * NT;
                const int r = t / wa, c = t % wa, k = k0 - 2 + r;
                v[u] = (t < n_el && k >= -SP && k <= b + SP)
                           ? (Q.ec ? state_after_prolong(L, Q.Lc, Sg, Q.ec, c - SP, k, zsgn)
                                   : ld_state(Sg + IX(L, c - SP, k)))
                           : T(0);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int t = t0 + u * NT;
                if (t >= n_el) break;
                const int r = t / wa, c = t % wa;
                for (int q = 0; q < nbuf; q++) buf[q * bsz + (size_t)r * W + c] = v[u];
            }
        }
    }
    if (tid == 0 && C > 1) {
        // 0-2: the sweep buffers; 3: the residual rows of the fused restriction
        // sweep buffers: one arrival per warp (its values stored) plus the
        // halo bytes; the residual rows: one arrival plus their bytes
        for (int q = 0; q < 4; q++) mbar_init(smem_addr(&bar[q]), q < 3 ? NT / 32 : 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // bytes this CTA receives per sweep: its halo rows that other CTAs own
    int expect = 0;
    for (int k = k0 - 2; k <= k1 + 2; k++)
        if ((k < k0 || k > k1) && k >= 1 && k <= b - 1) expect += cols * (int)sizeof(T);
    cl.sync();  // buffers loaded and mbarriers initialised cluster-wide
    int phase = 0;  // bit q: parity of mbarrier q's current phase
    int cur_b = 0;
    bool timed_out = false;
    if (Q.test_flag != nullptr) {
        int gave_up = 0;
        if (tid == 0) {
            int it = 0;
            while (*(volatile const int*)Q.test_flag == 0 && ++it <= VISIT_TEST_WAIT_LIMIT) {
            }
            gave_up = 1;
        }
        timed_out = __syncthreads_or(gave_up) != 0;
    }
    const size_t tab_base = (size_t)(i - 1) + (size_t)(kr - 1) * cols;
    // table prefetch ring (FP64 per-point level): factors of sweeps n, n+1
    T pre0[P], pre1[P];
#pragma unroll
    for (int p = 0; p < P; p++) {
        const bool ld = !kDivide && Q.per_point && act[p];
        pre0[p] = (ld && Q.nsweeps > 0) ? __ldg(ctab + tab_base + (size_t)p * cols) : T(0);
        pre1[p] = (ld && Q.nsweeps > 1) ? __ldg(ctab + (size_t)npl + tab_base + (size_t)p * cols) : T(0);
    }
    for (int n = 0; n < Q.nsweeps && !timed_out; n++) {
        const int nxt_b = (cur_b + 1 == nbuf) ? 0 : cur_b + 1;
        const T* cur = buf + (size_t)cur_b * bsz;
        T* nxt = buf + (size_t)nxt_b * bsz;
        if (act[0]) {
            T cp[P];
            if (Q.per_point && kDivide) {
                const T tn = Q.temp[n];
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = T(2) / (ca[p] + cbv[p] * tn);
            } else if (Q.per_point) {
#pragma unroll
                for (int p = 0; p < P; p++) {
                    cp[p] = pre0[p];
                    pre0[p] = pre1[p];
                    pre1[p] = (act[p] && n + 2 < Q.nsweeps)
                                  ? __ldg(ctab + (size_t)(n + 2) * npl + tab_base + (size_t)p * cols)
                                  : T(0);
                }
            } else {
                const T c = Q.c[n];
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = c;
            }
            // strip values: centre column rows r0-2..r0+P+1, columns i+-1 rows
            // r0-1..r0+P, columns i+-2 rows r0..r0+P-1 (rows past the band are
            // inside the padded buffer; their results are not stored)
            const T* cb = cur + (size_t)r0 * W + cc;
            T v0[P + 4], vm1[P + 2], vp1[P + 2], vm2[P], vp2[P];
#pragma unroll
            for (int q = 0; q < P + 4; q++) v0[q] = cb[(q - 2) * W];
#pragma unroll
            for (int q = 0; q < P + 2; q++) {
                vm1[q] = cb[(q - 1) * W - 1];
                vp1[q] = cb[(q - 1) * W + 1];
            }
#pragma unroll
            for (int q = 0; q < P; q++) {
                vm2[q] = cb[q * W - 2];
                vp2[q] = cb[q * W + 2];
            }
            // folded_residual tap order per point: (0,0) (-1,0) (1,0) (-2,0)
            // (2,0) (0,-1) (0,1) (0,-2) (0,2) (-1,-1) (1,-1) (-1,1) (1,1); the
            // P chains are independent and interleave
            T acc[P];
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][0], v0[p + 2], rh[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][1], vm1[p + 1], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][2], vp1[p + 1], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][3], vm2[p], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][4], vp2[p], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][5], v0[p + 1], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][6], v0[p + 3], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][7], v0[p], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][8], v0[p + 4], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][9], vm1[p], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][10], vp1[p], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][11], vm1[p + 2], acc[p]);
#pragma unroll
            for (int p = 0; p < P; p++) acc[p] = fma(cf[p][12], vp1[p + 2], acc[p]);
            T v[P];
#pragma unroll
            for (int p = 0; p < P; p++) v[p] = fma(cp[p] * dt[p], acc[p], v0[p + 2]);
            T* nb = nxt + (size_t)r0 * W + cc;
#pragma unroll
            for (int p = 0; p < P; p++)
                if (act[p]) nb[p * W] = v[p];
            if (has_side) {
                T* ns = nxt + (size_t)r0 * W + side;
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (act[p]) ns[p * W] = -v[p];
            }
            if (has_grow) {
#pragma unroll
                for (int p = 0; p < P; p++) {
                    if (!act[p]) continue;
                    if (kr + p == 1) nb[(p - 2) * W] = zsgn * v[p];
                    if (kr + p == b - 1) nb[(p + 2) * W] = zsgn * v[p];
                }
            }
            if (remote) {
                const uint32_t nbar = smem_addr(&bar[nxt_b]);
#pragma unroll
                for (int p = 0; p < P; p++) {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        if (!(remote & (1 << (4 * p + j)))) continue;
                        const int o = me + ((j < 2) ? j - 2 : j - 1);
                        const int ok0 = 1 + o * rpc;
                        const uint32_t dst = smem_addr(nxt + (size_t)(kr + p - ok0 + 2) * W + cc);
                        st_async(cluster_addr(dst, o), v[p], cluster_addr(nbar, o));
                    }
                }
            }
        }
        if (C > 1) {
            // the phase completes when every warp has stored its values (one
            // arrival per warp after __syncwarp) and the halo bytes of the
            // neighbours have landed; no block-wide barrier per sweep
            const uint32_t nb = smem_addr(&bar[nxt_b]);
            __syncwarp();
            if (tid == 0) mbar_arrive_expect(nb, expect);
            else if ((tid & 31) == 0) mbar_arrive(nb);
            int it = 0;
            bool to = false;
            while (!mbar_try_wait(nb, (phase >> nxt_b) & 1)) {
                if (++it > VISIT_WAIT_LIMIT) { to = true; break; }
            }
            phase ^= 1 << nxt_b;
            if (to) { timed_out = true; break; }
        } else {
            __syncthreads();
        }
        cur_b = nxt_b;
    }
    // one decision for the whole CTA: a thread that gave up leaves its loop
    // at once, the others give up at their next wait (its warp no longer
    // arrives), so every thread gets here
    timed_out = __syncthreads_or(timed_out ? 1 : 0) != 0;
    if (timed_out) {
        if (tid == 0) atomicExch(timeout_flag, 1);
    } else {
        // final state: owned rows (with side ghosts) to global, then the residual
        const T* fin = buf + (size_t)cur_b * bsz;
        const int wa = a + 1 + 2 * SP;
        for (int t = tid; t < (k1 - k0 + 1) * wa; t += NT) {
            const int rr = 2 + t / wa, c = t % wa;
            Sg[IX(L, c - SP, k0 - 2 + rr)] = fin[(size_t)rr * W + c];
        }
        if (res != nullptr || Q.rc != nullptr) {
            // residual of the final state at the owned points; with the fused
            // restriction it goes to a free buffer (where the neighbours' edge
            // rows k0-1 and k1+1 arrive too) instead of global memory
            T* rb = buf + (size_t)((cur_b + 1) % nbuf) * bsz;
#pragma unroll
            for (int p = 0; p < P; p++) {
                if (!act[p]) continue;
                const int r = r0 + p;
                const size_t xs = (size_t)r * W + cc;
                T acc = rh[p];
                acc = fma(cf[p][0], fin[xs], acc);
                acc = fma(cf[p][1], fin[xs - 1], acc);
                acc = fma(cf[p][2], fin[xs + 1], acc);
                acc = fma(cf[p][3], fin[xs - 2], acc);
                acc = fma(cf[p][4], fin[xs + 2], acc);
                acc = fma(cf[p][5], fin[xs - W], acc);
                acc = fma(cf[p][6], fin[xs + W], acc);
                acc = fma(cf[p][7], fin[xs - 2 * W], acc);
                acc = fma(cf[p][8], fin[xs + 2 * W], acc);
                acc = fma(cf[p][9], fin[xs - 1 - W], acc);
                acc = fma(cf[p][10], fin[xs + 1 - W], acc);
                acc = fma(cf[p][11], fin[xs - 1 + W], acc);
                acc = fma(cf[p][12], fin[xs + 1 + W], acc);
                if (Q.rc == nullptr) {
                    res[IX(L, i, kr + p)] = acc;
                    continue;
                }
                rb[xs] = acc;
                const int k = kr + p;
                if (k == k0 && me > 0) {
                    const int ok0 = 1 + (me - 1) * rpc;
                    const uint32_t dst = smem_addr(rb + (size_t)(k - ok0 + 2) * W + cc);
                    st_async(cluster_addr(dst, me - 1), acc, cluster_addr(smem_addr(&bar[3]), me - 1));
                }
                if (k == k1 && me < C - 1) {
                    const int ok0 = 1 + (me + 1) * rpc;
                    const uint32_t dst = smem_addr(rb + (size_t)(k - ok0 + 2) * W + cc);
                    st_async(cluster_addr(dst, me + 1), acc, cluster_addr(smem_addr(&bar[3]), me + 1));
                }
            }
        }
        if (Q.rc != nullptr) {
            int rto = 0;
            if (C > 1) {
                const int rexp = (((me > 0) ? cols : 0) + ((me < C - 1) ? cols : 0)) * (int)sizeof(T);
                if (tid == 0) mbar_arrive_expect(smem_addr(&bar[3]), rexp);
                __syncthreads();
                int it = 0, w = 0;
                while (!mbar_try_wait(smem_addr(&bar[3]), 0)) {
                    if (++it > VISIT_WAIT_LIMIT) { w = 1; break; }
                }
                rto = __syncthreads_or(w);
            } else {
                __syncthreads();
            }
            if (rto) {
                timed_out = true;
                if (tid == 0) atomicExch(timeout_flag, 1);
            } else {
                // restrict (iterative_solver.f90:596-626; restrict9's terms and
                // order, the repeated corner included) for the coarse rows K
                // whose fine centre row 2K this CTA owns
                const T* rb = buf + (size_t)((cur_b + 1) % nbuf) * bsz;
                const int ncol = Q.Lr.a - 1;
                const int K0 = max(1, (k0 + 1) / 2), K1 = min(Q.Lr.b - 1, k1 / 2);
                for (int t = tid; t < (K1 - K0 + 1) * ncol; t += NT) {
                    const int K = K0 + t / ncol, I = 1 + t % ncol;
                    const T* q = rb + (size_t)(2 * K - k0 + 2) * W + (2 * I + SP);
                    const T corners = (q[-W - 1] + q[W - 1] + q[W + 1] + q[W - 1]) / T(16);
                    const T sides = (q[-1] + q[-W] + q[1] + q[W]) / T(8);
                    const T centre = q[0] / T(4);
                    Q.rc[IX(Q.Lr, I, K)] = corners + sides + centre;
                }
                if (Q.zc != nullptr)
                    for (size_t t = (size_t)me * NT + tid; t < Q.zn; t += (size_t)C * NT) Q.zc[t] = T(0);
            }
        }
    }
    __threadfence();
    cl.sync();  // global rows written; no CTA leaves while another may still address its shared memory
    pdl_done();
    if (timed_out) return;
    // top/bottom ghost rows from the (now global) interior rows
    if (me == 0 || me == C - 1) {
        const int wa = a + 1 + 2 * SP;
        for (int t = tid; t < 2 * wa; t += NT) {
            const int g = 1 + t / wa, c = t % wa, ii = c - SP;
            if (me == 0) Sg[IX(L, ii, -g)] = zsgn * ld_state(Sg + IX(L, ii, g));
            if (me == C - 1) Sg[IX(L, ii, b + g)] = zsgn * ld_state(Sg + IX(L, ii, b - g));
        }
    }
}

// ---- host side ----------------------------------------------------------------
// shared-memory row-stride classes (a + 5 for a = 32..512, rounded to 8)
#define VISIT_FOR_EACH_W(X) X(40) X(72) X(136) X(264) X(520)
static int w_class(int a) {
    const int need = a + 1 + 2 * SP;
    const int cls[5] = {40, 72, 136, 264, 520};
    for (int c : cls)
        if (need <= c) return c;
    return 0;
}

template <typename T, int P, int NT, int W>
static bool visit_attrs1() {
    auto k = k_visit_cluster<T, P, NT, W>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return false;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, VISIT_SMEM_MAX) == cudaSuccess;
}
template <typename T, int P, int NT>
static bool visit_attrs() {
    bool ok = true;
#define X(w) ok = ok && visit_attrs1<T, P, NT, w>();
    VISIT_FOR_EACH_W(X)
#undef X
    return ok;
}

// Sets the kernel attributes; returns how many 16-CTA clusters of the
// largest configuration can be resident (0 = fused visits unavailable).
int visit_cluster_setup() {
    if (!visit_attrs<double, 1, 256>() || !visit_attrs<float, 1, 256>() || !visit_attrs<float, 2, 512>()) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(VISIT_MAX_CLUSTER, 1, 1);
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = VISIT_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = VISIT_MAX_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_visit_cluster<float, 2, 512, 520>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

struct VisitShape {
    int C, rpc, nt, p, w;
    size_t smem;
};

// FP32: strips of 4 points, as few CTAs as the columns allow (one CTA for a
// level whose rows fit; the sweep is bound by per-CTA shared-memory loads and
// the exchange, so fuller CTAs win).  FP64: strips of 1 point spread over up
// to 16 CTAs (the FP64 pipe of each SM is the bound, so more SMs win).
//
// cfg != 0 asks for a specific shape instead (tc_autotune): cfg = 100*P + C
// with P = 1 (256 threads) or 2 (512 threads, FP32 only) points per strip and
// C CTAs wanted; false if it does not fit.
static bool visit_shape(const Lay& L, int nsweeps, bool fp32, int cfg, VisitShape* s) {
    const int cols = L.a - 1, rows = L.b - 1;
    if (nsweeps > VISIT_MAX_SWEEPS || rows < 2 || cols < 1) return false;
    s->w = w_class(L.a);
    if (s->w == 0) return false;
    const int spread_C = rows < VISIT_MAX_CLUSTER ? rows : VISIT_MAX_CLUSTER;
    const int spread_rpc = (rows + spread_C - 1) / spread_C;
    if (cfg != 0) {
        const int p = cfg / 100, want = cfg % 100;
        if (!(p == 1 || (p == 2 && fp32)) || want < 1 || want > VISIT_MAX_CLUSTER) return false;
        s->p = p;
        s->nt = (p == 1) ? 256 : 512;
        s->rpc = (rows + want - 1) / want;
        s->C = (rows + s->rpc - 1) / s->rpc;
        if ((s->nt / cols) * p < s->rpc) return false;
    } else if (fp32 && spread_rpc * cols > 256) {
        // too many points to spread one per thread over 16 CTAs of 256:
        // 512 threads in strips of 2 (four warps per scheduler hide the
        // shared-memory and FMA latencies better than strips of 4 on 256)
        s->p = 2;
        s->nt = 512;
        if (cols > s->nt) return false;
        s->rpc = (s->nt / cols) * s->p;
        s->C = (rows + s->rpc - 1) / s->rpc;
    } else {
        // one point per thread over up to 16 CTAs: more SMs issue the sweep
        // (measured faster than fewer, fuller CTAs for levels of <= 4K points)
        s->p = 1;
        s->nt = 256;
        s->rpc = spread_rpc;
        s->C = (rows + s->rpc - 1) / s->rpc;
        if (s->rpc * cols > s->nt) return false;
    }
    if (s->C > VISIT_MAX_CLUSTER) return false;
    if (s->C == 1) s->rpc = rows;
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    const int nbuf = (s->C > 1) ? 3 : 2;
    const int rpcp = ((s->rpc + s->p - 1) / s->p) * s->p;
    s->smem = 32 + esz * nbuf * (size_t)(rpcp + 4) * (size_t)s->w;
    return s->smem <= VISIT_SMEM_MAX;
}

int visit_cluster_fits(const Lay& L, int nsweeps, int fp32, int cfg) {
    VisitShape s;
    return visit_shape(L, nsweeps, fp32 != 0, cfg, &s) ? 1 : 0;
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
// the FP32 smoother's per-point factors 2/(cA + cB*temp) in FP32 (temps rounded to float)
void launch_cheb_table32(cudaStream_t s, const Level& lv, const double* tvals, int nsweeps, float* tab) {
    cheb_table_t<float>(s, lv.L, tvals, nsweeps, lv.cA32, lv.cB32, tab);
}

template <typename T, int P, int NT>
static cudaError_t visit_launch(const VisitShape& sh, cudaStream_t s, const VisitParams<T>& Q, T* S, const T* coef,
                                const T* rhs, const T* dts, const T* ctab, const T* cA, const T* cB, T* res,
                                int* flag) {
    void (*kern)(VisitParams<T>, T*, const T*, const T*, const T*, const T*, const T*, const T*, T*, int*) = nullptr;
    switch (sh.w) {
#define X(w) \
    case w: kern = k_visit_cluster<T, P, NT, w>; break;
        VISIT_FOR_EACH_W(X)
#undef X
        default: return cudaErrorInvalidValue;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)sh.C, 1, 1);
    cfg.blockDim = dim3((unsigned)NT, 1, 1);
    cfg.dynamicSmemBytes = sh.smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)sh.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cudaLaunchKernelEx(&cfg, kern, Q, S, coef, rhs, dts, ctab, cA, cB, res, flag);
}

template <typename T>
static int visit_t(cudaStream_t s, const Lay& L, T* S, const T* coef, const T* rhs, const T* dts, const T* ctab,
                   const T* cA, const T* cB, T* res, const double* cvals, const double* tvals, int nsweeps,
                   int per_point, int Vbc, int* flag, int cfg, const VisitXfer<T>* x, const int* test_flag) {
    VisitShape sh;
    if (!visit_shape(L, nsweeps, sizeof(T) == sizeof(float), cfg, &sh)) return 1;
    if (per_point && sizeof(T) == sizeof(double) && ctab == nullptr) return 1;
    VisitParams<T> Q;
    Q.L = L;
    Q.nsweeps = nsweeps;
    Q.per_point = per_point;
    Q.Vbc = Vbc;
    Q.rpc = sh.rpc;
    const VisitXfer<T> none;
    const VisitXfer<T>& X = x ? *x : none;
    Q.ec = X.ec;
    Q.Lc = X.Lc;
    Q.rc = X.rc;
    Q.Lr = X.Lr;
    Q.zc = X.rc ? X.zc : nullptr;
    Q.zn = X.rc ? X.zn : 0;
    Q.test_flag = test_flag;
    for (int n = 0; n < nsweeps; n++) {
        Q.c[n] = (T)cvals[n];
        Q.temp[n] = (T)tvals[n];
    }
    cudaError_t e;
    if constexpr (sizeof(T) == sizeof(double)) {
        e = visit_launch<T, 1, 256>(sh, s, Q, S, coef, rhs, dts, ctab, cA, cB, res, flag);
    } else {
        if (sh.p == 1) e = visit_launch<T, 1, 256>(sh, s, Q, S, coef, rhs, dts, ctab, cA, cB, res, flag);
        else e = visit_launch<T, 2, 512>(sh, s, Q, S, coef, rhs, dts, ctab, cA, cB, res, flag);
    }
    if (e != cudaSuccess) return 2;
    tc_note_launch();
    return 0;
}

// Returns 0 if the level was handled here (caller skips the per-sweep path).
int launch_visit_cluster(cudaStream_t s, const Level& lv, double* S, const double* cvals, const double* tvals,
                         const double* ctab, int nsweeps, int per_point, int Vbc, int* timeout_flag,
                         const VisitXfer<double>* x, const int* test_flag) {
    return visit_t<double>(s, lv.L, S, lv.coef, lv.rhs, lv.dt_stream, ctab, lv.cA, lv.cB, lv.res, cvals, tvals,
                           nsweeps, per_point, Vbc, timeout_flag, lv.visit_cfg, x, test_flag);
}
int launch_visit_cluster32(cudaStream_t s, const Level& lv, float* S, const double* cvals, const double* tvals,
                           int nsweeps, int per_point, int Vbc, int* timeout_flag, const VisitXfer<float>* x,
                           const int* test_flag) {
    return visit_t<float>(s, lv.L, S, lv.coef32, lv.rhs32, lv.dts32, nullptr, lv.cA32, lv.cB32, lv.res32, cvals,
                          tvals, nsweeps, per_point, Vbc, timeout_flag, lv.visit_cfg, x, test_flag);
}
