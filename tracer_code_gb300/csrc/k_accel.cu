// k_accel.cu -- residual-minimising corrections of the level-1
// streamfunction along a few directions: the learned start and the
// correction after every level-1 visit (the learned coarse-level correction).
//
// Given the current streamfunction psi (level 1, FP64), its RHS and the
// folded operator A, and directions v_1..v_m (m <= 2), the correction
//
//     psi <- psi + sum_j alpha_j v_j,   G alpha = b,
//     G_ij = sum w (A v_i)(A v_j),   b_i = sum w (A v_i) r,   r = RHS - A psi,
//     w = 1 / |r|                                        (interior sums)
//
// minimises the weighted 2-norm sum w (r - sum_j alpha_j A v_j)^2, which at
// alpha = 0 equals the L1 norm of the residual -- the norm of the
// reference's convergence test (iterative_solver.f90:147-156) -- and is one
// reweighted least-squares step towards its minimum over psi + span{v_j}.
// The plain 2-norm (w = 1) and the energy-norm Galerkin step do not work
// here: at 1024x256 with a 1e5 viscosity contrast the W-cycle lowers the L1
// residual but not its 2-norm, and both steps drove alpha to -1 (cancelling
// each cycle) and stalled the solve; pseudo-time-step weights stalled too.
// The directions used:
//
//   DNN   the network's predicted solution change (its guess minus the
//         streamfunction it started from), formed once per multigrid call;
//   DK    psi's change over the last W-cycle, psi - psi_prev (psi_prev = psi
//         after the previous correction).
//
// One kernel forms A v_j and the residual at every interior point and the
// sums (deterministic block partials, fixed-order fold by the last block),
// whose last block also solves the 2x2 (or 1x1) system into the device
// scalars; a second kernel applies the update with the stream BCs' ghost
// copies and, for DK, records psi_prev.  No host synchronisation, so both
// run inside the W-cycle's CUDA graph.  Safeguards: a direction with
// A v = 0, or a 2x2 system whose determinant is below 1e-12 of the product
// of its diagonal (nearly parallel directions), drops to the 1x1 system of
// the first direction (or to no correction).
#include "tc_device.cuh"

namespace {

constexpr int kNV = 6;  // sums: G11, G12, G21 (= G12), G22, b1, b2

// direction value at offset y: DK = psi - psi_prev, DNN = dnn
__device__ __forceinline__ double dir_at(int kind, const double* psi, const double* prev, const double* dnn, size_t y) {
    return kind == TC_ACCEL_DK ? ld_state(psi + y) - ld_state(prev + y) : ld_state(dnn + y);
}

// grid-stride over the interior points (a fixed number of blocks keeps the
// final fold short: each of the six sums is folded by its own warp)
__global__ void __launch_bounds__(256) k_accel_dots(Lay L, const double* __restrict__ coef, const double* rhs,
                                                    const double* psi, const double* prev, const double* dnn, int k1,
                                                    int k2, RedScratch rs, DevScalars* ds) {
    pdl_entry();
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    const int a1i = L.a - 1, npts = (L.a - 1) * (L.b - 1);
    const bool useq = (k1 == TC_ACCEL_DK || k2 == TC_ACCEL_DK), usen = (k1 == TC_ACCEL_DNN || k2 == TC_ACCEL_DNN);
    double s[kNV] = {0, 0, 0, 0, 0, 0};
    for (int pnt = blockIdx.x * blockDim.x + threadIdx.x; pnt < npts; pnt += gridDim.x * blockDim.x) {
        const size_t x = IX(L, 1 + pnt % a1i, 1 + pnt / a1i);
        // A psi, A v1, A v2 from one load of each tap
        double ap = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) {
            const double c = __ldg(coef + x + d * L.plane);
            const size_t y = (size_t)((ptrdiff_t)x + off[d]);
            const double p = ld_state(psi + y);
            const double q = useq ? ld_state(prev + y) : 0.0;
            const double n = usen ? ld_state(dnn + y) : 0.0;
            ap = fma(c, p, ap);
            a1 = fma(c, (k1 == TC_ACCEL_DK) ? p - q : n, a1);
            if (k2 != TC_ACCEL_NONE) a2 = fma(c, (k2 == TC_ACCEL_DK) ? p - q : n, a2);
        }
        const double res = ld_state(rhs + x) - ap;
        // w = 1/|r| (a weight: single-precision reciprocal is enough)
        const float fr = fabsf((float)res);
        const double w = (fr > 0.0f) ? (double)(1.0f / fr) : 0.0;
        const double wa1 = w * a1, wa2 = w * a2;
        s[0] += wa1 * a1;
        s[1] += wa1 * a2;
        s[3] += wa2 * a2;
        s[4] += wa1 * res;
        s[5] += wa2 * res;
    }
    s[2] = s[1];
    // block sums (warp shuffle, then one warp over the warps' partials)
    __shared__ double sh[kNV][32];
    __shared__ bool last;
    const int tid = threadIdx.x;
    const int nth = blockDim.x;
    const int bid = blockIdx.x;
    const int nb = gridDim.x;
#pragma unroll
    for (int q = 0; q < kNV; q++) {
        double v = s[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) sh[q][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < 32) {
#pragma unroll
        for (int q = 0; q < kNV; q++) {
            double v = (tid < ((nth + 31) >> 5)) ? sh[q][tid] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (tid == 0) rs.part[(size_t)q * nb + bid] = v;
        }
        if (tid == 0) {
            __threadfence();
            const unsigned int t = atomicAdd(rs.count, 1u);
            last = (t == (unsigned int)(nb - 1));
        }
    }
    __syncthreads();
    if (last) {
        __threadfence();
        // warp q folds sum q over the blocks (lane-strided, fixed order)
        __shared__ double tot[kNV];
        const int wq = tid >> 5, lane = tid & 31;
        if (wq < kNV) {
            double v = 0.0;
            for (int b = lane; b < nb; b += 32) v += __ldcg(rs.part + (size_t)wq * nb + b);
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) tot[wq] = v;
        }
        __syncthreads();
        if (tid == 0) {
            double al1 = 0.0, al2 = 0.0;
            const double g11 = tot[0], g12 = tot[1], g21 = tot[2], g22 = tot[3], b1 = tot[4], b2 = tot[5];
            bool done = false;
            if (k2 != TC_ACCEL_NONE && g11 > 0.0 && g22 > 0.0) {
                const double det = g11 * g22 - g12 * g21;
                if (fabs(det) > 1e-12 * g11 * g22) {
                    al1 = (b1 * g22 - g12 * b2) / det;
                    al2 = (g11 * b2 - g21 * b1) / det;
                    done = true;
                }
            }
            if (!done) {
                // one direction: the first if usable, else the second
                if (g11 > 0.0) al1 = b1 / g11;
                else if (k2 != TC_ACCEL_NONE && g22 > 0.0) al2 = b2 / g22;
            }
            ds->acc_alpha[0] = al1;
            ds->acc_alpha[1] = al2;
            *rs.count = 0u;
        }
    }
    pdl_done();
}

__global__ void k_accel_update(Lay L, Range2 r, double* psi, double* prev, const double* dnn, int k1, int k2,
                               const DevScalars* ds, int record_prev, int Vbc) {
    pdl_entry();
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(L, i, k);
    const double al1 = __ldcg(&ds->acc_alpha[0]), al2 = __ldcg(&ds->acc_alpha[1]);
    const double p0 = ld_state(psi + x);
    const double v1 = dir_at(k1, psi, prev, dnn, x);
    const double v2 = (k2 != TC_ACCEL_NONE) ? dir_at(k2, psi, prev, dnn, x) : 0.0;
    const double pn = p0 + al1 * v1 + al2 * v2;
    store_stream<double>(L, psi, i, k, pn, Vbc);
    if (record_prev) store_stream<double>(L, prev, i, k, pn, Vbc);
    pdl_done();
}

// dst = a - b over the whole plane (ghosts included: both follow the same
// linear mirror rule, so the difference does too)
__global__ void k_plane_diff(double* dst, const double* a, const double* b, size_t n) {
    pdl_entry();
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        dst[t] = ld_state(a + t) - ld_state(b + t);
    pdl_done();
}

// ---- windowed correction ---------------------------------------------------
// Directions j = 0..nd-1: j = 0 the newest change d = psi - prev (written to
// slot (head + 1) % TC_WIN this launch), j = 1..nold the stored changes from
// the newest back, then the network's direction.  Sums: the upper triangle
// of G (kWT entries, row-major over kWD) and b.
//
// One stencil application per cycle: with rp = RHS - A prev (kept from the
// previous correction, see k_win_update) and r = RHS - A psi, the newest
// direction's image is A d = rp - r, and the network direction's image A dnn
// is formed once per solve (k_win_init).
constexpr int kWD = TC_WIN + 1;               // directions at most
constexpr int kWT = kWD * (kWD + 1) / 2;      // Gram entries
constexpr int kWS = kWT + kWD;                // sums

__device__ __forceinline__ int win_slot(int head, int back) { return (head - back + 2 * TC_WIN) % TC_WIN; }

// rp = RHS - A prev and, with a network direction, A dnn (interior points)
__global__ void k_win_init(Lay L, Range2 r, const double* __restrict__ coef, const double* rhs, const double* prev,
                           const double* dnn, double* rp, double* adnn) {
    RANGE_IK(r);
    if (!inr) return;
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    const size_t x = IX(L, i, k);
    double ap = 0.0, an = 0.0;
#pragma unroll
    for (int d = 0; d < TC_NCOEF; d++) {
        const double c = __ldg(coef + x + d * L.plane);
        const size_t y = (size_t)((ptrdiff_t)x + off[d]);
        ap = fma(c, ld_state(prev + y), ap);
        if (adnn) an = fma(c, ld_state(dnn + y), an);
    }
    rp[x] = ld_state(rhs + x) - ap;
    if (adnn) adnn[x] = an;
}

// the grid-stride sums for ND directions
template <int ND>
__device__ __forceinline__ void win_sums(const Lay& L, const double* __restrict__ coef, const double* rhs,
                                         const double* psi, const double* prev, const double* rp, double* P,
                                         double* AP, double* rn, const double* adnn, int snew, int nold,
                                         double* s) {
    const ptrdiff_t ld = (ptrdiff_t)L.ld;
    const ptrdiff_t off[TC_NCOEF] = {0, -1, 1, -2, 2, -ld, ld, -2 * ld, 2 * ld, -1 - ld, 1 - ld, -1 + ld, 1 + ld};
    const int a1i = L.a - 1, npts = (L.a - 1) * (L.b - 1);
    for (int pnt = blockIdx.x * blockDim.x + threadIdx.x; pnt < npts; pnt += gridDim.x * blockDim.x) {
        const size_t x = IX(L, 1 + pnt % a1i, 1 + pnt / a1i);
        // all loads first (coefficients, taps, the stored images), then the arithmetic
        double cf[TC_NCOEF], tp[TC_NCOEF];
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) {
            cf[d] = __ldg(coef + x + d * L.plane);
            tp[d] = ld_state(psi + (size_t)((ptrdiff_t)x + off[d]));
        }
        double old[ND > 1 ? ND - 1 : 1];
#pragma unroll
        for (int j = 1; j < ND; j++)
            old[j - 1] = (j <= nold) ? ld_state(AP + (size_t)win_slot(snew, j) * L.plane + x) : ld_state(adnn + x);
        const double rhsx = ld_state(rhs + x), rpx = ld_state(rp + x), px0 = ld_state(prev + x);
        double ap = 0.0;
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) ap = fma(cf[d], tp[d], ap);
        const double res = rhsx - ap;
        double v[ND];
        v[0] = rpx - res;  // A (psi - prev)
        P[(size_t)snew * L.plane + x] = tp[0] - px0;
        AP[(size_t)snew * L.plane + x] = v[0];
        rn[x] = res;
#pragma unroll
        for (int j = 1; j < ND; j++) v[j] = old[j - 1];
        // w = 1/|r| (a weight: single-precision reciprocal is enough)
        const float fr = fabsf((float)res);
        const double w = (fr > 0.0f) ? (double)(1.0f / fr) : 0.0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            const double wi = w * v[i];
            const int row = i * kWD - i * (i - 1) / 2;  // upper-triangle start of row i over kWD
#pragma unroll
            for (int j = i; j < ND; j++) s[row + (j - i)] += wi * v[j];
            s[kWT + i] += wi * res;
        }
    }
}

__global__ void __launch_bounds__(256) k_win_dots(Lay L, const double* __restrict__ coef, const double* rhs,
                                                  const double* psi, const double* prev, const double* rp, double* P,
                                                  double* AP, double* rn, const double* adnn, int use_dnn,
                                                  RedScratch rs, DevScalars* ds) {
    pdl_entry();
    const int n = __ldcg(&ds->win_n), head = __ldcg(&ds->win_head);
    const int nold = min(n, TC_WIN - 1);
    // the network's direction joins the corrections while the window of
    // changes fills; once it holds TC_WIN changes their span has taken up
    // what the direction adds, and the correction costs what it costs
    // without the network
    const int dnn_now = (use_dnn && n < TC_WIN) ? 1 : 0;
    const int nd = 1 + nold + dnn_now;
    const int snew = (n == 0) ? 0 : (head + 1) % TC_WIN;
    double s[kWS];
#pragma unroll
    for (int q = 0; q < kWS; q++) s[q] = 0.0;
    // the direction count is the same for the whole grid
    switch (nd) {
        case 1: win_sums<1>(L, coef, rhs, psi, prev, rp, P, AP, rn, adnn, snew, nold, s); break;
        case 2: win_sums<2>(L, coef, rhs, psi, prev, rp, P, AP, rn, adnn, snew, nold, s); break;
        case 3: win_sums<3>(L, coef, rhs, psi, prev, rp, P, AP, rn, adnn, snew, nold, s); break;
        case 4: win_sums<4>(L, coef, rhs, psi, prev, rp, P, AP, rn, adnn, snew, nold, s); break;
        default: win_sums<kWD>(L, coef, rhs, psi, prev, rp, P, AP, rn, adnn, snew, nold, s); break;
    }
    // block sums (warp shuffle, then one warp over the warps' partials)
    __shared__ double sh[kWS][16];
    __shared__ bool last;
    const int tid = threadIdx.x, bid = blockIdx.x, nb = gridDim.x;
#pragma unroll
    for (int q = 0; q < kWS; q++) {
        double v = s[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) sh[q][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < 32) {
        for (int q = 0; q < kWS; q++) {
            double v = (tid < (int)(blockDim.x >> 5)) ? sh[q][tid] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (tid == 0) rs.part[(size_t)q * nb + bid] = v;
        }
        if (tid == 0) {
            __threadfence();
            const unsigned int t = atomicAdd(rs.count, 1u);
            last = (t == (unsigned int)(nb - 1));
        }
    }
    __syncthreads();
    if (!last) {
        pdl_done();
        return;
    }
    __threadfence();
    // warp w folds sums w, w + 8, ... over the blocks (lane-strided, fixed order)
    __shared__ double tot[kWS];
    {
        const int wq = tid >> 5, lane = tid & 31;
        for (int q = wq; q < kWS; q += (int)(blockDim.x >> 5)) {
            double v = 0.0;
            const double* pq = rs.part + (size_t)q * nb;
            int b = lane;
            for (; b + 32 * 7 < nb; b += 32 * 8) {
                double t[8];
#pragma unroll
                for (int u = 0; u < 8; u++) t[u] = __ldcg(pq + b + 32 * u);
#pragma unroll
                for (int u = 0; u < 8; u++) v += t[u];
            }
            for (; b < nb; b += 32) v += __ldcg(pq + b);
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) tot[q] = v;
        }
    }
    __syncthreads();
    if (tid == 0) {
        // LDL^T of G in direction order, dropping a direction whose pivot
        // falls below 1e-10 of its diagonal (nearly in the span of the kept
        // ones) or whose diagonal is not positive; then G beta = b on the
        // kept directions
        double G[kWD][kWD], Lm[kWD][kWD], D[kWD], y[kWD], beta[kWD];
        bool keep[kWD];
        int t = 0;
        for (int i = 0; i < kWD; i++)
            for (int j = i; j < kWD; j++) {
                G[i][j] = tot[t];
                G[j][i] = tot[t];
                t++;
            }
        for (int i = 0; i < kWD; i++) {
            keep[i] = false;
            D[i] = 0.0;
            beta[i] = 0.0;
            y[i] = 0.0;
            for (int j = 0; j < kWD; j++) Lm[i][j] = 0.0;
        }
        for (int j = 0; j < nd; j++) {
            double dj = G[j][j];
            for (int k = 0; k < j; k++)
                if (keep[k]) dj -= Lm[j][k] * Lm[j][k] * D[k];
            if (!(G[j][j] > 0.0) || !(dj > 1e-10 * G[j][j])) continue;
            keep[j] = true;
            D[j] = dj;
            Lm[j][j] = 1.0;
            for (int i = j + 1; i < nd; i++) {
                double v = G[i][j];
                for (int k = 0; k < j; k++)
                    if (keep[k]) v -= Lm[i][k] * Lm[j][k] * D[k];
                Lm[i][j] = v / dj;
            }
        }
        for (int i = 0; i < nd; i++) {
            if (!keep[i]) continue;
            double v = tot[kWT + i];
            for (int k = 0; k < i; k++)
                if (keep[k]) v -= Lm[i][k] * y[k];
            y[i] = v;
        }
        for (int i = nd - 1; i >= 0; i--) {
            if (!keep[i]) continue;
            double v = y[i] / D[i];
            for (int k = i + 1; k < nd; k++)
                if (keep[k]) v -= Lm[k][i] * beta[k];
            beta[i] = v;
        }
        for (int i = 0; i < kWD; i++) ds->win_beta[i] = beta[i];
        ds->win_nd = nd;
        ds->win_dnn = dnn_now;
        ds->win_head = snew;
        ds->win_n = min(n + 1, TC_WIN);
        *rs.count = 0u;
    }
    pdl_done();
}

// psi += sum_j beta_j v_j (ghosts by the stream BCs); prev = the new psi;
// rp = r - sum_j beta_j A v_j, the residual of the new psi by linearity
// (from this cycle's directly computed r, so rounding does not accumulate),
// also written to the level's residual plane with its mean |.| (the value
// the convergence test reads, as the residual kernel would give it up to
// rounding)
__global__ void k_win_update(Lay L, Range2 r, double* psi, double* prev, const double* P, const double* AP,
                             const double* rn, double* rp, const double* dnn, const double* adnn, int use_dnn,
                             const DevScalars* ds, int Vbc, double* res, RedScratch rs, double* res_out,
                             double div1, double div2) {
    pdl_entry();
    RANGE_IK(r);
    double mag = 0.0;
    if (inr) {
    const size_t x = IX(L, i, k);
    const int nd = __ldcg(&ds->win_nd), head = __ldcg(&ds->win_head);
    const int dnn_now = use_dnn ? __ldcg(&ds->win_dnn) : 0;
    const int nold = nd - 1 - dnn_now;
    double beta[kWD], pv[kWD], av[kWD];
#pragma unroll
    for (int j = 0; j < kWD; j++) beta[j] = __ldcg(&ds->win_beta[j]);
    // every used direction's values loaded before the sums (a zero beta
    // adds nothing); the network's direction sits in the last used slot
#pragma unroll
    for (int j = 0; j < kWD; j++) {
        pv[j] = 0.0;
        av[j] = 0.0;
        if (j <= nold) {
            const size_t o = (size_t)win_slot(head, j) * L.plane + x;
            pv[j] = ld_state(P + o);
            av[j] = ld_state(AP + o);
        } else if (dnn_now && j == nd - 1) {
            pv[j] = ld_state(dnn + x);
            av[j] = ld_state(adnn + x);
        }
    }
    double pn = ld_state(psi + x), rr = ld_state(rn + x);
#pragma unroll
    for (int j = 0; j < kWD; j++) {
        if (j >= nd) break;
        pn += beta[j] * pv[j];
        rr -= beta[j] * av[j];
    }
    store_stream<double>(L, psi, i, k, pn, Vbc);
    store_stream<double>(L, prev, i, k, pn, Vbc);
    rp[x] = rr;
    res[x] = rr;
    mag = fabs(rr);
    }
    reduce_to(RED_SUM, mag, rs.part, rs.count, res_out, div1, div2);
    pdl_done();
}

}  // namespace

void launch_accel_window_init(cudaStream_t s, const Level& l1, const double* prev, const double* dnn, double* rp,
                              double* adnn) {
    Range2 r{1, l1.L.a - 1, 1, l1.L.b - 1};
    k_win_init<<<grid_for(r), dim3(BX, BY), 0, s>>>(l1.L, r, (const double*)l1.coef, (const double*)l1.rhs, prev,
                                                   dnn, rp, adnn);
    tc_note_launch();
}

void launch_accel_window(cudaStream_t s, const Level& l1, double* psi, double* prev, double* P, double* AP,
                         double* rn, double* rp, const double* dnn, const double* adnn, int use_dnn, RedScratch rs,
                         DevScalars* ds, int Vbc) {
    Range2 r{1, l1.L.a - 1, 1, l1.L.b - 1};
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
    }
    const int npts = (l1.L.a - 1) * (l1.L.b - 1);
    // grid-stride over the points with one wave of CTAs (three per SM: the
    // kernel's launch bounds), so that the block sums and their fold stay few
    // one CTA of 256 threads per SM, grid-stride over the points: the block
    // sums of the up to 20 FP64 products cost per thread, so few threads with
    // several points each are fastest (measured at 1024x256: 1 x SMs 306 us per
    // level-1 visit, 2 x 317, 3 x 326, 6 x 358; 512 threads 317)
    int nb = (npts + 255) / 256;
    if (nb > nsm) nb = nsm;
    launch_pdl(k_win_dots, dim3((unsigned)nb), dim3(256), 0, s, l1.L, (const double*)l1.coef,
               (const double*)l1.rhs, (const double*)psi, (const double*)prev, (const double*)rp, P, AP, rn, adnn,
               use_dnn, rs, ds);
    launch_pdl(k_win_update, grid_for(r), dim3(BX, BY), 0, s, l1.L, r, psi, prev, (const double*)P,
               (const double*)AP, (const double*)rn, rp, dnn, adnn, use_dnn, (const DevScalars*)ds, Vbc, l1.res, rs,
               &ds->res_mag[1], (double)(l1.L.a - 1), (double)(l1.L.b - 1));
    tc_note_launch(2);
}

void launch_accel(cudaStream_t s, const Level& l1, double* psi, double* prev, const double* dnn, int k1, int k2,
                  int record_prev, RedScratch rs, DevScalars* ds, int Vbc) {
    Range2 r{1, l1.L.a - 1, 1, l1.L.b - 1};
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
    }
    const int npts = (l1.L.a - 1) * (l1.L.b - 1);
    int nb = (npts + 255) / 256;
    if (nb > 2 * nsm) nb = 2 * nsm;
    launch_pdl(k_accel_dots, dim3((unsigned)nb), dim3(256), 0, s, l1.L, (const double*)l1.coef,
               (const double*)l1.rhs, (const double*)psi, (const double*)prev, dnn, k1, k2, rs, ds);
    launch_pdl(k_accel_update, grid_for(r), dim3(BX, BY), 0, s, l1.L, r, psi, prev, dnn, k1, k2,
               (const DevScalars*)ds, record_prev, Vbc);
    tc_note_launch(2);
}

void launch_plane_diff(cudaStream_t s, double* dst, const double* a, const double* b, size_t n) {
    int nb = (int)((n + 255) / 256);
    if (nb > 2048) nb = 2048;
    launch_pdl(k_plane_diff, dim3((unsigned)nb), dim3(256), 0, s, dst, a, b, n);
    tc_note_launch();
}
