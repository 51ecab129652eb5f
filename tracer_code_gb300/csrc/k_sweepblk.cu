// k_sweepblk.cu -- NS smoother sweeps (iterate_stream, iterative_solver.f90:
// 860-963, with enforceBCs_stream after each sweep) per launch on a 2-D tile.
//
// Why: on levels too large for one thread-block cluster a sweep is one launch
// of k_sweep / k_sweep32, and below ~300K points the launch-to-launch latency
// (about 1.2 us inside a graph with programmatic dependent launch) is most of
// its cost.  Here a CTA owns a TX x TY tile of interior points, loads the tile
// plus a halo 2*NS points deep into shared memory and runs NS sweeps there:
// sweep s computes the tile grown by 2*(NS-1-s) points on each side (the
// points of neighbouring tiles redundantly, from the same coefficients, so
// with identical values), and only the last sweep's tile goes to global
// memory.  NS sweeps cost one launch; the redundant halo work is small next to
// the latency it hides.
//
// Arithmetic per point is k_sweep's / k_sweep32's: the folded 13-point
// operator in folded_residual's tap order, c = 2/(cA + cB*temp) for the
// per-point Chebyshev level, v = fma(c*dt, r, psi).  Ghost taps (column -1 /
// a+1, row -1 / b+1, which enforceBCs_stream fills) take the mirrored interior
// value with the boundary sign inside the registers, so shared memory holds
// only interior and wall values; the final store writes the ghosts to global
// memory as store_stream does.  The result equals NS launches of the
// per-sweep kernel bit for bit.
//
// Thread layout: thread t owns column col = t % RX of the first sweep's
// region (RX = TX + 4(NS-1) columns) and a vertical strip of P points of it
// (strip t / RX); it keeps the strip's coefficients, RHS and dt in
// registers for all NS sweeps.
#include "tc_device.cuh"

template <typename T, int NS>
struct BlkParams {
    Lay L;
    int per_point, Vbc;
    T c[NS];     // uniform Chebyshev/Richardson factor of each sweep
    T temp[NS];  // Chebyshev node of each sweep (per-point factor)
};

template <typename T, int NS, int P, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, (sizeof(T) == sizeof(float) && NT <= 256) ? 2 : 1) k_sweep_blk(BlkParams<T, NS> Q, const T* Sin,
                                                     T* Sout, const T* __restrict__ coef,
                                                     const T* rhs, const T* __restrict__ dts,
                                                     const T* __restrict__ cA, const T* __restrict__ cB) {
    constexpr int RX = TX + 4 * (NS - 1), RY = TY + 4 * (NS - 1);  // first sweep's region
    constexpr int NSTR = NT / RX;                                   // strips across the region
    static_assert(NSTR * P >= RY, "strips must cover the region");
    constexpr int SX = TX + 4 * NS;  // shared row: region plus the 2-point stencil reach
    constexpr int SY = (NSTR * P + 4 > TY + 4 * NS) ? NSTR * P + 4 : TY + 4 * NS;
    __shared__ __align__(16) T sbuf[2][SY * SX];
    const Lay& L = Q.L;
    const int a = L.a, b = L.b;
    const int x0 = 1 + (int)blockIdx.x * TX, y0 = 1 + (int)blockIdx.y * TY;  // tile origin
    const int gx = x0 - 2 * NS, gy = y0 - 2 * NS;                            // shared (0,0)
    const int tid = threadIdx.x;
    const int col = tid % RX, strip = tid / RX;
    const int x = x0 - 2 * (NS - 1) + col;           // this thread's column
    const int kr = y0 - 2 * (NS - 1) + strip * P;     // first row of its strip
    const int cx = x - gx, r0 = kr - gy;              // shared coordinates of the strip's first point
    const T zsgn = (Q.Vbc == 1) ? T(1) : T(-1);
    const bool colok = (tid < NSTR * RX) && x >= 1 && x <= a - 1;
    const bool mir_l = (x == 1), mir_r = (x == a - 1);
    bool act[P];
    T cf[P][TC_NCOEF], rh[P], dt[P], ca[P], cbv[P];
    // coefficients, dt and Chebyshev denominators are fixed within a solve:
    // loaded before waiting for the previous kernel of the stream
#pragma unroll
    for (int p = 0; p < P; p++) {
        const int y = kr + p;
        act[p] = colok && (strip * P + p < RY) && y >= 1 && y <= b - 1;
        const size_t xg = IX(L, act[p] ? x : 1, act[p] ? y : 1);
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) cf[p][d] = act[p] ? -__ldg(coef + xg + (size_t)d * L.plane) : T(0);
        dt[p] = act[p] ? __ldg(dts + xg) : T(0);
        ca[p] = (Q.per_point && act[p]) ? __ldg(cA + xg) : T(1);
        cbv[p] = (Q.per_point && act[p]) ? __ldg(cB + xg) : T(0);
        rh[p] = T(0);
    }
    pdl_entry();
#pragma unroll
    for (int p = 0; p < P; p++)
        if (act[p]) rh[p] = ld_state(rhs + IX(L, x, kr + p));
    // the tile with its halo (walls included, ghosts and points outside the
    // array as zero: no active point reads them) into both buffers; all of a
    // thread's loads are issued before its first store
    {
        constexpr int NLD = (SY * SX + NT - 1) / NT;
        T v[NLD];
#pragma unroll
        for (int u = 0; u < NLD; u++) {
            const int t = tid + u * NT, sy = t / SX, sx = t % SX, yy = gy + sy, xx = gx + sx;
            v[u] = (t < SY * SX && xx >= -SP && xx <= a + SP && yy >= -SP && yy <= b + SP) ? ld_state(Sin + IX(L, xx, yy))
                                                                                           : T(0);
        }
#pragma unroll
        for (int u = 0; u < NLD; u++) {
            const int t = tid + u * NT;
            if (t < SY * SX) {
                sbuf[0][t] = v[u];
                sbuf[1][t] = v[u];
            }
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < NS; s++) {
        const T* cur = sbuf[s & 1];
        T* nxt = sbuf[(s + 1) & 1];
        const int e = 2 * (NS - 1 - s);  // points computed beyond the tile on each side
        const bool xin = x >= x0 - e && x <= x0 + TX - 1 + e;
        bool on[P];
        bool any = false;
#pragma unroll
        for (int p = 0; p < P; p++) {
            on[p] = act[p] && xin && kr + p >= y0 - e && kr + p <= y0 + TY - 1 + e;
            any = any || on[p];
        }
        T v[P];
        if (any) {
            T cp[P];
            if (Q.per_point) {
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = T(2) / (ca[p] + cbv[p] * Q.temp[s]);
            } else {
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = Q.c[s];
            }
            const T* cb = cur + r0 * SX + cx;
            T v0[P + 4], vm1[P + 2], vp1[P + 2], vm2[P], vp2[P];
#pragma unroll
            for (int q = 0; q < P + 4; q++) v0[q] = cb[(q - 2) * SX];
#pragma unroll
            for (int q = 0; q < P + 2; q++) {
                vm1[q] = cb[(q - 1) * SX - 1];
                vp1[q] = cb[(q - 1) * SX + 1];
            }
#pragma unroll
            for (int q = 0; q < P; q++) {
                vm2[q] = cb[q * SX - 2];
                vp2[q] = cb[q * SX + 2];
            }
            // ghost taps: row -1 mirrors row 1 and row b+1 row b-1 (sign zsgn),
            // column -1 mirrors column 1 and column a+1 column a-1 (sign -1)
#pragma unroll
            for (int q = 0; q < P + 2; q++)
                if (kr - 2 + q == -1) v0[q] = zsgn * v0[q + 2];
#pragma unroll
            for (int q = 2; q < P + 4; q++)
                if (kr - 2 + q == b + 1) v0[q] = zsgn * v0[q - 2];
            if (mir_l) {
#pragma unroll
                for (int q = 0; q < P; q++) vm2[q] = -v0[q + 2];
            }
            if (mir_r) {
#pragma unroll
                for (int q = 0; q < P; q++) vp2[q] = -v0[q + 2];
            }
            // folded_residual's tap order: (0,0) (-1,0) (1,0) (-2,0) (2,0)
            // (0,-1) (0,1) (0,-2) (0,2) (-1,-1) (1,-1) (-1,1) (1,1)
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
#pragma unroll
            for (int p = 0; p < P; p++) v[p] = fma(cp[p] * dt[p], acc[p], v0[p + 2]);
            if (s + 1 < NS) {
                T* nb = nxt + r0 * SX + cx;
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (on[p]) nb[p * SX] = v[p];
            } else {
                // the tile after the last sweep, with its ghost copies
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (on[p]) store_stream<T>(L, Sout, x, kr + p, v[p], Q.Vbc);
            }
        }
        if (s + 1 < NS) __syncthreads();
    }
    pdl_done();
}

// ---- level-1 FP32 variant: coefficients from the five viscosity fields ----------
// NS sweeps of k_sweep_g32 per launch on TX x TY tiles, as k_sweep_blk does
// them (the same region growth, ghost mirroring, tap order and final store),
// but each thread's 13 coefficients per point are formed once per launch from
// the fields G (fold_from_fields, k_sweep_g32's arithmetic) and kept in
// shared memory, [d][p][thread] (the register file cannot hold them for the
// tiles that fill the GPU in one wave at level 1).  Equal to NS launches of
// k_sweep_g32 bit for bit.
template <int NS, int P, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, 2) k_sweep_gblk(BlkParams<float, NS> Q, FoldG32 F, const float* Sin,
                                                      float* Sout, const float* __restrict__ g, const float* rhs,
                                                      const float* __restrict__ dts, const float* __restrict__ cA,
                                                      const float* __restrict__ cB) {
    constexpr int RX = TX + 4 * (NS - 1), RY = TY + 4 * (NS - 1);
    constexpr int NSTR = NT / RX;
    static_assert(NSTR * P >= RY, "strips must cover the region");
    constexpr int SX = TX + 4 * NS;
    constexpr int SY = (NSTR * P + 4 > TY + 4 * NS) ? NSTR * P + 4 : TY + 4 * NS;
    extern __shared__ __align__(16) float gsm[];
    float* sbuf0 = gsm;
    float* sbuf1 = gsm + SY * SX;
    float* scf = gsm + 2 * SY * SX;  // [TC_NCOEF][P][NT]
    const Lay& L = Q.L;
    const int a = L.a, b = L.b;
    const int x0 = 1 + (int)blockIdx.x * TX, y0 = 1 + (int)blockIdx.y * TY;
    const int gx = x0 - 2 * NS, gy = y0 - 2 * NS;
    const int tid = threadIdx.x;
    const int col = tid % RX, strip = tid / RX;
    const int x = x0 - 2 * (NS - 1) + col;
    const int kr = y0 - 2 * (NS - 1) + strip * P;
    const int cx = x - gx, r0 = kr - gy;
    const float zsgn = (Q.Vbc == 1) ? 1.f : -1.f;
    const bool colok = (tid < NSTR * RX) && x >= 1 && x <= a - 1;
    const bool mir_l = (x == 1), mir_r = (x == a - 1);
    const size_t pl = L.plane;
    bool act[P];
    float rh[P], dt[P], ca[P], cbv[P];
    // coefficients, dt and Chebyshev denominators are fixed within a solve:
    // formed before waiting for the previous kernel of the stream
#pragma unroll
    for (int p = 0; p < P; p++) {
        const int y = kr + p;
        act[p] = colok && (strip * P + p < RY) && y >= 1 && y <= b - 1;
        const size_t xg = IX(L, act[p] ? x : 1, act[p] ? y : 1);
        float G[5], cf[TC_NCOEF];
#pragma unroll
        for (int j = 0; j < 5; j++) G[j] = act[p] ? __ldg(g + xg + j * pl) : 0.f;
        fold_from_fields(F, G, cf);
#pragma unroll
        for (int d = 0; d < TC_NCOEF; d++) scf[(d * P + p) * NT + tid] = act[p] ? cf[d] : 0.f;
        dt[p] = act[p] ? __ldg(dts + xg) : 0.f;
        ca[p] = (Q.per_point && act[p]) ? __ldg(cA + xg) : 1.f;
        cbv[p] = (Q.per_point && act[p]) ? __ldg(cB + xg) : 0.f;
        rh[p] = 0.f;
    }
    pdl_entry();
#pragma unroll
    for (int p = 0; p < P; p++)
        if (act[p]) rh[p] = ld_state(rhs + IX(L, x, kr + p));
    {
        constexpr int NLD = (SY * SX + NT - 1) / NT;
        float v[NLD];
#pragma unroll
        for (int u = 0; u < NLD; u++) {
            const int t = tid + u * NT, sy = t / SX, sx = t % SX, yy = gy + sy, xx = gx + sx;
            v[u] = (t < SY * SX && xx >= -SP && xx <= a + SP && yy >= -SP && yy <= b + SP)
                       ? ld_state(Sin + IX(L, xx, yy))
                       : 0.f;
        }
#pragma unroll
        for (int u = 0; u < NLD; u++) {
            const int t = tid + u * NT;
            if (t < SY * SX) {
                sbuf0[t] = v[u];
                sbuf1[t] = v[u];
            }
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < NS; s++) {
        const float* cur = (s & 1) ? sbuf1 : sbuf0;
        float* nxt = (s & 1) ? sbuf0 : sbuf1;
        const int e = 2 * (NS - 1 - s);
        const bool xin = x >= x0 - e && x <= x0 + TX - 1 + e;
        bool on[P];
        bool any = false;
#pragma unroll
        for (int p = 0; p < P; p++) {
            on[p] = act[p] && xin && kr + p >= y0 - e && kr + p <= y0 + TY - 1 + e;
            any = any || on[p];
        }
        if (any) {
            float cp[P];
            if (Q.per_point) {
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = 2.0f / (ca[p] + cbv[p] * Q.temp[s]);
            } else {
#pragma unroll
                for (int p = 0; p < P; p++) cp[p] = Q.c[s];
            }
            const float* cb = cur + r0 * SX + cx;
            float v0[P + 4], vm1[P + 2], vp1[P + 2], vm2[P], vp2[P];
#pragma unroll
            for (int q = 0; q < P + 4; q++) v0[q] = cb[(q - 2) * SX];
#pragma unroll
            for (int q = 0; q < P + 2; q++) {
                vm1[q] = cb[(q - 1) * SX - 1];
                vp1[q] = cb[(q - 1) * SX + 1];
            }
#pragma unroll
            for (int q = 0; q < P; q++) {
                vm2[q] = cb[q * SX - 2];
                vp2[q] = cb[q * SX + 2];
            }
            // ghost taps: row -1 mirrors row 1 and row b+1 row b-1 (sign zsgn),
            // column -1 mirrors column 1 and column a+1 column a-1 (sign -1)
#pragma unroll
            for (int q = 0; q < P + 2; q++)
                if (kr - 2 + q == -1) v0[q] = zsgn * v0[q + 2];
#pragma unroll
            for (int q = 2; q < P + 4; q++)
                if (kr - 2 + q == b + 1) v0[q] = zsgn * v0[q - 2];
            if (mir_l) {
#pragma unroll
                for (int q = 0; q < P; q++) vm2[q] = -v0[q + 2];
            }
            if (mir_r) {
#pragma unroll
                for (int q = 0; q < P; q++) vp2[q] = -v0[q + 2];
            }
            // k_sweep_g32's tap order: (0,0) (-1,0) (1,0) (-2,0) (2,0) (0,-1)
            // (0,1) (0,-2) (0,2) (-1,-1) (1,-1) (-1,1) (1,1)
            float v[P];
#pragma unroll
            for (int p = 0; p < P; p++) {
                const float* c = scf + p * NT + tid;
                float acc = fmaf(c[0 * P * NT], v0[p + 2], rh[p]);
                acc = fmaf(c[1 * P * NT], vm1[p + 1], acc);
                acc = fmaf(c[2 * P * NT], vp1[p + 1], acc);
                acc = fmaf(c[3 * P * NT], vm2[p], acc);
                acc = fmaf(c[4 * P * NT], vp2[p], acc);
                acc = fmaf(c[5 * P * NT], v0[p + 1], acc);
                acc = fmaf(c[6 * P * NT], v0[p + 3], acc);
                acc = fmaf(c[7 * P * NT], v0[p], acc);
                acc = fmaf(c[8 * P * NT], v0[p + 4], acc);
                acc = fmaf(c[9 * P * NT], vm1[p], acc);
                acc = fmaf(c[10 * P * NT], vp1[p], acc);
                acc = fmaf(c[11 * P * NT], vm1[p + 2], acc);
                acc = fmaf(c[12 * P * NT], vp1[p + 2], acc);
                v[p] = fmaf(cp[p] * dt[p], acc, v0[p + 2]);
            }
            if (s + 1 < NS) {
                float* nb = nxt + r0 * SX + cx;
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (on[p]) nb[p * SX] = v[p];
            } else {
#pragma unroll
                for (int p = 0; p < P; p++)
                    if (on[p]) store_stream<float>(L, Sout, x, kr + p, v[p], Q.Vbc);
            }
        }
        if (s + 1 < NS) __syncthreads();
    }
    pdl_done();
}

// ---- host side ----------------------------------------------------------------
int sweep_blk_tiles(const Lay& L) { return ((L.a - 1 + 31) / 32) * ((L.b - 1 + 15) / 16); }

// tiles of TX = 32 x TY = 16 interior points; (NS, P, NT) below
template <typename T, int NS, int P, int NT>
static bool blk_launch(cudaStream_t s, const Level& lv, const T* Sin, T* Sout, const T* coef, const T* rhs,
                       const T* dts, const T* cA, const T* cB, const float* cvals, const float* tvals, int per_point,
                       int Vbc) {
    constexpr int TX = 32, TY = 16;
    BlkParams<T, NS> Q;
    Q.L = lv.L;
    Q.per_point = per_point;
    Q.Vbc = Vbc;
    for (int n = 0; n < NS; n++) {
        Q.c[n] = (T)cvals[n];
        Q.temp[n] = (T)tvals[n];
    }
    const dim3 grid((unsigned)((lv.L.a - 1 + TX - 1) / TX), (unsigned)((lv.L.b - 1 + TY - 1) / TY), 1);
    if (launch_pdl(k_sweep_blk<T, NS, P, TX, TY, NT>, grid, dim3(NT), 0, s, Q, Sin, Sout, coef, rhs, dts, cA, cB) !=
        cudaSuccess)
        return false;
    tc_note_launch();
    return true;
}

// NS = 1..6 sweeps of the FP32 smoother (c/temp: the NS sweeps' factors,
// already rounded to float as launch_sweep32 receives them).  256 threads
// for NS <= 3 (two CTAs per SM), 512 for deeper halos.
bool launch_sweep_blk32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, int ns, const float* c,
                        const float* temp, int per_point, int Vbc) {
#define BLK32(NS, P, NT)                                                                                            \
    case NS:                                                                                                      \
        return blk_launch<float, NS, P, NT>(s, lv, Sin, Sout, lv.coef32, lv.rhs32, lv.dts32, lv.cA32, lv.cB32, c, \
                                            temp, per_point, Vbc);
    switch (ns) {
        BLK32(1, 2, 256)
        BLK32(2, 3, 256)
        BLK32(3, 4, 256)
        BLK32(4, 3, 512)
        BLK32(5, 4, 512)
        BLK32(6, 4, 512)
        default: return false;
    }
#undef BLK32
}

// NS = 2 sweeps of the FP64 smoother (c/temp as launch_sweep receives them)
template <int NS, int P>
static bool blk_launch64(cudaStream_t s, const Level& lv, const double* Sin, double* Sout, const double* c,
                         const double* temp, int per_point, int Vbc) {
    constexpr int TX = 32, TY = 16, NT = 256;
    BlkParams<double, NS> Q;
    Q.L = lv.L;
    Q.per_point = per_point;
    Q.Vbc = Vbc;
    for (int n = 0; n < NS; n++) {
        Q.c[n] = c[n];
        Q.temp[n] = temp[n];
    }
    const dim3 grid((unsigned)((lv.L.a - 1 + TX - 1) / TX), (unsigned)((lv.L.b - 1 + TY - 1) / TY), 1);
    if (launch_pdl(k_sweep_blk<double, NS, P, TX, TY, NT>, grid, dim3(NT), 0, s, Q, Sin, Sout, lv.coef, lv.rhs,
                   lv.dt_stream, lv.cA, lv.cB) != cudaSuccess)
        return false;
    tc_note_launch();
    return true;
}
bool launch_sweep_blk64(cudaStream_t s, const Level& lv, const double* Sin, double* Sout, int ns, const double* c,
                        const double* temp, int per_point, int Vbc) {
    if (ns == 1) return blk_launch64<1, 2>(s, lv, Sin, Sout, c, temp, per_point, Vbc);
    if (ns == 2) return blk_launch64<2, 3>(s, lv, Sin, Sout, c, temp, per_point, Vbc);
    return false;
}

// NS = 2 or 3 sweeps of the level-1 field sweep (k_sweep_g32) per launch on
// 64 x 16 tiles, two CTAs per SM (the 256 tiles of 1023 x 255 in one wave)
template <int NS, int P, int NT>
static bool gblk_launch(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, const float* cvals,
                        const float* tvals, int per_point, int Vbc) {
    constexpr int TX = 64, TY = 16;
    constexpr int RX = TX + 4 * (NS - 1);
    constexpr int NSTR = NT / RX;
    constexpr int SX = TX + 4 * NS;
    constexpr int SY = (NSTR * P + 4 > TY + 4 * NS) ? NSTR * P + 4 : TY + 4 * NS;
    constexpr size_t smem = sizeof(float) * ((size_t)2 * SY * SX + (size_t)TC_NCOEF * P * NT);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_sweep_gblk<NS, P, TX, TY, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return false;
        attr = true;
    }
    BlkParams<float, NS> Q;
    Q.L = lv.L;
    Q.per_point = per_point;
    Q.Vbc = Vbc;
    for (int n = 0; n < NS; n++) {
        Q.c[n] = cvals[n];
        Q.temp[n] = tvals[n];
    }
    const dim3 grid((unsigned)((lv.L.a - 1 + TX - 1) / TX), (unsigned)((lv.L.b - 1 + TY - 1) / TY), 1);
    if (launch_pdl(k_sweep_gblk<NS, P, TX, TY, NT>, grid, dim3(NT), smem, s, Q, lv.gw, Sin, Sout,
                   (const float*)lv.g32, (const float*)lv.rhs32, (const float*)lv.dts32, (const float*)lv.cA32,
                   (const float*)lv.cB32) != cudaSuccess)
        return false;
    tc_note_launch();
    return true;
}

bool launch_sweep_gblk32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, int ns, const float* c,
                         const float* temp, int per_point, int Vbc) {
    if (lv.g32 == nullptr) return false;
    if (ns == 2) return gblk_launch<2, 3, 476>(s, lv, Sin, Sout, c, temp, per_point, Vbc);
    if (ns == 3) return gblk_launch<3, 3, 576>(s, lv, Sin, Sout, c, temp, per_point, Vbc);
    return false;
}
