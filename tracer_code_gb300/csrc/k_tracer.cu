// k_tracer.cu -- tracer kernels: Runge-Kutta stage updates with the
// grid-to-tracer Taylor interpolant, the per-corner-volume histogram and the
// tracer-ratio composition.
//
// Reference: energy.f90:169-225,261-315,352-381,417-443 (tracer loops of
// energy_time), composition.f90:838-898 (interpolate) and 669-803
// (tracers_to_corners, enforceBCs_comp).  One thread per tracer in id order.
// The interpolant and the position updates are written in the reference's
// operation order and compiled without FMA contraction, so positions and
// therefore cell indices equal the CPU restatement bit for bit.
#include "tc_device.cuh"

// Cell indices of a tracer: int(x/h) and nint(x/h) of the correctly rounded
// quotient, as composition.f90 takes them, without the FP64 division (on this
// GPU the FP64 pipe, not memory, bounds the tracer kernels).  The 64 high bits
// of the product of the significands of x and hinv = RN(1/h) give x*hinv in
// fixed point with 64 fraction bits; for 0 < x/h < 2^21 this value, x/h and
// RN(x/h) lie within 2^-30 of one another (hinv contributes 2^-53 relative, the
// truncated product 2^-43 absolute, RN(x/h) 2^-53 relative).  When the fraction
// is farther than 2^-24 from the boundary in question (an integer for int(),
// a half-integer for nint()), RN(x/h) lies on the same side of it as the
// fixed-point value and the index is read off the bits; otherwise, and for x
// outside that range, the division is done.  Either way the result equals
// that of the division.
struct QuotFix {
    unsigned long long ip, fr;  // integer part, fraction * 2^64
    bool ok;
};
__device__ __forceinline__ QuotFix quot_fix(double x, double hinv) {
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
    const unsigned long long bh = (unsigned long long)__double_as_longlong(hinv);
    const int ex = (int)(bx >> 52), eh = (int)(bh >> 52) & 0x7ff;   // ex includes the sign bit
    const unsigned long long mx = ((bx & 0xfffffffffffffull) | (1ull << 52)) << 11;
    const unsigned long long mh = ((bh & 0xfffffffffffffull) | (1ull << 52)) << 11;
    const unsigned long long p = __umul64hi(mx, mh);    // in [2^62, 2^64)
    const int sh = 2108 - ex - eh;                      // x*hinv = p / 2^sh
    QuotFix q;
    q.ok = ex > 0 && ex < 0x7ff && sh >= 43 && sh < 128;
    if (sh >= 43 && sh < 64) {
        q.ip = p >> sh;
        q.fr = p << (64 - sh);
    } else {
        q.ip = 0;
        q.fr = (sh >= 64 && sh < 128) ? (sh == 64 ? p : p >> (sh - 64)) : 0;
    }
    return q;
}
constexpr unsigned long long kQuotGuard = 1ull << 40;  // 2^-24 in fraction units
__device__ __forceinline__ int quot_trunc(double x, double h, double hinv) {
    const QuotFix q = quot_fix(x, hinv);
    if (q.ok && q.fr > kQuotGuard && q.fr < 0ull - kQuotGuard) return (int)q.ip;
    return (int)(x / h);
}
__device__ __forceinline__ int quot_nint(double x, double h, double hinv) {
    const QuotFix q = quot_fix(x, hinv);
    const unsigned long long half = 1ull << 63;
    if (q.ok && (q.fr > half + kQuotGuard || q.fr < half - kQuotGuard)) return (int)q.ip + (q.fr > half ? 1 : 0);
    return (int)round(x / h);
}

// interpolate (composition.f90:838-898) with order=2: one r-derivative table
// DER(1,i,k) and a 3-point s-stencil; int() truncates, as in Fortran.  The
// position part (cell, offsets, branch) is shared by every field
// interpolated at the same point.
struct TaylorPos {
    int i, k;      // column of the r-Taylor step (i or i+1) and the s cell
    double a1;     // r offset from that column
    double hs;     // s offset (from k, or ds minus it on the upper branch)
    bool slo;      // hs <= ds/2
};
__device__ __forceinline__ TaylorPos taylor_pos(const Phys& P, double r, double s) {
    TaylorPos t;
    const int i = quot_trunc(r, P.dr, P.rdr);
    t.k = quot_trunc(s, P.ds, P.rds);
    double hr = r - (double)i * P.dr;
    if (hr <= P.dro2) {
        t.i = i;
        t.a1 = hr / 1.0;
    } else {
        hr = P.dr - hr;
        t.i = i + 1;
        t.a1 = (-hr) / 1.0;
    }
    const double hs = s - (double)t.k * P.ds;
    t.slo = hs <= P.dso2;
    t.hs = t.slo ? hs : P.ds - hs;
    return t;
}
__device__ __forceinline__ double taylor_eval(const Lay& L, const Phys& P, const double* __restrict__ f,
                                              const double* __restrict__ der, const TaylorPos& t) {
    const int i = t.i, k = t.k;
    const double fR0 = __ldg(f + IX(L, i, k - 1)) + __ldg(der + IX(L, i, k - 1)) * t.a1;
    const double fR1 = __ldg(f + IX(L, i, k)) + __ldg(der + IX(L, i, k)) * t.a1;
    const double fR2 = __ldg(f + IX(L, i, k + 1)) + __ldg(der + IX(L, i, k + 1)) * t.a1;
    const double fR3 = __ldg(f + IX(L, i, k + 2)) + __ldg(der + IX(L, i, k + 2)) * t.a1;
    double fin;
    if (t.slo) {
        double DERs = (-0.5 * fR0 + 0.5 * fR2) / P.ds;
        fin = fR1 + DERs * (t.hs / 1.0);
    } else {
        double DERs = (-0.5 * fR1 + 0.5 * fR3) / P.ds;
        fin = fR2 + DERs * ((-t.hs) / 1.0);
    }
    return fin;
}
__device__ __forceinline__ double interp_taylor(const Lay& L, const Phys& P, const double* __restrict__ f,
                                                const double* __restrict__ der, double r, double s) {
    return taylor_eval(L, P, f, der, taylor_pos(P, r, s));
}

// Temperature tracers (tracer = 1): the tracer_space value at the stage
// position, interpolated like u and w, drives Ttr the way u drives rtr.
struct TracerT {
    const double* f;    // tracer_space_array (nullptr: no temperature tracers)
    const double* der;  // its r-derivative table
    const double* T0;   // Ttr0
    double* acc;        // Ttr
    double* out;        // Ttr1 / Ttr2 of the stage
};

// stage 1: (rin,sin)=(rtr0,str0) -> acc=k1, out=rtr1
// stage 2: (rin,sin)=(rtr1,str1) -> RK2: acc=final rtr;  RK4: acc+=2k2, out=rtr2
// stage 3: (rin,sin)=(rtr2,str2) -> acc+=2k3, out=rtr1
// stage 4: (rin,sin)=(rtr1,str1) -> acc=final rtr
__global__ void k_tracer_stage(Lay L, Phys P, int torder, int stage, int64_t ntr, const double* __restrict__ rin,
                               const double* __restrict__ sin, const double* __restrict__ r0,
                               const double* __restrict__ s0, double* __restrict__ racc, double* __restrict__ sacc,
                               double* __restrict__ rout, double* __restrict__ sout, const double* __restrict__ u,
                               const double* __restrict__ w, const double* __restrict__ du,
                               const double* __restrict__ dw, const DevScalars* __restrict__ ds, TracerT tT) {
    int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntr) return;
    const double dt = ds->dt;
    const double r = rin[id], s = sin[id];
    // positions outside the box were already reported by the histogram that
    // precedes every stage (the reference stops there); never index with them
    if (!(r > 0.0 && r < P.aspect && s > 0.0 && s < 1.0)) return;
    const TaylorPos tp = taylor_pos(P, r, s);
    double tr = taylor_eval(L, P, u, du, tp);
    double ts = taylor_eval(L, P, w, dw, tp);
    // stretched grids: the computational velocity, divided by the metric
    // interpolated the same way (interpolate_xr / interpolate_zs,
    // composition.f90:938-998; energy.f90:195-203)
    if (P.M.gx) tr = tr / (mt(P.M.xr, tp.i) + mt(P.M.dxr, tp.i) * tp.a1);
    if (P.M.gz)
        ts = ts / (tp.slo ? mt(P.M.zs, tp.k) + mt(P.M.dzs, tp.k) * (tp.hs / 1.0)
                          : mt(P.M.zs, tp.k + 1) + mt(P.M.dzs, tp.k + 1) * ((-tp.hs) / 1.0));
    if (tT.f) {
        // energy.f90:213-223, 292-310, 371-375, 437-440
        const double te = taylor_eval(L, P, tT.f, tT.der, tp);
        if (stage == 1) {
            tT.acc[id] = te;
            tT.out[id] = tT.T0[id] + ((torder == 2) ? dt : 0.5 * dt) * te;
        } else if (stage == 2) {
            if (torder == 2) {
                const double a = tT.acc[id] + te;
                tT.acc[id] = tT.T0[id] + (0.5 * dt) * a;
            } else {
                tT.acc[id] = tT.acc[id] + 2.0 * te;
                tT.out[id] = tT.T0[id] + (0.5 * dt) * te;
            }
        } else if (stage == 3) {
            tT.acc[id] = tT.acc[id] + 2.0 * te;
            tT.out[id] = tT.T0[id] + dt * te;
        } else {
            tT.acc[id] = tT.T0[id] + (dt / 6.0) * (tT.acc[id] + te);
        }
    }
    if (stage == 1) {
        const double dtstage = (torder == 2) ? dt : 0.5 * dt;
        racc[id] = tr;
        sacc[id] = ts;
        rout[id] = r + dtstage * tr;
        sout[id] = s + dtstage * ts;
    } else if (stage == 2) {
        const double dtstage = 0.5 * dt;
        if (torder == 2) {
            double a = racc[id] + tr, b = sacc[id] + ts;
            racc[id] = r0[id] + dtstage * a;
            sacc[id] = s0[id] + dtstage * b;
        } else {
            racc[id] = racc[id] + 2.0 * tr;
            sacc[id] = sacc[id] + 2.0 * ts;
            rout[id] = r0[id] + dtstage * tr;
            sout[id] = s0[id] + dtstage * ts;
        }
    } else if (stage == 3) {
        racc[id] = racc[id] + 2.0 * tr;
        rout[id] = r0[id] + dt * tr;
        sacc[id] = sacc[id] + 2.0 * ts;
        sout[id] = s0[id] + dt * ts;
    } else {
        const double dto6 = dt / 6.0;
        racc[id] = r0[id] + dto6 * (racc[id] + tr);
        sacc[id] = s0[id] + dto6 * (sacc[id] + ts);
    }
}
void launch_tracer_stage(cudaStream_t s, const Lay& L, const Phys& P, int torder, int stage, int64_t ntr,
                         const double* rin, const double* sin, const double* r0, const double* s0, double* racc,
                         double* sacc, double* rout, double* sout, const double* u, const double* w,
                         const double* du, const double* dw, const DevScalars* ds, const double* tsa,
                         const double* dT, const double* Ttr0, double* Ttr, double* Tout) {
    if (ntr <= 0) return;
    unsigned nb = (unsigned)((ntr + 255) / 256);
    const TracerT tT{tsa, dT, Ttr0, Ttr, Tout};
    k_tracer_stage<<<nb, 256, 0, s>>>(L, P, torder, stage, ntr, rin, sin, r0, s0, racc, sacc, rout, sout, u, w, du,
                                      dw, ds, tT); tc_note_launch();
}

// ---- exact per-volume sums of the tracer temperatures ------------------------
// Each Ttr enters as round-toward-zero(Ttr * 2^64), a 128-bit integer built
// from the IEEE-754 fields (|Ttr| >= 2^62 saturates, NaN and magnitudes
// below 2^-64 count as 0); a volume's sum is a 128-bit integer kept as two
// 64-bit words (the low word's atomic add reports its carry into the high
// word), so it does not depend on the order the tracers arrive in; it is
// rounded to double once.  The CPU restatement computes the same integers.
__device__ __forceinline__ __int128 tracer_fixq(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0x7ff && (b & 0xfffffffffffffULL)) return 0;
    const bool neg = (b >> 63) != 0;
    unsigned __int128 v;
    if (E == 0) {
        v = 0;
    } else {
        const unsigned long long m = (b & 0xfffffffffffffULL) | (1ULL << 52);  // |x| = m * 2^(E-1075)
        const int sh = E - 1011;                                               // |x| * 2^64 = m * 2^sh
        if (sh > 73 || E == 0x7ff) v = (unsigned __int128)1 << 126;
        else if (sh >= 0) v = (unsigned __int128)m << sh;
        else if (sh > -53) v = (unsigned __int128)(m >> (-sh));
        else v = 0;
    }
    return neg ? -(__int128)v : (__int128)v;
}
__device__ __forceinline__ void tracer_add128(unsigned long long* lo, unsigned long long* hi, __int128 q) {
    const unsigned __int128 u = (unsigned __int128)q;
    const unsigned long long ql = (unsigned long long)u, qh = (unsigned long long)(u >> 64);
    const unsigned long long old = atomicAdd(lo, ql);
    const unsigned long long c = qh + ((old + ql < old) ? 1ULL : 0ULL);
    if (c) atomicAdd(hi, c);
}
// the 128-bit sum * 2^-64 rounded to nearest (ties to even)
__device__ __forceinline__ double tracer_fixd(unsigned long long lo, unsigned long long hi) {
    const __int128 S = (__int128)(((unsigned __int128)hi << 64) | (unsigned __int128)lo);
    if (S == 0) return 0.0;
    const bool neg = S < 0;
    unsigned __int128 m = neg ? (unsigned __int128)0 - (unsigned __int128)S : (unsigned __int128)S;
    const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
    const int nb = mh ? 128 - __clzll((long long)mh) : 64 - __clzll((long long)ml);
    int e = 0;
    if (nb > 53) {
        const int drop = nb - 53;
        const unsigned __int128 rem = m & (((unsigned __int128)1 << drop) - 1);
        const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
        m >>= drop;
        e = drop;
        if (rem > half || (rem == half && (m & 1))) {
            m += 1;
            if (m >> 53) { m >>= 1; e += 1; }
        }
    }
    const double d = ldexp((double)(unsigned long long)m, e - 64);
    return neg ? -d : d;
}

// histogram of tracers_to_corners (composition.f90:695-726): nint() rounds
// half away from zero (CUDA round()).  Tracers of a warp that land in the
// same counter are combined before one atomic (they are mostly cell-sorted).
__global__ void k_histogram(Lay L, Phys P, int64_t ntr, const double* __restrict__ rr, const double* __restrict__ ss,
                            const int* __restrict__ ttype, int* __restrict__ counts, int* __restrict__ flag,
                            const double* __restrict__ Tt, unsigned long long* tlo, unsigned long long* thi) {
    int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    if (id < ntr) {
        const double r = rr[id], s = ss[id];
        if (r <= 0.0 || r >= P.aspect || s <= 0.0 || s >= 1.0) {
            atomicOr(flag, 1);
        } else {
            const int i = quot_nint(r, P.dr, P.rdr);
            const int k = quot_nint(s, P.ds, P.rds);
            const int t = ttype[id];
            if (t < 0 || t > P.ntype || i < 0 || i > P.nx || k < 0 || k > P.nz) atomicOr(flag, 2);
            else {
                key = (int)((size_t)t * L.plane + IX(L, i, k));
                if (Tt) tracer_add128(tlo + IX(L, i, k), thi + IX(L, i, k), tracer_fixq(Tt[id]));
            }
        }
    }
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(counts + key, __popc(peers));
}
void launch_histogram(cudaStream_t s, const Lay& L, const Phys& P, int64_t ntr, const double* r, const double* sv,
                      const int* ttype, int* counts, DevScalars* ds, const double* Tt, unsigned long long* tsum) {
    cudaMemsetAsync(counts, 0, sizeof(int) * L.plane * (size_t)(P.ntype + 1), s);
    if (Tt) cudaMemsetAsync(tsum, 0, sizeof(unsigned long long) * 2 * L.plane, s);
    if (ntr <= 0) return;
    unsigned nb = (unsigned)((ntr + 255) / 256);
    k_histogram<<<nb, 256, 0, s>>>(L, P, ntr, r, sv, ttype, counts, &ds->flag_outside, Tt, Tt ? tsum : nullptr,
                                   Tt ? tsum + L.plane : nullptr); tc_note_launch();
}

// ghost mirror of count_type, nempty and the tracer ratio (composition.f90:745-776)
__global__ void k_counts_to_comp(Lay L, Phys P, Range2 r, int* __restrict__ counts, int* __restrict__ nempty,
                                 CPtrsW Cn, const unsigned long long* __restrict__ tsum, double* __restrict__ Tratio) {
    RANGE_IK(r);
    if (!inr) return;
    const int nx = L.a, nz = L.b;
    const bool inx = (i >= 0 && i <= nx), inz = (k >= 0 && k <= nz);
    int si = i, sk = k;
    bool zero = false;
    if (!inx && inz) si = (i < 0) ? -i : 2 * nx - i;
    else if (inx && !inz) sk = (k < 0) ? -k : 2 * nz - k;
    else if (!inx && !inz) zero = true;  // corners stay 0
    const size_t x = IX(L, i, k), sx = IX(L, si, sk);
    int ne = 0;
    for (int t = 0; t <= P.ntype; t++) {
        int c = zero ? 0 : counts[(size_t)t * L.plane + sx];
        if (!inx || !inz) counts[(size_t)t * L.plane + x] = c;
        ne += c;
    }
    nempty[x] = ne;
    if (Tratio && inx && inz && ne > 0) Tratio[x] = tracer_fixd(tsum[x], tsum[L.plane + x]) / (double)ne;
    if (inx && inz && ne > 0)
        for (int t = 1; t <= P.ntype; t++) {
            int ct = counts[(size_t)t * L.plane + x];
            double v;
            if (ct == ne) v = 1.0;
            else if (ct == 0) v = 0.0;
            else v = (double)ct / (double)ne;
            Cn.p[t - 1][x] = v;
        }
}
void launch_counts_to_comp(cudaStream_t s, const Lay& L, const Phys& P, int* counts, int* nempty,
                           double* const* Cnew, const unsigned long long* tsum, double* Tratio) {
    CPtrsW C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cnew[j];
    Range2 r{-SP, L.a + SP, -SP, L.b + SP};
    k_counts_to_comp<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, counts, nempty, C, tsum, Tratio); tc_note_launch();
}

// extendT + tracer_space (energy.f90:478-499, 82-115) on (-1:nx+1, -1:nz+1):
// energy_space without advection, on Tratio extended by extendT's mirrors
// (antisymmetric about T=1 at the bottom for Tbot=0, symmetric for Tbot=1,
// antisymmetric about 0 at the top; rows 0 and nz set to 1 and 0 last)
__device__ __forceinline__ double textend(const Lay& L, const Phys& P, const double* __restrict__ Tr, int i, int k) {
    const int nx = L.a, nz = L.b;
    const int ii = (i < 0) ? -i : ((i > nx) ? 2 * nx - i : i);
    if (k == nz) return 0.0;
    if (k == 0 && P.Tbot == 0) return 1.0;
    if (k >= 0 && k < nz) return Tr[IX(L, ii, k)];
    if (k < 0) {
        const double v = Tr[IX(L, ii, -k)];
        return (P.Tbot == 0) ? -(v - 1.0) + 1.0 : v;
    }
    return -Tr[IX(L, ii, 2 * nz - k)];
}
__global__ void k_tracer_space(Lay L, Phys P, Range2 r, const double* __restrict__ Tr, const double* __restrict__ cd,
                               const double* __restrict__ cr, const double* __restrict__ cs, CPtrs Cv,
                               double* __restrict__ out) {
    RANGE_IK(r);
    if (!inr) return;
    const size_t x = IX(L, i, k);
    const double c = textend(L, P, Tr, i, k);
    const double fm = textend(L, P, Tr, i - 1, k), fp = textend(L, P, Tr, i + 1, k);
    const double gm = textend(L, P, Tr, i, k - 1), gp = textend(L, P, Tr, i, k + 1);
    const double Trd = (-0.5 * fm + 0.5 * fp) / P.dr;
    const double Tsd = (-0.5 * gm + 0.5 * gp) / P.ds;
    const double Trr = (fm + -2.0 * c + fp) / P.dr2;
    const double Tss = (gm + -2.0 * c + gp) / P.ds2;
    double heat;
    if (P.comp == 0) heat = P.H;
    else {
        double sC = 0.0;
        for (int j = 0; j < P.ntype; j++) sC = sC + Cv.p[j][x];
        heat = P.H * (1.0 - sC);
        for (int j = 0; j < P.ntype; j++) heat = P.Htype[j] * Cv.p[j][x] + heat;
    }
    if (P.M.on) {
        // tracer_space on a stretched grid (energy.f90:82-100)
        const double x1 = mt(P.M.xr, i), z1 = mt(P.M.zs, k);
        const double kx = cr[x] / x1, kz = cs[x] / z1;
        const double Tx = Trd / x1, Tz = Tsd / z1;
        const double Txx = (Trr - Tx * mt(P.M.xrr, i)) / (x1 * x1);
        const double Tzz = (Tss - Tz * mt(P.M.zss, k)) / (z1 * z1);
        out[x] = cd[x] * (Txx + Tzz) + (kx * Tx + kz * Tz) + heat;
        return;
    }
    out[x] = cd[x] * (Trr + Tss) + (cr[x] * Trd + cs[x] * Tsd) + heat;
}
void launch_tracer_space(cudaStream_t s, const Lay& L, const Phys& P, const double* Tratio, const double* conduct,
                         const double* conduct_r, const double* conduct_s, const double* const* Cvis, double* tsa) {
    CPtrs C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cvis[j];
    Range2 r{-1, L.a + 1, -1, L.b + 1};
    k_tracer_space<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, Tratio, conduct, conduct_r, conduct_s, C, tsa); tc_note_launch();
}

// ---- cell sort of the tracer arrays -------------------------------------------
// The tracers are kept in the order of the corner control volume that
// tracers_to_corners counts them in, so the warps of k_tracer_stage gather
// from neighbouring grid rows and those of k_histogram meet few distinct
// counters.  A counting sort: per-cell counts, an exclusive scan, and a
// scatter that takes each tracer's slot with an atomic on its cell's offset
// (the order inside a cell is left free: nothing the step computes depends on
// it, every tracer is advanced on its own and the counts are integers).
// perm[j] is the reference's index of the tracer stored at slot j.
namespace {
__device__ __forceinline__ int tracer_cell(const Lay& L, const Phys& P, double r, double s) {
    int i = quot_nint(r, P.dr, P.rdr), k = quot_nint(s, P.ds, P.rds);
    i = min(max(i, 0), P.nx);
    k = min(max(k, 0), P.nz);
    return (int)IX(L, i, k);
}

__global__ void k_sort_count(Lay L, Phys P, int64_t ntr, const double* rr, const double* ss, int* cnt) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int key = (id < ntr) ? tracer_cell(L, P, ld_state(rr + id), ld_state(ss + id)) : -1;
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    if (key >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(cnt + key, __popc(peers));
}

// exclusive scan of one 1024-element block in shared memory; returns the block total
__device__ int block_exclusive_scan(int v, int* warp_tot, int* out_excl) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
        int ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int n = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += n;
        }
        warp_tot[lane] = ti - t;  // exclusive prefix of the warps
        if (lane == 31) warp_tot[32] = ti;
    }
    __syncthreads();
    *out_excl = warp_tot[wid] + incl - v;
    const int tot = warp_tot[32];
    __syncthreads();
    return tot;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(const int* cnt, int n, int* bsum) {
    __shared__ int wt[33];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    int ex;
    const int tot = block_exclusive_scan(i < n ? cnt[i] : 0, wt, &ex);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}
// one block: exclusive scan of the block totals, 1024 at a time with a carry
__global__ void __launch_bounds__(1024) k_scan_bsums(int* bsum, int nb) {
    __shared__ int wt[33];
    int carry = 0;
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = (i < nb) ? bsum[i] : 0;
        int ex;
        const int tot = block_exclusive_scan(v, wt, &ex);
        if (i < nb) bsum[i] = carry + ex;
        carry += tot;
    }
}
__global__ void __launch_bounds__(1024) k_scan_final(const int* cnt, int n, const int* bsum, int* off) {
    __shared__ int wt[33];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    int ex;
    block_exclusive_scan(i < n ? cnt[i] : 0, wt, &ex);
    if (i < n) off[i] = bsum[blockIdx.x] + ex;
}

__global__ void k_sort_scatter(Lay L, Phys P, int64_t ntr, const double* rr, const double* ss, const int* tt,
                               const int* perm, int* off, double* r2, double* s2, int* t2, int* p2,
                               const double* Tt, double* T2) {
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntr) return;
    const double r = ld_state(rr + id), s = ld_state(ss + id);
    const int pos = atomicAdd(off + tracer_cell(L, P, r, s), 1);
    r2[pos] = r;
    s2[pos] = s;
    t2[pos] = ld_state(tt + id);
    p2[pos] = ld_state(perm + id);
    if (Tt) T2[pos] = ld_state(Tt + id);
}

template <typename T>
__global__ void k_perm_scatter(int64_t n, const int* perm, const T* in, T* out) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[ld_state(perm + j)] = ld_state(in + j);
}
template <typename T>
__global__ void k_perm_gather(int64_t n, const int* perm, const T* in, T* out) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = ld_state(in + ld_state(perm + j));
}
__global__ void k_iota(int64_t n, int* p) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) p[j] = (int)j;
}
}  // namespace

// cnt, off: L.plane ints each; bsum: (L.plane + 1023) / 1024 ints
void launch_sort_tracers(cudaStream_t s, const Lay& L, const Phys& P, int64_t ntr, const double* rr, const double* ss,
                         const int* tt, const int* perm, int* cnt, int* off, int* bsum, double* r2, double* s2,
                         int* t2, int* p2, const double* Tt, double* T2) {
    if (ntr <= 0) return;
    const int n = (int)L.plane, nb = (n + 1023) / 1024;
    const unsigned tb = (unsigned)((ntr + 255) / 256);
    cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)n, s);
    k_sort_count<<<tb, 256, 0, s>>>(L, P, ntr, rr, ss, cnt); tc_note_launch();
    k_scan_blocks<<<nb, 1024, 0, s>>>(cnt, n, bsum); tc_note_launch();
    k_scan_bsums<<<1, 1024, 0, s>>>(bsum, nb); tc_note_launch();
    k_scan_final<<<nb, 1024, 0, s>>>(cnt, n, bsum, off); tc_note_launch();
    k_sort_scatter<<<tb, 256, 0, s>>>(L, P, ntr, rr, ss, tt, perm, off, r2, s2, t2, p2, Tt, T2); tc_note_launch();
}
void launch_perm_scatter(cudaStream_t s, int64_t n, const int* perm, const double* in, double* out) {
    if (n <= 0) return;
    k_perm_scatter<double><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, perm, in, out); tc_note_launch();
}
void launch_perm_scatter(cudaStream_t s, int64_t n, const int* perm, const int* in, int* out) {
    if (n <= 0) return;
    k_perm_scatter<int><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, perm, in, out); tc_note_launch();
}
void launch_perm_gather(cudaStream_t s, int64_t n, const int* perm, const double* in, double* out) {
    if (n <= 0) return;
    k_perm_gather<double><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, perm, in, out); tc_note_launch();
}
void launch_iota(cudaStream_t s, int64_t n, int* p) {
    if (n <= 0) return;
    k_iota<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, p); tc_note_launch();
}

// ---- tracer repositioning, TRA (composition.f90:7-580) ----------------------
// The reference runs equalize_tracers with OpenMP threads, each drawing from
// its own mzran stream over a static-schedule share of each loop; its result
// depends on the thread count.  Here each of its NR threads is one GPU
// thread: the per-volume shuffles run as NR threads over their shares, and
// the donor search, the lottery passes and the serial remainder run in one
// block whose first NR threads are the ranks (all threads take part in the
// reductions between passes).  Every loop is bounded.
namespace {

__device__ __forceinline__ double eq_mzran(int* sd, int rank, int NR) {
    int* si = sd;
    int* sj = sd + NR;
    int* sk = sd + 2 * NR;
    int* sn = sd + 3 * NR;
    int r = si[rank] - sk[rank];
    if (r < 0) r += 2147483579;
    si[rank] = sj[rank];
    sj[rank] = sk[rank];
    sk[rank] = r;
    sn[rank] = (int)(69069u * (unsigned)sn[rank] + 1013904243u);
    r = (int)((unsigned)r + (unsigned)sn[rank]);
    return 0.5 + (0.2328306e-9) * (double)r;
}
// shuffle_serial on a(istart:N), `a` indexed absolutely
__device__ void eq_shuffle(int* a, int istart, int N, int* sd, int rank, int NR) {
    for (int i = istart; i <= N - 1; i++) {
        const double ran = eq_mzran(sd, rank, NR);
        const int r = (int)floor(ran * (double)(N - i)) + i + 1;
        const int t = a[i];
        a[i] = a[r];
        a[r] = t;
    }
}
// iterations [lo, lo+cnt) of thread t in a static OpenMP loop of N iterations
__device__ __forceinline__ void eq_static(int N, int NR, int t, int& lo, int& cnt) {
    const int q = N / NR, r = N % NR;
    if (t < r) { cnt = q + 1; lo = t * cnt; } else { cnt = q; lo = t * q + r; }
}

struct EqDev {
    Lay L;
    int nx, nz, ntype, NT, NR, comp, tracer, tpc;
    int64_t ntr;
    double dr, ds, aspect, dist_r, dist_s;
    int* counts;       // count_type (L1 planes per type)
    const int* nempty; // L1
    CPtrs C;           // Cnew per type (L1)
    double* rtr;       // slot order
    double* str;
    int* ttype;
    const int* perm;   // slot -> reference index
    int* iperm;        // reference index -> slot
    int* nex;          // (nx+1)*(nz+1), i-major
    int* off;          // (nx+1)*(nz+1)+1
    int* cur;          // per-volume cursors
    int* ids;          // per-volume lists of reference ids (1-based)
    int* sd;           // mzran state [4][NR]
    int* donor;        // [NR][NT][cap]
    int64_t cap;
    int* isv;          // index_save [NR][NT]
    int* isv2;
    int* nfr;          // nfree_rank [NR][NT]
    int* nx_loop;
    int* nz_loop;
    long long* sc;     // scalars, see EQ_*
};
enum { EQ_NFREE = 0, EQ_NONZERO, EQ_DEFICIT, EQ_MOVED, EQ_ERR, EQ_PASSES, EQ_TPC0, EQ_MIN0 = EQ_TPC0 + 8,
       EQ_COUNT0 = EQ_MIN0 + 8, EQ_NIDEAL0 = EQ_COUNT0 + 8, EQ_TSUM0 = EQ_NIDEAL0 + 8, EQ_TCNT0 = EQ_TSUM0 + 8,
       EQ_NSC = EQ_TCNT0 + 8 };

__device__ __forceinline__ size_t eq_cell(const EqDev& E, int i, int k) { return (size_t)i * (E.nz + 1) + k; }
__device__ __forceinline__ int eq_count(const EqDev& E, int t, int i, int k) {
    return E.counts[(size_t)t * E.L.plane + IX(E.L, i, k)];
}
__device__ __forceinline__ bool eq_type_mask(const EqDev& E, int t, int i, int k) {
    const size_t x = IX(E.L, i, k);
    if (t == 0) {
        double sC = 0.0;
        for (int j = 0; j < E.ntype; j++) sC = sC + E.C.p[j][x];
        return sC == 0.0;
    }
    return E.C.p[t - 1][x] == 1.0;
}

// tpc_type sums over the pure volumes (comp = 1): per type, count and count_type sum
__global__ void k_eq_tpc(EqDev E) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncell = (E.nx + 1) * (E.nz + 1);
    if (c >= ncell) return;
    const int i = c / (E.nz + 1), k = c % (E.nz + 1);
    for (int t = 0; t < E.NT; t++)
        if (eq_type_mask(E, t, i, k)) {
            atomicAdd((unsigned long long*)&E.sc[EQ_TCNT0 + t], 1ULL);
            atomicAdd((unsigned long long*)&E.sc[EQ_TSUM0 + t], (unsigned long long)eq_count(E, t, i, k));
        }
}
// nexcess (composition.f90:114-160), nfree and whether any volume is off its target
__global__ void k_eq_nexcess(EqDev E) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncell = (E.nx + 1) * (E.nz + 1);
    if (c >= ncell) return;
    const int i = c / (E.nz + 1), k = c % (E.nz + 1);
    const int ne = E.nempty[IX(E.L, i, k)];
    int v = 0;
    if (E.comp == 0) {
        v = (ne > 0) ? ne - E.tpc : 0;
    } else {
        for (int t = 0; t < E.NT; t++) {
            bool all = true;
            for (int a = -1; a <= 1 && all; a++)
                for (int b = -1; b <= 1 && all; b++)
                    if (eq_count(E, t, i + a, k + b) != E.nempty[IX(E.L, i + a, k + b)]) all = false;
            if (all && ne > 0) {
                const long long n = E.sc[EQ_TCNT0 + t];
                const int tp = (n > 0) ? (int)llround((double)E.sc[EQ_TSUM0 + t] / (double)n) : 0;
                v = ne - tp;
                break;
            }
        }
    }
    E.nex[c] = v;
    if (v > 0) atomicAdd((unsigned long long*)&E.sc[EQ_NFREE], (unsigned long long)v);
    if (v != 0) atomicOr((unsigned long long*)&E.sc[EQ_NONZERO], 1ULL);
}
// per-volume lists of reference ids: scatter, then ascending order in each list
__global__ void k_eq_offsets_in(EqDev E, int* cnt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncell = (E.nx + 1) * (E.nz + 1);
    if (c >= ncell) return;
    cnt[c] = E.nempty[IX(E.L, c / (E.nz + 1), c % (E.nz + 1))];
    E.cur[c] = 0;
}
__global__ void k_eq_scatter(EqDev E) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= E.ntr) return;
    const int id = E.perm[j];
    E.iperm[id] = (int)j;
    const int i = (int)round(E.rtr[j] / E.dr), k = (int)round(E.str[j] / E.ds);
    const size_t c = eq_cell(E, i, k);
    const int pos = atomicAdd(E.cur + c, 1);
    E.ids[E.off[c] + pos] = id + 1;
}
__global__ void k_eq_sort_lists(EqDev E) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncell = (E.nx + 1) * (E.nz + 1);
    if (c >= ncell) return;
    int* a = E.ids + E.off[c];
    const int n = E.off[c + 1] - E.off[c];
    for (int p = 1; p < n; p++) {
        const int v = a[p];
        int q = p - 1;
        while (q >= 0 && a[q] > v) { a[q + 1] = a[q]; q--; }
        a[q + 1] = v;
    }
}
// mzran with the stream state held in registers (same draws as eq_mzran)
struct EqMz {
    int i, j, k, n;
};
__device__ __forceinline__ double eq_mz_next(EqMz& m) {
    int r = m.i - m.k;
    if (r < 0) r += 2147483579;
    m.i = m.j;
    m.j = m.k;
    m.k = r;
    m.n = (int)(69069u * (unsigned)m.n + 1013904243u);
    r = (int)((unsigned)r + (unsigned)m.n);
    return 0.5 + (0.2328306e-9) * (double)r;
}
// composition.f90:188-199: each rank shuffles the lists of its share of
// columns; a list of up to 64 ids is shuffled in a thread-local copy
__global__ void k_eq_shuffle_lists(EqDev E) {
    const int rank = blockIdx.x * blockDim.x + threadIdx.x;
    if (rank >= E.NR) return;
    const int NR = E.NR;
    EqMz m{E.sd[rank], E.sd[NR + rank], E.sd[2 * NR + rank], E.sd[3 * NR + rank]};
    int loc[65];
    int lo, cnt;
    eq_static(E.nx + 1, NR, rank, lo, cnt);
    for (int i = lo; i < lo + cnt; i++)
        for (int k = 0; k <= E.nz; k++) {
            const size_t c = eq_cell(E, i, k);
            int* a = E.ids + E.off[c] - 1;  // a[1..N]
            const int N = E.off[c + 1] - E.off[c];
            const bool small = N <= 64;
            if (small)
                for (int q = 1; q <= N; q++) loc[q] = a[q];
            int* b = small ? loc : a;
            for (int q = 1; q <= N - 1; q++) {
                const double ran = eq_mz_next(m);
                const int r = (int)floor(ran * (double)(N - q)) + q + 1;
                const int t = b[q];
                b[q] = b[r];
                b[r] = t;
            }
            if (small)
                for (int q = 1; q <= N; q++) a[q] = loc[q];
        }
    E.sd[rank] = m.i;
    E.sd[NR + rank] = m.j;
    E.sd[2 * NR + rank] = m.k;
    E.sd[3 * NR + rank] = m.n;
}

__device__ __forceinline__ int* eq_D(const EqDev& E, int rank, int t) {
    return E.donor + ((size_t)rank * E.NT + t) * (size_t)E.cap;
}
// donors of one volume: the first nexcess ids of its list (near_wall: only
// those within dist of a wall, or only those away from every wall)
__device__ void eq_take(const EqDev& E, int i, int k, int rank, int mode) {
    const size_t c = eq_cell(E, i, k);
    if (E.nex[c] <= 0) return;
    const int* a = E.ids + E.off[c] - 1;
    const int n = E.off[c + 1] - E.off[c];
    for (int q = 1; q <= n; q++) {
        const int ID = a[q];
        const int slot = E.iperm[ID - 1];
        const double r = E.rtr[slot], s = E.str[slot];
        const bool nw = (s < E.dist_s) || (s > 1.0 - E.dist_s) || (r < E.dist_r) || (r > E.aspect - E.dist_r);
        if (mode == 1 && !nw) continue;
        if (mode == 2 && nw) continue;
        const int t = E.ttype[slot];
        int& is = E.isv[rank * E.NT + t];
        is = is + 1;
        eq_D(E, rank, t)[is] = ID;
        E.nex[c] = E.nex[c] - 1;
        if (E.nex[c] == 0) break;
    }
}
// composition.f90:226-334: the left and right columns split over k, then the
// bottom and top rows (corners excluded) split over i; every thread of the
// block calls it (threads >= NR only meet the barriers)
__device__ void eq_edges(const EqDev& E, int rank, int mode) {
    const bool isrank = rank < E.NR;
    for (int i = 0; i <= E.nx; i += E.nx) {
        int lo = 0, cnt = 0;
        if (isrank) eq_static(E.nz + 1, E.NR, rank, lo, cnt);
        for (int k = lo; k < lo + cnt; k++) eq_take(E, i, k, rank, mode);
        __syncthreads();
    }
    for (int k = 0; k <= E.nz; k += E.nz) {
        int lo = 0, cnt = 0;
        if (isrank) eq_static(E.nx - 1, E.NR, rank, lo, cnt);
        for (int i = 1 + lo; i < 1 + lo + cnt; i++) eq_take(E, i, k, rank, mode);
        __syncthreads();
    }
}
__device__ int eq_maxloc(const EqDev& E, int i, int k) {
    int best = 0;
    for (int t = 1; t < E.NT; t++)
        if (eq_count(E, t, i, k) > eq_count(E, best, i, k)) best = t;
    return best;
}
// block-wide minval of nexcess <= 0 over the volumes of type mask t
// (use_type false: all volumes); HUGE when none
__device__ int eq_minval(const EqDev& E, int t, bool use_type, int* red) {
    const int ncell = (E.nx + 1) * (E.nz + 1);
    int m = 2147483647;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
        const int v = E.nex[c];
        if (v > 0) continue;
        if (use_type && !eq_type_mask(E, t, c / (E.nz + 1), c % (E.nz + 1))) continue;
        m = min(m, v);
    }
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int r = 2147483647;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = min(r, red[w]);
        red[32] = r;
    }
    __syncthreads();
    const int r = red[32];
    __syncthreads();
    return r;
}
__device__ long long eq_blocksum(long long v, long long* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long r = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += red[w];
        red[32] = r;
    }
    __syncthreads();
    const long long r = red[32];
    __syncthreads();
    return r;
}
__device__ void eq_tracer_counts(const EqDev& E, long long* tc, long long* red) {
    const int ncell = (E.nx + 1) * (E.nz + 1);
    for (int t = 0; t < E.NT; t++) {
        long long s = 0;
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) s += eq_count(E, t, c / (E.nz + 1), c % (E.nz + 1));
        tc[t] = eq_blocksum(s, red);
    }
}
// places donor `rank`,`t`'s next id at a random point of corner volume (i,k)
__device__ int eq_place(const EqDev& E, int rank, int t, int i, int k) {
    const double r = E.dr * (double)i, s = E.ds * (double)k;
    double pr = eq_mzran(E.sd, rank, E.NR), ps = eq_mzran(E.sd, rank, E.NR);
    pr = (pr - 0.5) * E.dr;
    ps = (ps - 0.5) * E.ds;
    int& is = E.isv[rank * E.NT + t];
    is = is + 1;
    const int ID = eq_D(E, rank, t)[is];
    const int slot = E.iperm[ID - 1];
    double R = r + pr, S = s + ps;
    if (R <= 0.0) R = E.dist_r;
    if (R >= E.aspect) R = E.aspect - E.dist_r;
    if (S <= 0.0) S = E.dist_s;
    if (S >= 1.0) S = 1.0 - E.dist_s;
    E.rtr[slot] = R;
    E.str[slot] = S;
    return ID;
}

// donor search, lottery and serial remainder (composition.f90:226-543) in
// one block; threads < NR are the ranks
__global__ void __launch_bounds__(1024) k_eq_main(EqDev E, int64_t nfree) {
    __shared__ long long redl[33];
    __shared__ int redi[33];
    __shared__ long long tcount[8];
    __shared__ int minex[8];
    __shared__ int flags[4];  // 0: escape, 1: stop, 2: changed
    const int rank = threadIdx.x;
    const bool isrank = rank < E.NR;
    const int NT = E.NT, NR = E.NR;
    // ---- donors near the walls of edge volumes, shuffled per rank ----
    eq_edges(E, rank, 1);
    if (isrank)
        for (int t = 0; t < NT; t++) eq_shuffle(eq_D(E, rank, t), 1, E.isv[rank * NT + t], E.sd, rank, NR);
    __syncthreads();
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) E.isv2[q] = E.isv[q];
    __syncthreads();
    // ---- the rest of the edge volumes, then the interior volumes ----
    eq_edges(E, rank, 2);
    if (isrank) {
        int lo, cnt;
        eq_static(E.nx - 1, NR, rank, lo, cnt);
        for (int i = 1 + lo; i < 1 + lo + cnt; i++)
            for (int k = 1; k <= E.nz - 1; k++) eq_take(E, i, k, rank, 0);
    }
    __syncthreads();
    long long found = 0;
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) {
        E.nfr[q] = E.isv[q];
        found += E.isv[q];
    }
    found = eq_blocksum(found, redl);
    if (found != nfree) {
        if (threadIdx.x == 0) E.sc[EQ_ERR] = 1;
        return;
    }
    if (isrank)
        for (int t = 0; t < NT; t++)
            eq_shuffle(eq_D(E, rank, t), E.isv2[rank * NT + t] + 1, E.isv[rank * NT + t], E.sd, rank, NR);
    __syncthreads();
    // ---- lottery ----
    for (int i = threadIdx.x; i <= E.nx; i += blockDim.x) E.nx_loop[i] = i;
    for (int k = threadIdx.x; k <= E.nz; k += blockDim.x) E.nz_loop[k] = k;
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) E.isv[q] = 0;
    __syncthreads();
    eq_tracer_counts(E, tcount, redl);
    if (threadIdx.x == 0) {
        bool ideal = true;
        for (int t = 0; t < NT; t++) if (tcount[t] != E.sc[EQ_NIDEAL0 + t]) ideal = false;
        flags[0] = ideal ? 1 : 0;
    }
    __syncthreads();
    const int tpc0 = (int)E.sc[EQ_TPC0];
    long long passes = 0;
    for (int pass = 0; pass < 1000000; pass++) {
        if (flags[0] == 0) {
            eq_tracer_counts(E, tcount, redl);
            if (threadIdx.x == 0) {
                bool ideal = true;
                for (int t = 0; t < NT; t++) if (tcount[t] != E.sc[EQ_NIDEAL0 + t]) ideal = false;
                if (ideal) flags[0] = 1;
            }
            __syncthreads();
        }
        {
            const int m0 = (tpc0 > 0) ? eq_minval(E, 0, E.comp == 1, redi) : 0;
            if (threadIdx.x == 0) minex[0] = m0;
            for (int t = 1; t < NT; t++) {
                const int mt = ((int)E.sc[EQ_TPC0 + t] > 0) ? eq_minval(E, t, true, redi) : 0;
                if (threadIdx.x == 0) minex[t] = mt;
            }
        }
        long long used = 0;
        for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) used += E.isv[q];
        used = eq_blocksum(used, redl);
        if (threadIdx.x == 0) {
            bool allz = true;
            for (int t = 0; t < NT; t++) if (minex[t] != 0) allz = false;
            flags[1] = (allz || used >= nfree) ? 1 : 0;
            if (!flags[1]) {
                eq_shuffle(E.nx_loop, 0, E.nx, E.sd, 0, NR);
                eq_shuffle(E.nz_loop, 0, E.nz, E.sd, 0, NR);
            }
            flags[2] = 0;
        }
        __syncthreads();
        if (flags[1]) break;
        passes++;
        if (isrank) {
            int lo, cnt;
            eq_static(E.nx + 1, NR, rank, lo, cnt);
            int tt = 0;
            for (int ii = lo; ii < lo + cnt; ii++) {
                const int i = E.nx_loop[ii];
                for (int kk = 0; kk <= E.nz; kk++) {
                    const int k = E.nz_loop[kk];
                    const int type_save = eq_maxloc(E, i, k);
                    if (flags[0] == 0) {
                        for (int q = 0; q < NT; q++)
                            if (tcount[q] > E.sc[EQ_NIDEAL0 + q]) { tt = q; break; }
                    } else {
                        tt = type_save;
                    }
                    const size_t c = eq_cell(E, i, k);
                    if (E.nex[c] == minex[type_save] && E.isv[rank * NT + tt] < E.nfr[rank * NT + tt] && E.nex[c] < 0) {
                        const int ID = eq_place(E, rank, tt, i, k);
                        const int slot = E.iperm[ID - 1];
                        if (E.comp == 1) E.ttype[slot] = type_save;
                        E.counts[(size_t)tt * E.L.plane + IX(E.L, i, k)] -= 1;
                        E.counts[(size_t)E.ttype[slot] * E.L.plane + IX(E.L, i, k)] += 1;
                        E.nex[c] = E.nex[c] + 1;
                        flags[2] = 1;
                    }
                }
            }
        }
        __syncthreads();
        if (!flags[2]) break;
        __syncthreads();
    }
    // ---- remaining donors, one thread, ranks in turn ----
    for (int pass = 0; pass < 1000000; pass++) {
        {
            const int m0 = (tpc0 > 0) ? eq_minval(E, 0, E.comp == 1, redi) : 0;
            if (threadIdx.x == 0) minex[0] = m0;
            for (int t = 1; t < NT; t++) {
                const int mt = (tpc0 > 0) ? eq_minval(E, t, true, redi) : 0;
                if (threadIdx.x == 0) minex[t] = mt;
            }
        }
        long long used = 0;
        for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) used += E.isv[q];
        used = eq_blocksum(used, redl);
        if (threadIdx.x == 0) {
            bool allz = true;
            for (int t = 0; t < NT; t++) if (minex[t] != 0) allz = false;
            flags[1] = (allz || used >= nfree) ? 1 : 0;
            flags[2] = 0;
            if (!flags[1]) {
                int rk = 0;
                eq_shuffle(E.nx_loop, 0, E.nx, E.sd, 0, NR);
                eq_shuffle(E.nz_loop, 0, E.nz, E.sd, 0, NR);
                for (int ii = 0; ii <= E.nx; ii++) {
                    const int i = E.nx_loop[ii];
                    for (int kk = 0; kk <= E.nz; kk++) {
                        const int k = E.nz_loop[kk];
                        const int tt = eq_maxloc(E, i, k);
                        long long u = 0, a = 0;
                        for (int q = 0; q < NR; q++) { u += E.isv[q * NT + tt]; a += E.nfr[q * NT + tt]; }
                        const size_t c = eq_cell(E, i, k);
                        if (E.nex[c] == minex[tt] && u < a && E.nex[c] < 0) {
                            for (int g = 0; g < NR; g++) {
                                rk = rk + 1;
                                if (rk == NR) rk = 0;
                                if (E.isv[rk * NT + tt] < E.nfr[rk * NT + tt]) break;
                            }
                            const int ID = eq_place(E, rk, tt, i, k);
                            if (E.comp == 1) E.ttype[E.iperm[ID - 1]] = eq_maxloc(E, i, k);
                            E.nex[c] = E.nex[c] + 1;
                            flags[2] = 1;
                        }
                    }
                }
            }
        }
        __syncthreads();
        if (flags[1] || !flags[2]) break;
        __syncthreads();
    }
    // ---- the equalize.dat row ----
    for (int t = 0; t < NT; t++) {
        const int m = (E.comp == 0) ? eq_minval(E, 0, false, redi) : eq_minval(E, t, true, redi);
        if (threadIdx.x == 0) E.sc[EQ_MIN0 + t] = m;
    }
    const int ncell = (E.nx + 1) * (E.nz + 1);
    long long d = 0;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) if (E.nex[c] <= 0) d += E.nex[c];
    d = eq_blocksum(d, redl);
    long long used = 0;
    for (int q = threadIdx.x; q < NR * NT; q += blockDim.x) used += E.isv[q];
    used = eq_blocksum(used, redl);
    eq_tracer_counts(E, tcount, redl);
    if (threadIdx.x == 0) {
        E.sc[EQ_DEFICIT] = d;
        E.sc[EQ_MOVED] = used;
        E.sc[EQ_PASSES] = passes;
        for (int t = 0; t < NT; t++) E.sc[EQ_COUNT0 + t] = tcount[t];
    }
}

// temperatures of the moved tracers from Textend (composition.f90:545-556)
__global__ void k_eq_textend(Lay L, Phys P, const double* __restrict__ Tr, double* __restrict__ out) {
    Range2 r{-1, L.a + 1, -1, L.b + 1};
    RANGE_IK(r);
    if (!inr) return;
    out[IX(L, i, k)] = textend(L, P, Tr, i, k);
}
__global__ void k_eq_interp_T(Lay L, Phys P, EqDev E, const double* __restrict__ Td, const double* __restrict__ dTd,
                              double* __restrict__ Ttr) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)E.cap;
    if (g >= (int64_t)E.NR * E.NT * per) return;
    const int rank = (int)(g / ((int64_t)E.NT * per));
    const int t = (int)((g / per) % E.NT);
    const int p = (int)(g % per);
    if (p < 1 || p > E.isv[rank * E.NT + t]) return;
    const int slot = E.iperm[eq_D(E, rank, t)[p] - 1];
    Ttr[slot] = interp_taylor(L, P, Td, dTd, E.rtr[slot], E.str[slot]);
}

}  // namespace

static EqDev eq_dev(const EqHost& H) {
    EqDev E{};
    E.L = H.L; E.nx = H.L.a; E.nz = H.L.b; E.ntype = H.ntype; E.NT = H.ntype + 1; E.NR = H.NR; E.comp = H.comp;
    E.tracer = H.tracer; E.tpc = H.tpc; E.ntr = H.ntr; E.dr = H.P.dr; E.ds = H.P.ds; E.aspect = H.P.aspect;
    E.dist_r = H.dist_r; E.dist_s = H.dist_s; E.counts = H.counts; E.nempty = H.nempty;
    for (int j = 0; j < H.ntype && j < TC_MAX_TYPES; j++) E.C.p[j] = H.Cnew[j];
    E.rtr = H.rtr; E.str = H.str; E.ttype = H.ttype; E.perm = H.perm; E.iperm = H.iperm; E.nex = H.nex;
    E.off = H.off; E.cur = H.cur; E.ids = H.ids; E.sd = H.seeds; E.isv = H.isv; E.isv2 = H.isv2; E.nfr = H.nfr;
    E.nx_loop = H.nx_loop; E.nz_loop = H.nz_loop; E.sc = H.sc;
    return E;
}
__global__ void k_eq_set_total(int* off, int n, int64_t total) { off[n] = (int)total; }

// equalize_tracers, first part (composition.f90:99-162): nexcess of every
// corner volume; *nfree and whether any volume is off its target
int launch_equalize_count(cudaStream_t s, const EqHost& H, int64_t* nfree, int* nonzero) {
    EqDev E = eq_dev(H);
    const int ncell = (E.nx + 1) * (E.nz + 1);
    const unsigned cb = (unsigned)((ncell + 255) / 256);
    long long hsc[EQ_NSC] = {};
    for (int t = 0; t < E.NT; t++) hsc[EQ_NIDEAL0 + t] = H.Nideal[t];
    cudaMemcpyAsync(H.sc, hsc, sizeof(hsc), cudaMemcpyHostToDevice, s);
    if (E.comp == 1) { k_eq_tpc<<<cb, 256, 0, s>>>(E); tc_note_launch(); }
    k_eq_nexcess<<<cb, 256, 0, s>>>(E); tc_note_launch();
    cudaMemcpyAsync(hsc, H.sc, sizeof(hsc), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    *nfree = hsc[EQ_NFREE];
    *nonzero = hsc[EQ_NONZERO] ? 1 : 0;
    // tpc_type for the lottery's minexcess tests and the row
    for (int t = 0; t < E.NT; t++) {
        const long long n = hsc[EQ_TCNT0 + t];
        hsc[EQ_TPC0 + t] = (E.comp == 0) ? (t == 0 ? E.tpc : 0)
                                         : (n > 0 ? llround((double)hsc[EQ_TSUM0 + t] / (double)n) : 0);
    }
    cudaMemcpyAsync(H.sc + EQ_TPC0, hsc + EQ_TPC0, sizeof(long long) * 8, cudaMemcpyHostToDevice, s);
    return 0;
}

// equalize_tracers, the rest (composition.f90:163-556) with `donor` holding
// NR x NT x (nfree+1) ints; row receives the equalize.dat values (see
// tc_equalize_row); returns 0, TC_ERR_EQUALIZE or -1 on a CUDA error
int launch_equalize_move(cudaStream_t s, const EqHost& H, int64_t nfree, int* donor, int64_t* row, int* row_len) {
    EqDev E = eq_dev(H);
    E.cap = nfree + 1;
    E.donor = donor;
    const int ncell = (E.nx + 1) * (E.nz + 1);
    const unsigned cb = (unsigned)((ncell + 255) / 256);
    cudaMemsetAsync(E.donor, 0, sizeof(int) * (size_t)E.NR * E.NT * (size_t)E.cap, s);
    cudaMemsetAsync(E.isv, 0, sizeof(int) * E.NR * E.NT, s);
    cudaMemsetAsync(H.sc + EQ_ERR, 0, sizeof(long long), s);
    // per-volume id lists, ascending, then shuffled by the ranks
    k_eq_offsets_in<<<cb, 256, 0, s>>>(E, H.cnt); tc_note_launch();
    const int nbk = (ncell + 1023) / 1024;
    k_scan_blocks<<<nbk, 1024, 0, s>>>(H.cnt, ncell, H.bsum); tc_note_launch();
    k_scan_bsums<<<1, 1024, 0, s>>>(H.bsum, nbk); tc_note_launch();
    k_scan_final<<<nbk, 1024, 0, s>>>(H.cnt, ncell, H.bsum, E.off); tc_note_launch();
    k_eq_set_total<<<1, 1, 0, s>>>(E.off, ncell, E.ntr); tc_note_launch();
    const unsigned tb = (unsigned)((E.ntr + 255) / 256);
    k_eq_scatter<<<tb, 256, 0, s>>>(E); tc_note_launch();
    k_eq_sort_lists<<<cb, 256, 0, s>>>(E); tc_note_launch();
    k_eq_shuffle_lists<<<(E.NR + 31) / 32, 32, 0, s>>>(E); tc_note_launch();
    // donors, lottery, serial remainder
    const int nb = (E.NR <= 256) ? 256 : ((E.NR + 31) / 32) * 32;
    k_eq_main<<<1, nb, 0, s>>>(E, nfree); tc_note_launch();
    if (E.tracer == 1) {
        Range2 r{-1, E.L.a + 1, -1, E.L.b + 1};
        k_eq_textend<<<grid_for(r), dim3(BX, BY), 0, s>>>(E.L, H.P, H.Tratio, H.Td); tc_note_launch();
        launch_derivatives(s, E.L, H.P, H.Td, H.dTd);
        const int64_t n = (int64_t)E.NR * E.NT * E.cap;
        k_eq_interp_T<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(E.L, H.P, E, H.Td, H.dTd, H.Ttr); tc_note_launch();
    }
    long long hsc[EQ_NSC];
    cudaMemcpyAsync(hsc, H.sc, sizeof(hsc), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    if (hsc[EQ_ERR]) return TC_ERR_EQUALIZE;
    int n = 0;
    row[n++] = E.NT;
    for (int t = 0; t < E.NT; t++) row[n++] = hsc[EQ_TPC0 + t];
    for (int t = 0; t < E.NT; t++) row[n++] = hsc[EQ_MIN0 + t];
    row[n++] = hsc[EQ_DEFICIT];
    row[n++] = hsc[EQ_MOVED];
    row[n++] = nfree;
    for (int t = 0; t < E.NT; t++) row[n++] = hsc[EQ_COUNT0 + t];
    *row_len = n;
    return 0;
}
