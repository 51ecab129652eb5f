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

// interpolate (composition.f90:838-898) with order=2: one r-derivative table
// DER(1,i,k) and a 3-point s-stencil; int() truncates, as in Fortran.
__device__ __forceinline__ double interp_taylor(const Lay& L, const Phys& P, const double* __restrict__ f,
                                                const double* __restrict__ der, double r, double s) {
    const int i = (int)(r / P.dr);
    const int k = (int)(s / P.ds);
    double hr = r - (double)i * P.dr;
    double fR0, fR1, fR2, fR3;  // jj = -1, 0, 1, 2
    if (hr <= P.dro2) {
        const double a1 = hr / 1.0;
        fR0 = __ldg(f + IX(L, i, k - 1)) + __ldg(der + IX(L, i, k - 1)) * a1;
        fR1 = __ldg(f + IX(L, i, k)) + __ldg(der + IX(L, i, k)) * a1;
        fR2 = __ldg(f + IX(L, i, k + 1)) + __ldg(der + IX(L, i, k + 1)) * a1;
        fR3 = __ldg(f + IX(L, i, k + 2)) + __ldg(der + IX(L, i, k + 2)) * a1;
    } else {
        hr = P.dr - hr;
        const double a1 = (-hr) / 1.0;
        fR0 = __ldg(f + IX(L, i + 1, k - 1)) + __ldg(der + IX(L, i + 1, k - 1)) * a1;
        fR1 = __ldg(f + IX(L, i + 1, k)) + __ldg(der + IX(L, i + 1, k)) * a1;
        fR2 = __ldg(f + IX(L, i + 1, k + 1)) + __ldg(der + IX(L, i + 1, k + 1)) * a1;
        fR3 = __ldg(f + IX(L, i + 1, k + 2)) + __ldg(der + IX(L, i + 1, k + 2)) * a1;
    }
    double hs = s - (double)k * P.ds;
    double fin;
    if (hs <= P.dso2) {
        double DERs = (-0.5 * fR0 + 0.5 * fR2) / P.ds;
        fin = fR1 + DERs * (hs / 1.0);
    } else {
        hs = P.ds - hs;
        double DERs = (-0.5 * fR1 + 0.5 * fR3) / P.ds;
        fin = fR2 + DERs * ((-hs) / 1.0);
    }
    return fin;
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
    const double tr = interp_taylor(L, P, u, du, r, s);
    const double ts = interp_taylor(L, P, w, dw, r, s);
    if (tT.f) {
        // energy.f90:213-223, 292-310, 371-375, 437-440
        const double te = interp_taylor(L, P, tT.f, tT.der, r, s);
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
            const int i = (int)round(r / P.dr);
            const int k = (int)round(s / P.ds);
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
    int i = (int)round(r / P.dr), k = (int)round(s / P.ds);
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
