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

// stage 1: (rin,sin)=(rtr0,str0) -> acc=k1, out=rtr1
// stage 2: (rin,sin)=(rtr1,str1) -> RK2: acc=final rtr;  RK4: acc+=2k2, out=rtr2
// stage 3: (rin,sin)=(rtr2,str2) -> acc+=2k3, out=rtr1
// stage 4: (rin,sin)=(rtr1,str1) -> acc=final rtr
__global__ void k_tracer_stage(Lay L, Phys P, int torder, int stage, int64_t ntr, const double* __restrict__ rin,
                               const double* __restrict__ sin, const double* __restrict__ r0,
                               const double* __restrict__ s0, double* __restrict__ racc, double* __restrict__ sacc,
                               double* __restrict__ rout, double* __restrict__ sout, const double* __restrict__ u,
                               const double* __restrict__ w, const double* __restrict__ du,
                               const double* __restrict__ dw, const DevScalars* __restrict__ ds) {
    int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ntr) return;
    const double dt = ds->dt;
    const double r = rin[id], s = sin[id];
    // positions outside the box were already reported by the histogram that
    // precedes every stage (the reference stops there); never index with them
    if (!(r > 0.0 && r < P.aspect && s > 0.0 && s < 1.0)) return;
    const double tr = interp_taylor(L, P, u, du, r, s);
    const double ts = interp_taylor(L, P, w, dw, r, s);
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
                         const double* du, const double* dw, const DevScalars* ds) {
    if (ntr <= 0) return;
    unsigned nb = (unsigned)((ntr + 255) / 256);
    k_tracer_stage<<<nb, 256, 0, s>>>(L, P, torder, stage, ntr, rin, sin, r0, s0, racc, sacc, rout, sout, u, w, du,
                                      dw, ds); tc_note_launch();
}

// histogram of tracers_to_corners (composition.f90:695-726): nint() rounds
// half away from zero (CUDA round()).  Tracers of a warp that land in the
// same counter are combined before one atomic (they are mostly cell-sorted).
__global__ void k_histogram(Lay L, Phys P, int64_t ntr, const double* __restrict__ rr, const double* __restrict__ ss,
                            const int* __restrict__ ttype, int* __restrict__ counts, int* __restrict__ flag) {
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
            else key = (int)((size_t)t * L.plane + IX(L, i, k));
        }
    }
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(counts + key, __popc(peers));
}
void launch_histogram(cudaStream_t s, const Lay& L, const Phys& P, int64_t ntr, const double* r, const double* sv,
                      const int* ttype, int* counts, DevScalars* ds) {
    cudaMemsetAsync(counts, 0, sizeof(int) * L.plane * (size_t)(P.ntype + 1), s);
    if (ntr <= 0) return;
    unsigned nb = (unsigned)((ntr + 255) / 256);
    k_histogram<<<nb, 256, 0, s>>>(L, P, ntr, r, sv, ttype, counts, &ds->flag_outside); tc_note_launch();
}

// ghost mirror of count_type, nempty and the tracer ratio (composition.f90:745-776)
__global__ void k_counts_to_comp(Lay L, Phys P, Range2 r, int* __restrict__ counts, int* __restrict__ nempty,
                                 CPtrsW Cn) {
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
                           double* const* Cnew) {
    CPtrsW C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cnew[j];
    Range2 r{-SP, L.a + SP, -SP, L.b + SP};
    k_counts_to_comp<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, counts, nempty, C); tc_note_launch();
}
