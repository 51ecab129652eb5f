// k_field.cu -- fine-grid field kernels: boundary conditions, the T and C
// filters, conductivity, velocities, energy-equation RK stages, time-step
// bound and the stats.dat integrals.
//
// Reference: energy.f90 (load_conductivity_array :31-58, energy_space :60-80,
// energy_time :117-453, enforceBCs :455-475, stability_RK4 :600-646, eigA /
// eigD :686-706), smoother.f90 / multigrid_cycle.f90 (smoothness, smoother_space,
// smoother_time, smoother_time_T), momentum.f90 (compute_strain_rate_invariant
// :32-62, compute_velocities :532-551), composition.f90 (enforceBCs_comp
// :792-803, velocityBCs :806-836, compute_derivatives :900-919) and basics.f90
// (stats :236-324, integrate2D / integrate1Dx / integrate1Dz :341-403).
// On a uniform grid the metrics are xr = zs = 1, xrr = zss = 0 and the
// kernels skip them; on a stretched grid (P.M.on) they apply them as the
// reference does.  Every kernel keeps the reference's operation order (no
// FMA contraction), so with identical inputs its output equals the CPU
// restatement bit for bit.
#include "tc_device.cuh"

// enforceBCs (energy.f90:455-475): every ghost / boundary-row value as a
// function of interior values only.
__global__ void k_enforce_T(Lay L, Range2 r, double* __restrict__ T, int Tbot) {
    RANGE_IK(r);
    if (!inr) return;
    const int nx = L.a, nz = L.b;
    if (i >= 0 && i <= nx && k >= 1 && k <= nz - 1) return;
    int mi = (i < 0) ? -i : ((i > nx) ? 2 * nx - i : i);
    double v;
    if (k > nz) v = -T[IX(L, mi, 2 * nz - k)];
    else if (k == nz) v = 0.0;
    else if (k < 0) {
        double src = T[IX(L, mi, -k)];
        v = (Tbot == 0) ? (-(src - 1.0) + 1.0) : src;
    } else if (k == 0) v = (Tbot == 0) ? 1.0 : T[IX(L, mi, 0)];
    else v = T[IX(L, mi, k)];
    T[IX(L, i, k)] = v;
}
void launch_enforce_T(cudaStream_t s, const Lay& L, double* T, int Tbot) {
    Range2 r{-SP, L.a + SP, -SP, L.b + SP};
    k_enforce_T<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, r, T, Tbot); tc_note_launch();
}

// enforceBCs_comp (composition.f90:792-803).  Its four statements share one
// loop over i, so rows -1 and nz+1 take the PREVIOUS values of the outer side
// ghosts at columns -2 and nx+2 (they are refreshed only in the i=2 pass).
// Cprev holds those previous values (it may alias C: the thread that owns a
// side ghost reads its old value before overwriting it).
__global__ void k_enforce_comp(Lay L, Range2 r, double* C, const double* Cprev) {
    RANGE_IK(r);
    if (!inr) return;
    const int nx = L.a, nz = L.b;
    if (i >= 0 && i <= nx && k >= 0 && k <= nz) return;
    const bool outer = (i == -2 || i == nx + 2);
    if (outer && (k == -1 || k == nz + 1)) return;  // written by the owner of (i, 1) / (i, nz-1)
    int mi = (i < 0) ? -i : ((i > nx) ? 2 * nx - i : i);
    if (k >= 0 && k <= nz) {
        double v = C[IX(L, mi, k)];
        if (outer && (k == 1 || k == nz - 1)) {
            double old = Cprev[IX(L, i, k)];
            C[IX(L, i, (k == 1) ? -1 : nz + 1)] = old;
            if (k == 1 && nz - 1 == 1) C[IX(L, i, nz + 1)] = old;
        }
        C[IX(L, i, k)] = v;
        return;
    }
    int mk = (k < 0) ? -k : 2 * nz - k;
    C[IX(L, i, k)] = C[IX(L, mi, mk)];
}
void launch_enforce_comp(cudaStream_t s, const Lay& L, double* C, const double* Cprev_ghosts) {
    Range2 r{-SP, L.a + SP, -SP, L.b + SP};
    k_enforce_comp<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, r, C, Cprev_ghosts ? Cprev_ghosts : C); tc_note_launch();
}

// smoothness (multigrid_cycle.f90:175-195): largest jump to the five
// neighbours (i,k-1),(i+1,k-1),(i+1,k),(i,k+1),(i+1,k+1).
__global__ void k_smoothness(Lay L, Range2 r, const double* __restrict__ T, RedScratch rs, double* out) {
    RANGE_IK(r);
    double a = -INFINITY;
    if (inr) {
        const size_t ld = (size_t)L.ld;
        size_t x = IX(L, i, k);
        double c = T[x];
        double a1 = fabs(T[x - ld] - c), a2 = fabs(T[x + 1 - ld] - c), a3 = fabs(T[x + 1] - c);
        double a4 = fabs(T[x + ld] - c), a5 = fabs(T[x + 1 + ld] - c);
        a = fmax(fmax(fmax(fmax(a1, a2), a3), a4), a5);
        if (a < 0.0) a = 0.0;
    }
    reduce_to(RED_MAX, a, rs.part, rs.count, out);
}
void launch_smoothness(cudaStream_t s, const Lay& L, const double* f, RedScratch rs, DevScalars* ds) {
    Range2 r{0, L.a - 1, 1, L.b - 1};
    k_smoothness<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, r, f, rs, &ds->diff); tc_note_launch();
}

__device__ __forceinline__ double lap5(const double* __restrict__ T, size_t x, size_t ld, double dr2, double ds2) {
    double c = T[x];
    double Trr = (T[x - 1] + -2.0 * c + T[x + 1]) / dr2;
    double Tss = (T[x - ld] + -2.0 * c + T[x + ld]) / ds2;
    return Trr + Tss;
}
// smoother_space (smoother.f90:122-140) at node (i, k), stretched or uniform
__device__ __forceinline__ double smoother_space(const Phys& P, const double* __restrict__ T, size_t x, size_t ld,
                                                 int i, int k) {
    if (!P.M.on) return lap5(T, x, ld, P.dr2, P.ds2);
    const double c = T[x];
    const double Tr = (-0.5 * T[x - 1] + 0.5 * T[x + 1]) / P.dr, Ts = (-0.5 * T[x - ld] + 0.5 * T[x + ld]) / P.ds;
    const double Trr = (T[x - 1] + -2.0 * c + T[x + 1]) / P.dr2, Tss = (T[x - ld] + -2.0 * c + T[x + ld]) / P.ds2;
    const double x1 = mt(P.M.xr, i), z1 = mt(P.M.zs, k);
    const double Tx = Tr / x1, Tz = Ts / z1;
    const double Txx = (Trr - Tx * mt(P.M.xrr, i)) / (x1 * x1);
    const double Tzz = (Tss - Tz * mt(P.M.zss, k)) / (z1 * z1);
    return Txx + Tzz;
}

// one Richardson step of smoother_time_T (smoother.f90:343-377)
__global__ void k_smooth_T(Lay L, Phys P, Range2 r, const double* __restrict__ Tin, double* __restrict__ Tout,
                           const double* __restrict__ dts) {
    RANGE_IK(r);
    if (!inr) return;
    size_t x = IX(L, i, k);
    double temp = smoother_space(P, Tin, x, (size_t)L.ld, i, k);
    double d = dts[x] * P.courantT;
    Tout[x] = Tin[x] + d * temp;
}
void launch_smooth_T_step(cudaStream_t s, const Lay& L, const Phys& P, const double* Tin, double* Tout,
                          const double* dts) {
    Range2 r{0, L.a, 0, L.b};
    k_smooth_T<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, Tin, Tout, dts); tc_note_launch();
}

// one step of smoother_time (smoother.f90:287-341) for one type
__global__ void k_smooth_C(Lay L, Phys P, Range2 r, const double* __restrict__ Cin, double* __restrict__ Cout,
                           const double* __restrict__ dts, double c, const double* cdev) {
    RANGE_IK(r);
    if (!inr) return;
    if (cdev) c = *cdev;  // the factor the device-side filter loop chose
    size_t x = IX(L, i, k);
    double temp = smoother_space(P, Cin, x, (size_t)L.ld, i, k);
    double d = dts[x] * P.courantC;
    double v = Cin[x] + c * d * temp;
    if (v < 0.0) v = 0.0;
    if (v > 1.0) v = 1.0;
    Cout[x] = v;
}
void launch_smooth_C_step(cudaStream_t s, const Lay& L, const Phys& P, const double* Cin, double* Cout,
                          const double* dts, double c, const double* cdev) {
    Range2 r{0, L.a, 0, L.b};
    k_smooth_C<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, Cin, Cout, dts, c, cdev); tc_note_launch();
}

// load_conductivity_array (energy.f90:31-58)
__global__ void k_conduct(Lay L, Phys P, Range2 r, CPtrs Cv, double* __restrict__ cd) {
    RANGE_IK(r);
    if (!inr) return;
    const int nx = L.a, nz = L.b;
    int mi = (i < 0) ? -i : ((i > nx) ? 2 * nx - i : i);
    int mk = (k < 0) ? -k : ((k > nz) ? 2 * nz - k : k);
    double c = 1.0;
    if (P.comp != 0)
        for (int j = 0; j < P.ntype; j++) c = exp(-Cv.p[j][IX(L, mi, mk)] * P.lncf[j]);
    cd[IX(L, i, k)] = c;
}
__global__ void k_conduct_grad(Lay L, Phys P, Range2 r, const double* __restrict__ cd, double* __restrict__ cr,
                               double* __restrict__ cs) {
    RANGE_IK(r);
    if (!inr) return;
    const size_t ld = (size_t)L.ld;
    size_t x = IX(L, i, k);
    cr[x] = (-0.5 * cd[x - 1] + 0.5 * cd[x + 1]) / P.dr;
    cs[x] = (-0.5 * cd[x - ld] + 0.5 * cd[x + ld]) / P.ds;
}
void launch_conductivity(cudaStream_t s, const Lay& L, const Phys& P, const double* const* Cvis, double* conduct,
                         double* conduct_r, double* conduct_s) {
    CPtrs C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cvis[j];
    Range2 r{-SP, L.a + SP, -SP, L.b + SP};
    k_conduct<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, C, conduct); tc_note_launch();
    Range2 r2{-1, L.a + 1, -1, L.b + 1};
    k_conduct_grad<<<grid_for(r2), dim3(BX, BY), 0, s>>>(L, P, r2, conduct, conduct_r, conduct_s); tc_note_launch();
}

// compute_velocities + velocityBCs (momentum.f90:532-551, composition.f90:806-836),
// span_interp = 1.  Each cell's final value is written from SF directly.
__device__ __forceinline__ double uf_(const Lay& L, const Phys& P, const double* SF, int i, int k) {
    const size_t ld = (size_t)L.ld;
    size_t x = IX(L, i, k);
    const double SFs = (-0.5 * SF[x - ld] + 0.5 * SF[x + ld]) / P.ds;
    return P.M.on ? SFs / mt(P.M.zs, k) : SFs;
}
__device__ __forceinline__ double wf_(const Lay& L, const Phys& P, const double* SF, int i, int k) {
    size_t x = IX(L, i, k);
    const double SFr = (-0.5 * SF[x - 1] + 0.5 * SF[x + 1]) / P.dr;
    return -(P.M.on ? SFr / mt(P.M.xr, i) : SFr);
}
__global__ void k_velocities(Lay L, Phys P, Range2 r, const double* __restrict__ SF, double* __restrict__ u,
                             double* __restrict__ w) {
    RANGE_IK(r);
    if (!inr) return;
    const int nx = L.a, nz = L.b;
    const double vs = (P.Vbc == 1) ? -1.0 : 1.0;
    // ---- u ----
    double uv;
    if (i == 0 || i == nx) uv = 0.0;
    else if (P.Vbc == 1 && (k == 0 || k == nz)) uv = 0.0;
    else {
        // value of u(ii,kk) after the first two statements of velocityBCs
        auto u_step1 = [&](int ii, int kk) -> double {
            if (kk < 0) return vs * uf_(L, P, SF, ii, -kk);
            if (kk > nz) return vs * uf_(L, P, SF, ii, 2 * nz - kk);
            return uf_(L, P, SF, ii, kk);
        };
        if (i < 0) uv = -u_step1(-i, k);
        else if (i > nx) uv = -u_step1(2 * nx - i, k);
        else uv = u_step1(i, k);
    }
    // ---- w ----
    double wv;
    if (k == 0 || k == nz) wv = 0.0;
    else {
        int mi = (i < 0) ? -i : ((i > nx) ? 2 * nx - i : i);
        if (k < 0) wv = -wf_(L, P, SF, mi, -k);
        else if (k > nz) wv = -wf_(L, P, SF, mi, 2 * nz - k);
        else wv = wf_(L, P, SF, mi, k);
    }
    size_t x = IX(L, i, k);
    u[x] = uv;
    w[x] = wv;
}
void launch_velocities(cudaStream_t s, const Lay& L, const Phys& P, const double* SF, double* u, double* w) {
    Range2 r{-1, L.a + 1, -1, L.b + 1};
    k_velocities<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, SF, u, w); tc_note_launch();
}

// compute_derivatives (composition.f90:900-919), order=2
__global__ void k_derivatives(Lay L, Phys P, Range2 r, const double* __restrict__ f, double* __restrict__ der) {
    RANGE_IK(r);
    if (!inr) return;
    size_t x = IX(L, i, k);
    der[x] = (-0.5 * f[x - 1] + 0.5 * f[x + 1]) / P.dr;
}
void launch_derivatives(cudaStream_t s, const Lay& L, const Phys& P, const double* f, double* der) {
    Range2 r{0, L.a, -1, L.b + 1};
    k_derivatives<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, f, der); tc_note_launch();
}

// stability_RK4 (energy.f90:600-646), tracer=0 branch of eigA
__global__ void k_stab(Lay L, Phys P, Range2 r, const double* __restrict__ cd, const double* __restrict__ cr,
                       const double* __restrict__ cs, const double* __restrict__ u, const double* __restrict__ w,
                       RedScratch rs, double* outA, int which) {
    RANGE_IK(r);
    double v = -INFINITY;
    if (inr) {
        size_t x = IX(L, i, k);
        if (P.M.on) {
            // eigA / eigD on a stretched grid (energy.f90:686-706)
            const double x1 = mt(P.M.xr, i), z1 = mt(P.M.zs, k);
            if (which == 0) {
                double ax = -(cd[x] * mt(P.M.xrr, i) / mt(P.M.xr3, i)) - u[x] / x1 + cr[x] / (x1 * x1);
                double az = -(cd[x] * mt(P.M.zss, k) / mt(P.M.zs3, k)) - w[x] / z1 + cs[x] / (z1 * z1);
                v = fabs(ax) * P.Tr_max + fabs(az) * P.Ts_max;
            } else {
                v = cd[x] * (fabs(P.Trr_max / (x1 * x1)) + fabs(P.Tss_max / (z1 * z1)));
            }
        } else if (which == 0) {
            double ax = -(cd[x] * 0.0) - u[x] + cr[x];
            double az = -(cd[x] * 0.0) - w[x] + cs[x];
            v = fabs(ax) * P.Tr_max + fabs(az) * P.Ts_max;
        } else {
            v = cd[x] * (fabs(P.Trr_max) + fabs(P.Tss_max));
        }
    }
    reduce_to(RED_MAX, v, rs.part, rs.count, outA);
}
__global__ void k_dt(Phys P, DevScalars* ds, double courant, double dt_manual) {
    double dt;
    if (P.RaT != 0.0) {
        double eA = ds->eA_max, eD = ds->eD_max, dtA, dtD;
        if (eA < 0.0) eA = 0.0;
        if (eD < 0.0) eD = 0.0;
        if (P.torder == 2) {
            if (eA >= eD) ds->flag_rk2 = 1;
            dtA = 1.0 / eA;
            dtD = 2.0 / eD;
        } else {
            dtA = 2.8 / eA;
            dtD = 2.8 / eD;
        }
        if (eA == 0.0) dt = dtD;
        else dt = 1.0 / (1.0 / dtA + 1.0 / dtD);
    } else {
        dt = dt_manual;
    }
    ds->dt = courant * dt;
}
void launch_stability(cudaStream_t s, const Lay& L, const Phys& P, const double* conduct, const double* conduct_r,
                      const double* conduct_s, const double* u, const double* w, double courant, double dt_manual,
                      RedScratch rs, DevScalars* ds) {
    Range2 r{0, L.a, 0, L.b};
    if (P.RaT != 0.0) {
        k_stab<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, conduct, conduct_r, conduct_s, u, w, rs, &ds->eA_max, 0); tc_note_launch();
        k_stab<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, conduct, conduct_r, conduct_s, u, w, rs, &ds->eD_max, 1); tc_note_launch();
    }
    k_dt<<<1, 1, 0, s>>>(P, ds, courant, dt_manual); tc_note_launch();
}

// energy_space (energy.f90:60-80) and the four RK stage updates of energy_time
__global__ void k_energy(Lay L, Phys P, Range2 r, int stage, const double* __restrict__ Tin,
                         const double* __restrict__ T0, double* __restrict__ T, double* __restrict__ Tout,
                         const double* __restrict__ cd, const double* __restrict__ cr, const double* __restrict__ cs,
                         const double* __restrict__ u, const double* __restrict__ w, CPtrs Cv, const DevScalars* ds) {
    RANGE_IK(r);
    if (!inr) return;
    const size_t ld = (size_t)L.ld;
    size_t x = IX(L, i, k);
    double Tr = (-0.5 * Tin[x - 1] + 0.5 * Tin[x + 1]) / P.dr;
    double Ts = (-0.5 * Tin[x - ld] + 0.5 * Tin[x + ld]) / P.ds;
    double c = Tin[x];
    double Trr = (Tin[x - 1] + -2.0 * c + Tin[x + 1]) / P.dr2;
    double Tss = (Tin[x - ld] + -2.0 * c + Tin[x + ld]) / P.ds2;
    double kx = cr[x], kz = cs[x];
    double heat;
    if (P.comp == 0) heat = P.H;
    else {
        double sC = 0.0;
        for (int j = 0; j < P.ntype; j++) sC = sC + Cv.p[j][x];
        heat = P.H * (1.0 - sC);
        for (int j = 0; j < P.ntype; j++) heat = P.Htype[j] * Cv.p[j][x] + heat;
    }
    double temp;
    if (P.M.on) {
        // energy_space on a stretched grid (energy.f90:60-80)
        const double x1 = mt(P.M.xr, i), z1 = mt(P.M.zs, k);
        kx = kx / x1;
        kz = kz / z1;
        const double Tx = Tr / x1, Tz = Ts / z1;
        const double Txx = (Trr - Tx * mt(P.M.xrr, i)) / (x1 * x1);
        const double Tzz = (Tss - Tz * mt(P.M.zss, k)) / (z1 * z1);
        temp = cd[x] * (Txx + Tzz) + (kx * Tx + kz * Tz) - u[x] * Tx - w[x] * Tz + heat;
    } else {
        temp = cd[x] * (Trr + Tss) + (kx * Tr + kz * Ts) - u[x] * Tr - w[x] * Ts + heat;
    }
    const double dt = ds->dt;
    if (stage == 1) {
        T[x] = temp;
        Tout[x] = T0[x] + 0.5 * dt * temp;
    } else if (stage == 2) {
        T[x] = T[x] + 2.0 * temp;
        Tout[x] = T0[x] + 0.5 * dt * temp;
    } else if (stage == 3) {
        T[x] = T[x] + 2.0 * temp;
        Tout[x] = T0[x] + dt * temp;
    } else {
        T[x] = T0[x] + (dt / 6.0) * (T[x] + temp);
    }
}
void launch_energy_stage(cudaStream_t s, const Lay& L, const Phys& P, int stage, const double* Tin,
                         const double* T0, double* T, double* Tout, const double* conduct, const double* conduct_r,
                         const double* conduct_s, const double* u, const double* w, const double* const* Cvis,
                         const DevScalars* ds) {
    CPtrs C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cvis[j];
    Range2 r{0, L.a, 0, L.b};
    k_energy<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, stage, Tin, T0, T, Tout, conduct, conduct_r, conduct_s, u,
                                                   w, C, ds); tc_note_launch();
}

// compute_strain_rate_invariant (momentum.f90:32-62), interior nodes
__global__ void k_strain(Lay L, Phys P, Range2 r, const double* __restrict__ u, const double* __restrict__ w,
                         double* __restrict__ st) {
    RANGE_IK(r);
    if (!inr) return;
    const size_t ld = (size_t)L.ld;
    size_t x = IX(L, i, k);
    double ur = (-0.5 * u[x - 1] + 0.5 * u[x + 1]) / P.dr;
    double us = (-0.5 * u[x - ld] + 0.5 * u[x + ld]) / P.ds;
    double wr = (-0.5 * w[x - 1] + 0.5 * w[x + 1]) / P.dr;
    double ws = (-0.5 * w[x - ld] + 0.5 * w[x + ld]) / P.ds;
    if (P.M.on) {
        // ux = ur / xr, uz = us / zs, wx = wr / xr, wz = ws / zs (momentum.f90:45-48)
        const double x1 = mt(P.M.xr, i), z1 = mt(P.M.zs, k);
        ur = ur / x1; us = us / z1; wr = wr / x1; ws = ws / z1;
    }
    double q = 0.5 * (2.0 * (ur * ur + ws * ws) + (us + wr) * (us + wr));
    st[x] = sqrt(q);
}
void launch_strain(cudaStream_t s, const Lay& L, const Phys& P, const double* u, const double* w, double* strain) {
    Range2 r{0, L.a, 0, L.b};
    k_strain<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, P, r, u, w, strain); tc_note_launch();
}

// ---------------------------------------------------------------------------
// stats: integrate1Dx of each row in the reference's serial order (one
// thread per row), then integrate1Dz serially; the host applies the final
// divisions and square roots exactly as basics.f90:236-324.
// integ layout: [0..3] C by type, [4..7] C from kent by type, [8] u^2+w^2,
// [9] T, [10] RaT/conduct/vis, [11] top-row u^2+w^2, [12] Nu numerator,
// [13] Nu denominator, [14] Nu_bot numerator, [15..18] q1..q4
// ---------------------------------------------------------------------------
#define NROWINT 7
// The integrands are evaluated in parallel into shared memory, CH columns at
// a time; one thread per running sum then adds them serially with the
// reference's expression, so every sum takes the same operations in the same
// order as the serial loop (the values are the same doubles).
constexpr int kStatCH = 512;
constexpr int kStatThreads = 256;

// integrand q at (i, k): 0..3 C by type, 4 u^2+w^2, 5 T, 6 RaT/conduct/vis
__device__ __forceinline__ double stat_integrand(const Lay& L, const Phys& P, const double* __restrict__ T,
                                                 const double* __restrict__ u, const double* __restrict__ w,
                                                 const double* __restrict__ cd, const double* __restrict__ vis,
                                                 const CPtrs& Cn, int q, int i, int k) {
    const size_t x = IX(L, i, k);
    if (q < 4) return (q < P.ntype) ? Cn.p[q][x] : 0.0;
    if (q == 4) return u[x] * u[x] + w[x] * w[x];
    if (q == 5) return T[x];
    return P.RaT / cd[x] / vis[x];
}
__device__ __forceinline__ bool stat_row_active(const Phys& P, int q) {
    if (q < 4 && q >= P.ntype) return false;
    if (q >= 5 && P.RaT == 0.0) return false;
    return true;
}

// integrate1Dx of every row k (basics.f90 trapezoid, left to right): one
// block per row
__global__ void __launch_bounds__(kStatThreads) k_stats_rows(Lay L, Phys P, const double* __restrict__ T,
                                                             const double* __restrict__ u,
                                                             const double* __restrict__ w,
                                                             const double* __restrict__ cd,
                                                             const double* __restrict__ vis, CPtrs Cn,
                                                             double* __restrict__ rows) {
    __shared__ double fv[NROWINT][kStatCH + 1];
    const int k = blockIdx.x;
    const int nx = L.a, nz = L.b;
    const int t = threadIdx.x;
    double fint = 0.0;
    for (int c0 = 0; c0 < nx; c0 += kStatCH) {
        const int n = min(kStatCH, nx - c0);  // sums over i = c0..c0+n-1 use f(c0..c0+n)
        for (int e = t; e < NROWINT * (n + 1); e += blockDim.x) {
            const int q = e / (n + 1), j = e % (n + 1);
            fv[q][j] = stat_row_active(P, q) ? stat_integrand(L, P, T, u, w, cd, vis, Cn, q, c0 + j, k) : 0.0;
        }
        __syncthreads();
        if (t < NROWINT && stat_row_active(P, t)) {
            double fprev = fv[t][0];
            double xprev = P.M.on ? mt(P.M.xr, c0) : 1.0;
            for (int j = 0; j < n; j++) {
                const double fn = fv[t][j + 1];
                const double xn = P.M.on ? mt(P.M.xr, c0 + j + 1) : 1.0;
                fint = fint + 0.5 * (fprev * xprev + fn * xn) * P.dr;
                fprev = fn;
                xprev = xn;
            }
        }
        __syncthreads();
    }
    if (t < NROWINT) rows[(size_t)t * (nz + 1) + k] = stat_row_active(P, t) ? fint : 0.0;
}

// integrate1Dz of the row integrals (from k = 0, and from kent for the C
// types), the top-row and Nusselt integrals along x, the corner fluxes and
// the top-row strain maximum.  One block.
__global__ void __launch_bounds__(kStatThreads) k_stats_final(Lay L, Phys P, int kent,
                                                              const double* __restrict__ rows,
                                                              const double* __restrict__ T,
                                                              const double* __restrict__ u,
                                                              const double* __restrict__ w,
                                                              const double* __restrict__ cd,
                                                              const double* __restrict__ st, DevScalars* ds) {
    __shared__ double fv[NROWINT][kStatCH + 1];
    __shared__ double red[kStatThreads / 32];
    const int nx = L.a, nz = L.b;
    const int t = threadIdx.x;
    const size_t ld = (size_t)L.ld;
    // z-integrals: thread t < NROWINT sums row t from k = 0; thread
    // NROWINT + q (q < 4) sums C type q from kent
    {
        const int q = (t < NROWINT) ? t : t - NROWINT;
        const int k0 = (t < NROWINT) ? 0 : kent;
        bool active = (t < NROWINT + 4);
        if (q < 4 && q >= P.ntype) active = false;
        if (t >= NROWINT && q >= 4) active = false;
        double fint = 0.0;
        for (int c0 = 0; c0 < nz; c0 += kStatCH) {
            const int n = min(kStatCH, nz - c0);
            for (int e = t; e < NROWINT * (n + 1); e += blockDim.x) {
                const int qq = e / (n + 1), j = e % (n + 1);
                fv[qq][j] = rows[(size_t)qq * (nz + 1) + c0 + j];
            }
            __syncthreads();
            if (active) {
                for (int j = 0; j < n; j++) {
                    if (c0 + j < k0) continue;
                    const double za = P.M.on ? mt(P.M.zs, c0 + j) : 1.0, zb = P.M.on ? mt(P.M.zs, c0 + j + 1) : 1.0;
                    fint = fint + 0.5 * (fv[q][j] * za + fv[q][j + 1] * zb) * P.ds;
                }
            }
            __syncthreads();
        }
        if (active) {
            const int slot = (t < NROWINT) ? ((q < 4) ? q : (q - 4 + 8)) : (4 + q);
            ds->integ[slot] = fint;
        }
    }
    // top-row mobility integrand and the Nusselt integrands: values 0 top(i),
    // 1 -cd*dT/dz at the top, 2 T at the bottom, 3 -cd*dT/dz at the bottom;
    // thread j < 4 keeps sum j
    {
        const bool rat = (P.RaT != 0.0);
        const double zs_top = P.M.on ? mt(P.M.zs, nz) : 1.0, zs_bot = P.M.on ? mt(P.M.zs, 0) : 1.0;
        double acc = 0.0;
        for (int c0 = 0; c0 < nx; c0 += kStatCH) {
            const int n = min(kStatCH, nx - c0);
            for (int e = t; e < 4 * (n + 1); e += blockDim.x) {
                const int q = e / (n + 1), i = c0 + e % (n + 1);
                double v = 0.0;
                if (q == 0) {
                    const size_t x = IX(L, i, nz);
                    v = u[x] * u[x] + w[x] * w[x];
                } else if (rat && q == 1) {
                    const size_t x = IX(L, i, nz);
                    v = -cd[x] * ((-0.5 * T[x - ld] + 0.5 * T[x + ld]) / P.ds / zs_top);
                } else if (rat && q == 2) {
                    v = T[IX(L, i, 0)];
                } else if (rat && q == 3) {
                    const size_t x = IX(L, i, 0);
                    v = -cd[x] * ((-0.5 * T[x - ld] + 0.5 * T[x + ld]) / P.ds / zs_bot);
                }
                fv[q][e % (n + 1)] = v;
            }
            __syncthreads();
            if (t < 4 && (t == 0 || rat)) {
                for (int j = 0; j < n; j++) {
                    const double xa = P.M.on ? mt(P.M.xr, c0 + j) : 1.0, xb = P.M.on ? mt(P.M.xr, c0 + j + 1) : 1.0;
                    acc = acc + 0.5 * (fv[t][j] * xa + fv[t][j + 1] * xb) * P.dr;
                }
            }
            __syncthreads();
        }
        if (t < 4) ds->integ[11 + t] = acc;
    }
    if (t == 0 && P.RaT != 0.0) {
        auto dz = [&](int i, int kk) { size_t x = IX(L, i, kk); return -0.5 * T[x - ld] + 0.5 * T[x + ld]; };
        const double zt = P.M.on ? mt(P.M.zs, nz) : 1.0, zb = P.M.on ? mt(P.M.zs, 0) : 1.0;
        ds->integ[15] = -(cd[IX(L, 0, nz)] * dz(0, nz)) / P.ds / zt;
        ds->integ[16] = -(cd[IX(L, nx, nz)] * dz(nx, nz)) / P.ds / zt;
        ds->integ[17] = -(cd[IX(L, nx, 0)] * dz(nx, 0)) / P.ds / zb;
        ds->integ[18] = -(cd[IX(L, 0, 0)] * dz(0, 0)) / P.ds / zb;
    }
    // top-row strain maximum (fmax is exact and order-free)
    double smax = -INFINITY;
    for (int i = t; i <= nx; i += blockDim.x) smax = fmax(smax, st[IX(L, i, nz)]);
    for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_down_sync(0xffffffffu, smax, o));
    if ((t & 31) == 0) red[t >> 5] = smax;
    __syncthreads();
    if (t == 0) {
        double m = -INFINITY;
        for (int j = 0; j < (int)(blockDim.x >> 5); j++) m = fmax(m, red[j]);
        ds->strain_max = m;
    }
}
__global__ void k_nempty_stats(Lay L, Range2 r, const int* __restrict__ ne, DevScalars* ds) {
    RANGE_IK(r);
    __shared__ int smin, smax, szero;
    int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if (tid == 0) { smin = 0x7fffffff; smax = -0x7fffffff; szero = 0; }
    __syncthreads();
    if (inr) {
        int v = ne[IX(L, i, k)];
        atomicMin(&smin, v);
        atomicMax(&smax, v);
        if (v == 0) atomicAdd(&szero, 1);
    }
    __syncthreads();
    if (tid == 0) {
        atomicMin(&ds->nempty_min, smin);
        atomicMax(&ds->nempty_max, smax);
        atomicAdd(&ds->empty_cells, szero);
    }
}
__global__ void k_nempty_init(DevScalars* ds) {
    ds->nempty_min = 0x7fffffff;
    ds->nempty_max = -0x7fffffff;
    ds->empty_cells = 0;
}
void launch_stats(cudaStream_t s, const Lay& L, const Phys& P, int kent, const double* T, const double* u,
                  const double* w, const double* conduct, const double* vis, const double* strain,
                  const double* const* Cnew, const int* nempty, double* rows, DevScalars* ds) {
    CPtrs C{};
    for (int j = 0; j < P.ntype && j < TC_MAX_TYPES; j++) C.p[j] = Cnew[j];
    k_stats_rows<<<L.b + 1, kStatThreads, 0, s>>>(L, P, T, u, w, conduct, vis, C, rows); tc_note_launch();
    k_stats_final<<<1, kStatThreads, 0, s>>>(L, P, kent, rows, T, u, w, conduct, strain, ds); tc_note_launch();
    if (P.comp == 1 || P.tracer == 1) {
        Range2 r{0, L.a, 0, L.b};
        k_nempty_init<<<1, 1, 0, s>>>(ds); tc_note_launch();
        k_nempty_stats<<<grid_for(r), dim3(BX, BY), 0, s>>>(L, r, nempty, ds); tc_note_launch();
    }
}
