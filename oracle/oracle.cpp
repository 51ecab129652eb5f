// oracle.cpp -- CPU restatement of the reference hot path (TEST INFRASTRUCTURE).
//
// This file is test infrastructure for the GB300 library, never part of it: only the
// tests, the smoke check and the CPU-baseline leg of the benchmark load the
// shared object built from it.  It restates, routine by routine and in the
// reference's own floating-point operation order, the Fortran/OpenMP code of
// seantrim/tracer_code that the hot path covers:
//
//   iterative_solver.f90 (all)        multigrid, smoother, residual, transfer,
//                                     coarse banded LU, per-level viscosity
//   multigrid_cycle.f90:1-99,131-218  cycle tables, smoothing parameters,
//                                     smoothness measures
//   smoother.f90 (field smoothers)    smoother_vis, smoother_time(_T), vis_space
//   momentum.f90:1-76,532-551         visf, strain rate, compute_velocities
//   composition.f90:669-998           tracers_to_corners, BCs, interpolate,
//                                     compute_derivatives
//   energy.f90 (all)                  energy_time (field T and temperature
//                                     tracers), energy_space, tracer_space,
//                                     extendT, stability
//   basics.f90:112-418, grid.f90, main.f90:350-469 (FD_coefficients)
//
// The reference cannot be compiled here (it is Fortran and no Fortran
// compiler exists on either machine), so this restatement is the oracle.
// Its pinning against the reference's own shipped outputs (Trestart +
// stats.dat + viscosity_smoother.dat, see tests/test_oracle_pins.py) covers
// FD_coefficients, compute_velocities, the strain-rate invariant, stats,
// visf(ivis=3), smoother_vis(level 1), viscosity_gradients, eigR/eigI,
// derivative_eigenvalues, stability_vis_smoother and the level-1 operator;
// the rest (coarse levels, banded LU, tracers, composition, energy_time) is
// "parity unpinned" by reference outputs and is checked by analytic tests.
//
// Third-party arithmetic: the reference calls Intel MKL LAPACK DGBEQU, DGBTRF
// and DGBTRS (iterative_solver.f90:97,117,140,1165), unversioned (Makefile:13).
// They are restated here from the published LAPACK 3.x reference algorithms
// (dgbequ, dgbtf2 unblocked LU with partial pivoting, dgbtrs + dtbsv).
//
// Build: g++ -O2 -ffp-contract=off -fopenmp (see oracle/Makefile).  FP
// contraction must stay off: the reference build (gfortran -O3 -m64 on
// x86-64) has no FMA, and aarch64 GCC contracts by default.

#include "tracer_gpu.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double pii = 3.1415926535897932;  // basics.f90:22

// Fortran-style 2-D array with arbitrary lower bounds, column-major.
struct Arr {
    int i0 = 0, k0 = 0, ni = 0, nk = 0;
    std::vector<double> v;
    void alloc(int ilo, int ihi, int klo, int khi, double fill = 0.0) {
        i0 = ilo; k0 = klo; ni = ihi - ilo + 1; nk = khi - klo + 1;
        v.assign((size_t)ni * nk, fill);
    }
    inline double& operator()(int i, int k) { return v[(size_t)(i - i0) + (size_t)(k - k0) * ni]; }
    inline double operator()(int i, int k) const { return v[(size_t)(i - i0) + (size_t)(k - k0) * ni]; }
    void fill(double x) { std::fill(v.begin(), v.end(), x); }
};
struct IArr {
    int i0 = 0, k0 = 0, ni = 0, nk = 0;
    std::vector<int> v;
    void alloc(int ilo, int ihi, int klo, int khi, int fill = 0) {
        i0 = ilo; k0 = klo; ni = ihi - ilo + 1; nk = khi - klo + 1;
        v.assign((size_t)ni * nk, fill);
    }
    inline int& operator()(int i, int k) { return v[(size_t)(i - i0) + (size_t)(k - k0) * ni]; }
    void fill(int x) { std::fill(v.begin(), v.end(), x); }
};
// 1-D array with lower bound.
struct V1 {
    int lo = 0;
    std::vector<double> v;
    void alloc(int l, int h, double fill = 0.0) { lo = l; v.assign((size_t)(h - l + 1), fill); }
    inline double& operator()(int i) { return v[(size_t)(i - lo)]; }
    inline double operator()(int i) const { return v[(size_t)(i - lo)]; }
};

inline double sq(double x) { return x * x; }  // x**2.d0 folds to x*x in gfortran

// Exact per-volume tracer temperature sums: x -> round-toward-zero(x * 2^64)
// as a 128-bit integer, from the IEEE-754 fields (|x| >= 2^62 saturates,
// NaN and values below 2^-64 count as 0); the sum back to double, rounded
// to nearest once.  The GPU library computes the same integers.
inline __int128 tracer_fixq(double x) {
    uint64_t b;
    std::memcpy(&b, &x, 8);
    const int E = (int)((b >> 52) & 0x7ff);
    if (E == 0x7ff && (b & 0xfffffffffffffULL)) return 0;  // NaN
    const bool neg = (b >> 63) != 0;
    unsigned __int128 v;
    if (E == 0) v = 0;  // zero and subnormals: below 2^-64
    else {
        const uint64_t m = (b & 0xfffffffffffffULL) | (1ULL << 52);  // |x| = m * 2^(E-1075)
        const int sh = E - 1011;                                   // |x| * 2^64 = m * 2^sh
        if (sh > 73 || E == 0x7ff) v = (unsigned __int128)1 << 126;  // |x| >= 2^62
        else if (sh >= 0) v = (unsigned __int128)m << sh;
        else if (sh > -53) v = (unsigned __int128)(m >> (-sh));
        else v = 0;
    }
    return neg ? -(__int128)v : (__int128)v;
}
inline double tracer_fixd(__int128 S) { return std::ldexp((double)S, -64); }

// Scaled derivative eigenvalue bounds (module globals Tr_max ... Trrss_max).
struct EigMax {
    double Tr, Trr, Trrr, Trrrr, Ts, Tss, Tsss, Tssss, Trs, Trrs, Trss, Trrss;
};

struct Oracle {
    tc_params p{};
    std::string err;
    // ---- derived scalars (basics) ----
    int nx = 0, nz = 0, order = 2, span = 2, span1 = 1, span_interp = 1, spanT = 2, Dnumber = 2;
    int grids = 2, nsteps = 0, ngrid_coarse = 0, kl = 0, ku = 0, ntype = 0, comp = 0;
    long ntr = 0;
    double dr = 0, ds = 0, dr2, ds2, dr3, ds3, dr4, ds4, drds, drds2, dr2ds, dr2ds2, dro2, dso2;
    double dist_r = 0, dist_s = 0, Ax = 0, Az = 0;
    double delta_T = 2, delta_T_init = 2;
    double delta_C[TC_MAX_TYPES];
    std::vector<int> multi;  // multi(0:nsteps+1)
    std::vector<int> nx_grid, nz_grid;  // 1-based
    std::vector<double> dr_grid, ds_grid, dr2_grid, ds2_grid, dr3_grid, ds3_grid, dr4_grid, ds4_grid,
        drds_grid, drds2_grid, dr2ds_grid, dr2ds2_grid;
    // ---- FD coefficients ----
    V1 D1, D2, D3, D4;
    Arr Drs, Drss, Drrs, Drrss;
    std::vector<V1> D;  // D(1:Dnumber, -si:si)
    std::vector<double> factorial, dr_power, ds_power;
    double Tr_base = 0, Trr_base = 0, Trrr_base = 0, Trrrr_base = 0, Ts_base = 0, Tss_base = 0,
           Tsss_base = 0, Tssss_base = 0, Trs_base = 0, Trrss_base = 0, Trss_base = 0, Trrs_base = 0;
    // ---- grid ----
    V1 xg, zg, xr, xrr, xrrr, xrrrr, zs, zss, zsss, zssss;
    std::vector<V1> DERxr, DERzs;  // (1:order-1, 0:n): compute_metric_interpolator_derivatives
    // ---- fields ----
    Arr T, SF, Tvis, Tbuoy, u, w, vis, strain, conduct, conduct_r, conduct_s, dts_array;
    std::vector<Arr> Cnew, Cvis, Cbuoy;  // per type (index tt-1)
    std::vector<Arr> dt_vis;             // per level (1-based)
    std::vector<Arr> error, vis_grid, vis_x, vis_z, vis_xx, vis_zz, vis_xz, RHS, dt_stream, ratio;
    std::vector<Arr> vis_gridf, vis_xf, vis_zf, vis_xxf, vis_zzf, vis_xzf;
    Arr residual;
    std::vector<double> res_ref, residual_mag;
    // coarse banded system
    std::vector<double> Mc, Bc, RowB;  // Mc: (2kl+ku+1) x ngrid_coarse column-major, 1-based rows
    std::vector<int> IPIV;
    int ldab = 0;
    // tracers
    std::vector<double> rtr, str, rtr0, str0, rtr1, str1, rtr2, str2;
    std::vector<int> Ttype;
    std::vector<IArr> count_type;  // 0..ntype
    IArr nempty;
    std::vector<Arr> DERr_u, DERr_w;  // per derivative j=1..order-1 : (0:nx, -si:nz+si)
    // temperature tracers (tracer = 1)
    int tracer = 0;
    std::vector<double> Ttr, Ttr0, Ttr1, Ttr2;
    Arr Tratio, Textend, tsa;  // tsa = tracer_space_array (-si:nx+si, -si:nz+si)
    std::vector<Arr> DERr_tracer;
    // tracer repositioning (equalize = 1): the mzran state of each OpenMP
    // thread of the reproduced run, Cinit, and the last equalize.dat row
    int eq_T = 1;
    std::vector<int32_t> sd_i, sd_j, sd_k, sd_n;
    double Cinit[TC_MAX_TYPES] = {};
    long nequalize = 0;
    std::vector<int64_t> eq_row;  // see tco_equalize_row
    // module state
    double time = 0, dt = 0;
    int tstep = 0, kent = 0;
    double mass[TC_MAX_TYPES];
    int n_eta = 0, n_temp = 0, n_comp[TC_MAX_TYPES];
    double eig_fine = 0;
    int Nvis_store = 0, nn_store = 1, smooth_vis = 1;
    int build = 0, scaling = 0, analysis = 0;
    bool uploaded = false;
    int status = TC_OK;  // sticky error from deep routines
    long loop_cap = 100000;

    // =====================================================================
    // setup
    // =====================================================================
    // compute_smoothing_parameters (multigrid_cycle.f90:131-173)
    void compute_smoothing_parameters() {
        if (p.ivis == 0 || p.RaT == 0.0) {
            delta_T = 2.0; delta_T_init = 2.0;
        } else {
            if (p.visT != 1.0) {
                delta_T = std::log(p.delta_visT) / std::log(p.visT);
                delta_T_init = std::log(2.0) / std::log(p.visT);  // delta_visT_init=2.0 (main.f90:65)
            } else {
                delta_T = 2.0; delta_T_init = 2.0;
            }
        }
        for (int i = 0; i < TC_MAX_TYPES; i++) delta_C[i] = 2.0;
        if (p.comp == 1) {
            for (int i = 0; i < p.ntype; i++)
                if (p.conduct_factor[i] != 1.0)
                    delta_C[i] = std::fabs(std::log(p.delta_visC[i]) / std::log(1.0 / p.conduct_factor[i]));
            if (p.ivis == 2)
                for (int i = 0; i < p.ntype; i++)
                    if (p.visC[i] != 1.0) delta_C[i] = std::fabs(std::log(p.delta_visC[i]) / std::log(p.visC[i]));
        }
    }

    // optimize_grid (iterative_solver.f90:1-61)
    static void optimize_grid(int& nx_, int& nz_, int& grids_, int n_points_min) {
        int n_points_max = std::min(nx_, nz_);
        int n_coarse_min = 1, n_coarse_max = grids_ - 1;
        int n_max = n_points_max * (1 << n_coarse_max);
        int nxbig, n_in;
        if (nz_ <= nx_) { nxbig = 1; n_in = nz_; } else { nxbig = 0; n_in = nx_; }
        int n_temp = n_max, n_coarse_temp = 0, n_points_temp = 0;
        for (int n_points = n_points_min; n_points <= n_points_max; n_points++)
            for (int n_coarse = n_coarse_min; n_coarse <= n_coarse_max; n_coarse++) {
                int n = n_points * (1 << n_coarse);
                if (n >= n_in && n < n_temp) { n_temp = n; n_coarse_temp = n_coarse; n_points_temp = n_points; }
            }
        grids_ = n_coarse_temp + 1;
        if (nxbig == 0) nx_ = n_temp; else nz_ = n_temp;
        n_in = (nz_ <= nx_) ? nx_ : nz_;
        // nint(real(n_in)/real(2**n_coarse_temp)) : round half away from zero
        n_points_temp = (int)std::lround((double)n_in / (double)(1 << n_coarse_temp));
        n_temp = n_points_temp * (1 << n_coarse_temp);
        if (nxbig == 0) nz_ = n_temp; else nx_ = n_temp;
    }

    // multigrid_setup (multigrid_cycle.f90:1-99): cycle tables actually selected.
    void multigrid_setup() {
        optimize_grid(nx, nz, grids, p.mingrid);
        std::vector<int> tab;
        if (grids == 2) tab = {1, 2};
        else if (grids == 3) tab = {1, 2, 3, 2, 3, 2};
        else if (grids == 4) tab = {1, 2, 3, 4, 3, 4, 3, 2, 3, 4, 3, 4, 3, 2};
        else if (grids == 5) tab = {1, 2, 3, 4, 5, 4, 5, 4, 3, 4, 5, 4, 3, 2, 3, 4, 5, 4, 3, 4, 5, 4, 5, 4, 3, 2};
        else if (grids == 6)
            tab = {1, 2, 3, 4, 5, 6, 5, 6, 5, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 3,
                   2, 3, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 5, 6, 5, 6, 5, 4, 3, 2};
        nsteps = (int)tab.size();
        multi.assign(nsteps + 2, 0);
        for (int i = 0; i < nsteps; i++) multi[i + 1] = tab[i];
        multi[0] = multi[nsteps];
        multi[nsteps + 1] = multi[1];
        residual_mag.assign(nsteps + 1, 0.0);
    }

    // compute_factorials (basics.f90:405-418)
    void compute_factorials() {
        factorial.assign(Dnumber + 1, 0.0); dr_power.assign(Dnumber + 1, 0.0); ds_power.assign(Dnumber + 1, 0.0);
        factorial[0] = 1.0; dr_power[0] = 1.0; ds_power[0] = 1.0;
        for (int j = 1; j <= Dnumber; j++) {
            factorial[j] = (double)j * factorial[j - 1];
            dr_power[j] = std::pow(dr, (double)j);
            ds_power[j] = std::pow(ds, (double)j);
        }
    }

    static double pw(double x, int n) {  // x**n.d0 as gfortran evaluates it
        if (n == 2) return x * x;
        if (n == 1) return x;
        return std::pow(x, (double)n);
    }

    // compute_basics (basics.f90:112-214) minus the PRNG seeds (equalize only).
    void compute_basics() {
        Dnumber = order;
        span1 = order / 2;
        span = order / 2 + 1;
        span_interp = (order + Dnumber - 2) / 2;
        spanT = span_interp + span1;
        dr = p.aspect / (double)nx;
        ds = 1.0 / (double)nz;
        dr2 = pw(dr, 2); ds2 = pw(ds, 2); dr3 = pw(dr, 3); ds3 = pw(ds, 3); dr4 = pw(dr, 4); ds4 = pw(ds, 4);
        drds = dr * ds; drds2 = dr * ds2; dr2ds = dr2 * ds; dr2ds2 = dr2 * ds2;
        dro2 = 0.5 * dr; dso2 = 0.5 * ds;
        Ax = std::pow(std::atan(p.spaceX * 0.5) - std::atan(p.spaceX * (-0.5)), -1.0);
        Az = std::pow(std::atan(p.spaceZ * 0.5) - std::atan(p.spaceZ * (-0.5)), -1.0);
        compute_factorials();
        ntr = (p.comp == 1 || p.tracer == 1) ? (long)(nx + 1) * (nz + 1) * p.tpc : 0;
        dist_r = p.dist_factor * dr;
        dist_s = p.dist_factor * ds;
        nx_grid.assign(grids + 1, 0); nz_grid.assign(grids + 1, 0);
        auto z = [&](std::vector<double>& a) { a.assign(grids + 1, 0.0); };
        z(dr_grid); z(ds_grid); z(dr2_grid); z(ds2_grid); z(dr3_grid); z(ds3_grid); z(dr4_grid); z(ds4_grid);
        z(drds_grid); z(drds2_grid); z(dr2ds_grid); z(dr2ds2_grid);
        for (int j = 1; j <= grids; j++) {
            nx_grid[j] = nx / (1 << (j - 1));
            nz_grid[j] = nz / (1 << (j - 1));
            dr_grid[j] = p.aspect / (double)nx_grid[j];
            ds_grid[j] = 1.0 / (double)nz_grid[j];
            dr2_grid[j] = pw(dr_grid[j], 2); ds2_grid[j] = pw(ds_grid[j], 2);
            dr3_grid[j] = pw(dr_grid[j], 3); ds3_grid[j] = pw(ds_grid[j], 3);
            dr4_grid[j] = pw(dr_grid[j], 4); ds4_grid[j] = pw(ds_grid[j], 4);
            drds_grid[j] = dr_grid[j] * ds_grid[j];
            drds2_grid[j] = dr_grid[j] * ds2_grid[j];
            dr2ds_grid[j] = dr2_grid[j] * ds_grid[j];
            dr2ds2_grid[j] = dr2_grid[j] * ds2_grid[j];
        }
        ngrid_coarse = (nx_grid[grids] + 1) * (nz_grid[grids] + 1);
    }

    void storage() {
        int s = span, si = span_interp;
        T.alloc(-s, nx + s, -s, nz + s); SF.alloc(-s, nx + s, -s, nz + s);
        Tvis.alloc(-s, nx + s, -s, nz + s); Tbuoy.alloc(-s, nx + s, -s, nz + s);
        vis.alloc(-s, nx + s, -s, nz + s); strain.alloc(-s, nx + s, -s, nz + s);
        u.alloc(-si, nx + si, -si, nz + si); w.alloc(-si, nx + si, -si, nz + si);
        conduct.alloc(-spanT, nx + spanT, -spanT, nz + spanT);
        conduct_r.alloc(-si, nx + si, -si, nz + si); conduct_s.alloc(-si, nx + si, -si, nz + si);
        dts_array.alloc(0, nx, 0, nz);
        xg.alloc(-(s + si), nx + s + si); zg.alloc(-(s + si), nz + s + si);
        xr.alloc(-si, nx + si); xrr.alloc(-si, nx + si); xrrr.alloc(0, nx); xrrrr.alloc(0, nx);
        zs.alloc(-si, nz + si); zss.alloc(-si, nz + si); zsss.alloc(0, nz); zssss.alloc(0, nz);
        DERxr.assign(order, V1()); DERzs.assign(order, V1());
        for (int j = 1; j <= order - 1; j++) { DERxr[j].alloc(0, nx); DERzs[j].alloc(0, nz); }
        ntype = p.comp == 1 ? p.ntype : 0;
        Cnew.assign(ntype, Arr()); Cvis.assign(ntype, Arr()); Cbuoy.assign(ntype, Arr());
        for (int t = 0; t < ntype; t++) {
            Cnew[t].alloc(-s, nx + s, -s, nz + s); Cvis[t].alloc(-s, nx + s, -s, nz + s);
            Cbuoy[t].alloc(-s, nx + s, -s, nz + s);
        }
        if (p.comp == 1 || p.tracer == 1) {
            count_type.assign(ntype + 1, IArr());
            for (int t = 0; t <= ntype; t++) count_type[t].alloc(-s, nx + s, -s, nz + s);
            nempty.alloc(-s, nx + s, -s, nz + s);
            rtr.assign(ntr, 0); str.assign(ntr, 0); rtr0.assign(ntr, 0); str0.assign(ntr, 0);
            rtr1.assign(ntr, 0); str1.assign(ntr, 0);
            if (p.torder > 2) { rtr2.assign(ntr, 0); str2.assign(ntr, 0); }
            Ttype.assign(ntr, 0);
            DERr_u.assign(order, Arr()); DERr_w.assign(order, Arr());
            for (int j = 1; j <= order - 1; j++) {
                DERr_u[j].alloc(0, nx, -si, nz + si); DERr_w[j].alloc(0, nx, -si, nz + si);
            }
            if (p.tracer == 1) {
                Ttr.assign(ntr, 0); Ttr0.assign(ntr, 0); Ttr1.assign(ntr, 0);
                if (p.torder > 2) Ttr2.assign(ntr, 0);
                Tratio.alloc(-s, nx + s, -s, nz + s);
                Textend.alloc(-spanT, nx + spanT, -spanT, nz + spanT);
                tsa.alloc(-si, nx + si, -si, nz + si);
                DERr_tracer.assign(order, Arr());
                for (int j = 1; j <= order - 1; j++) DERr_tracer[j].alloc(0, nx, -si, nz + si);
            }
        }
        dt_vis.assign(grids + 1, Arr());
        error.assign(grids + 1, Arr()); vis_grid.assign(grids + 1, Arr()); RHS.assign(grids + 1, Arr());
        vis_x.assign(grids + 1, Arr()); vis_z.assign(grids + 1, Arr()); vis_xx.assign(grids + 1, Arr());
        vis_zz.assign(grids + 1, Arr()); vis_xz.assign(grids + 1, Arr()); dt_stream.assign(grids + 1, Arr());
        ratio.assign(grids + 1, Arr());
        vis_gridf.assign(grids + 1, Arr()); vis_xf.assign(grids + 1, Arr()); vis_zf.assign(grids + 1, Arr());
        vis_xxf.assign(grids + 1, Arr()); vis_zzf.assign(grids + 1, Arr()); vis_xzf.assign(grids + 1, Arr());
        for (int l = 1; l <= grids; l++) {
            int a = nx_grid[l], b = nz_grid[l];
            dt_vis[l].alloc(0, a, 0, b);
            error[l].alloc(-s, a + s, -s, b + s); vis_grid[l].alloc(-s, a + s, -s, b + s);
            RHS[l].alloc(1, a - 1, 1, b - 1);
            vis_x[l].alloc(1, a - 1, 1, b - 1); vis_z[l].alloc(1, a - 1, 1, b - 1);
            vis_xx[l].alloc(1, a - 1, 1, b - 1); vis_zz[l].alloc(1, a - 1, 1, b - 1);
            vis_xz[l].alloc(1, a - 1, 1, b - 1); dt_stream[l].alloc(1, a - 1, 1, b - 1);
            ratio[l].alloc(1, a - 1, 1, b - 1, 0.0);
        }
        residual.alloc(1, nx - 1, 1, nz - 1);
        res_ref.assign(grids + 1, 0.0);
    }

    // FD_coefficients (main.f90:350-469): Fornberg's recurrence.
    void FD_coefficients() {
        int bigM = std::max(4, Dnumber);
        int bigN = order + bigM - 2;
        std::vector<double> a(bigN + 1, 0.0);
        // delta(-1:bigM, 0:bigN, 0:bigN)
        auto idx = [&](int m, int n, int i) { return (size_t)(m + 1) + (size_t)(bigM + 2) * ((size_t)n + (size_t)(bigN + 1) * i); };
        std::vector<double> delta((size_t)(bigM + 2) * (bigN + 1) * (bigN + 1), 0.0);
        double x0 = 0.0;
        a[0] = 0.0;
        int k = 1;
        for (int i = 1; i <= bigN; i += 2) {
            a[i] = (double)k;
            if (i + 1 <= bigN) a[i + 1] = -(double)k;
            k++;
        }
        delta[idx(0, 0, 0)] = 1.0;
        double c1 = 1.0;
        for (int n = 1; n <= bigN; n++) {
            double c2 = 1.0;
            for (int i = 0; i <= n - 1; i++) {
                double c3 = a[n] - a[i];
                c2 = c2 * c3;
                if (n <= bigM) delta[idx(n, n - 1, i)] = 0.0;
                for (int m = 0; m <= std::min(n, bigM); m++)
                    delta[idx(m, n, i)] = ((a[n] - x0) * delta[idx(m, n - 1, i)] - (double)m * delta[idx(m - 1, n - 1, i)]) / c3;
            }
            for (int m = 0; m <= std::min(n, bigM); m++)
                delta[idx(m, n, n)] = (c1 / c2) * ((double)m * delta[idx(m - 1, n - 1, n - 1)] - (a[n - 1] - x0) * delta[idx(m, n - 1, n - 1)]);
            c1 = c2;
        }
        D1.alloc(-span, span); D2.alloc(-span, span); D3.alloc(-span, span); D4.alloc(-span, span);
        D1(0) = delta[idx(1, order, 0)];
        D2(0) = delta[idx(2, order, 0)];
        k = 1;
        for (int i = 1; i <= order; i += 2) {
            D1(k) = delta[idx(1, order, i)]; D1(-k) = delta[idx(1, order, i + 1)];
            D2(k) = delta[idx(2, order, i)]; D2(-k) = delta[idx(2, order, i + 1)];
            k++;
        }
        D.assign(Dnumber + 1, V1());
        for (int m = 1; m <= Dnumber; m++) D[m].alloc(-span_interp, span_interp, 0.0);
        for (int m = 2; m <= Dnumber; m += 2) {
            D[m - 1](0) = delta[idx(m - 1, order + m - 2, 0)];
            D[m](0) = delta[idx(m, order + m - 2, 0)];
            k = 1;
            for (int i = 1; i <= order + m - 2; i += 2) {
                D[m - 1](k) = delta[idx(m - 1, order + m - 2, i)];
                D[m - 1](-k) = delta[idx(m - 1, order + m - 2, i + 1)];
                D[m](k) = delta[idx(m, order + m - 2, i)];
                D[m](-k) = delta[idx(m, order + m - 2, i + 1)];
                k++;
            }
        }
        for (int m = 1; m <= Dnumber; m += 2) {
            D[m](0) = 0.0;
            for (int i = 1; i <= span_interp; i++) {
                D[m](i) = -D[m](-i);
                D[m + 1](i) = D[m + 1](-i);
            }
        }
        D3(0) = delta[idx(3, order + 2, 0)];
        D4(0) = delta[idx(4, order + 2, 0)];
        k = 1;
        for (int i = 1; i <= order + 2; i += 2) {
            D3(k) = delta[idx(3, order + 2, i)]; D3(-k) = delta[idx(3, order + 2, i + 1)];
            D4(k) = delta[idx(4, order + 2, i)]; D4(-k) = delta[idx(4, order + 2, i + 1)];
            k++;
        }
        D1(0) = 0.0; D3(0) = 0.0;
        for (int i = 1; i <= span; i++) {
            D1(i) = -D1(-i); D2(i) = D2(-i); D3(i) = -D3(-i); D4(i) = D4(-i);
        }
        Drs.alloc(-span, span, -span, span); Drss.alloc(-span, span, -span, span);
        Drrs.alloc(-span, span, -span, span); Drrss.alloc(-span, span, -span, span);
        for (int kk = -span1; kk <= span1; kk++)
            for (int i = -span1; i <= span1; i++) {
                Drs(i, kk) = D1(kk) * D1(i);
                Drss(i, kk) = D2(kk) * D1(i);
                Drrs(i, kk) = D1(kk) * D2(i);
                Drrss(i, kk) = D2(kk) * D2(i);
            }
    }

    // xgrid / zgrid (grid.f90:1-35)
    double xgrid(double r) const {
        if (p.gridX == 1) return p.aspect * (Ax * std::atan(p.spaceX * (r / p.aspect - 0.5)) + 0.5);
        return r;
    }
    double zgrid(double s) const {
        if (p.gridZ == 1) return Az * std::atan(p.spaceZ * (s - 0.5)) + 0.5;
        if (p.gridZ == 2) {
            double dzin = (1.0 - 2.0 * p.thickness) / (double)(nz - 2 * p.nbound + 2);
            double s1 = (double)(p.nbound - 1) * ds;
            double s2 = 1.0 - s1;
            if (s < s1) return (p.thickness / (std::exp(p.spaceZ * s1) - 1.0)) * (std::exp(p.spaceZ * s) - 1.0);
            if (s > s2) return 1.0 - (p.thickness / (std::exp(p.spaceZ * s1) - 1.0)) * (std::exp(-p.spaceZ * (s - 1.0)) - 1.0);
            return p.thickness + (s - s1) * dzin / ds;
        }
        return s;
    }

    // build_grid (grid.f90:37-147), restart=0 coordinates.
    void build_grid() {
        for (int i = 0; i <= nx; i++) xg(i) = xgrid(dr * (double)i);
        for (int k = 0; k <= nz; k++) zg(k) = zgrid(ds * (double)k);
        for (int i = 1; i <= span + span_interp; i++) {
            xg(-i) = -xg(i);
            xg(nx + i) = p.aspect - xg(nx - i) + p.aspect;
        }
        for (int k = 1; k <= span + span_interp; k++) {
            zg(-k) = -zg(k);
            zg(nz + k) = 1.0 - zg(nz - k) + 1.0;
        }
        xg(0) = 0.0; zg(0) = 0.0; xg(nx) = p.aspect; zg(nz) = 1.0;
        auto dotD = [&](const V1& Dc, int sp, const V1& f, int c) {
            double s = 0.0;
            for (int j = -sp; j <= sp; j++) s = s + Dc(j) * f(c + j);
            return s;
        };
        for (int i = 0; i <= nx; i++) {
            if (p.gridX != 0) { xrrr(i) = dotD(D3, span, xg, i) / dr3; xrrrr(i) = dotD(D4, span, xg, i) / dr4; }
            else { xrrr(i) = 0.0; xrrrr(i) = 0.0; }
        }
        for (int i = -span_interp; i <= nx + span_interp; i++) {
            if (p.gridX != 0) { xr(i) = dotD(D1, span1, xg, i) / dr; xrr(i) = dotD(D2, span1, xg, i) / dr2; }
            else { xr(i) = 1.0; xrr(i) = 0.0; }
        }
        for (int k = 0; k <= nz; k++) {
            if (p.gridZ != 0) { zsss(k) = dotD(D3, span, zg, k) / ds3; zssss(k) = dotD(D4, span, zg, k) / ds4; }
            else { zsss(k) = 0.0; zssss(k) = 0.0; }
        }
        for (int k = -span_interp; k <= nz + span_interp; k++) {
            if (p.gridZ != 0) { zs(k) = dotD(D1, span1, zg, k) / ds; zss(k) = dotD(D2, span1, zg, k) / ds2; }
            else { zs(k) = 1.0; zss(k) = 0.0; }
        }
        // compute_metric_interpolator_derivatives (composition.f90:921-936);
        // the reference calls it for comp = 1 only (grid.f90:146), here for
        // every case so that temperature tracers read defined values
        for (int jj = 1; jj <= order - 1; jj++) {
            for (int i = 0; i <= nx; i++) DERxr[jj](i) = dotD(D[jj], span_interp, xr, i) / dr_power[jj];
            for (int k = 0; k <= nz; k++) DERzs[jj](k) = dotD(D[jj], span_interp, zs, k) / ds_power[jj];
        }
    }
    // interpolate_xr / interpolate_zs (composition.f90:938-998): the metric at
    // a tracer position by the forward or backward Taylor step of interpolate
    double interpolate_xr(double r) const {
        if (p.gridX == 0) return 1.0;
        const int i = (int)(r / dr);
        double hr = r - (double)i * dr;
        double x;
        if (hr <= dro2) {
            x = xr(i);
            for (int j = 1; j <= order - 1; j++) x = x + DERxr[j](i) * (pw(hr, j) / factorial[j]);
        } else {
            hr = dr - hr;
            x = xr(i + 1);
            for (int j = 1; j <= order - 1; j++) x = x + DERxr[j](i + 1) * (pw(-hr, j) / factorial[j]);
        }
        return x;
    }
    double interpolate_zs(double s) const {
        if (p.gridZ == 0) return 1.0;
        const int k = (int)(s / ds);
        double hs = s - (double)k * ds;
        double z;
        if (hs <= dso2) {
            z = zs(k);
            for (int j = 1; j <= order - 1; j++) z = z + DERzs[j](k) * (pw(hs, j) / factorial[j]);
        } else {
            hs = ds - hs;
            z = zs(k + 1);
            for (int j = 1; j <= order - 1; j++) z = z + DERzs[j](k + 1) * (pw(-hs, j) / factorial[j]);
        }
        return z;
    }
    // the tracer's computational velocity at (r, s): u / xr and w / zs with
    // the interpolated metrics on stretched axes (energy.f90:194-203)
    double tr_vel(double r, double s) const {
        double t = interpolate(r, s, DERr_u, u);
        if (p.gridX != 0) t = t / interpolate_xr(r);
        return t;
    }
    double ts_vel(double r, double s) const {
        double t = interpolate(r, s, DERr_w, w);
        if (p.gridZ != 0) t = t / interpolate_zs(s);
        return t;
    }

    // derivative_eigenvalues (energy.f90:501-598).  T_test uses CMPLX without
    // KIND, i.e. each factor is rounded to single precision and multiplied in
    // single precision before widening (energy.f90:597).
    void derivative_eigenvalues() {
        const int n_angle = (1 << 11) + 1;
        const double d_angle = 2.0 * pii / (double)(n_angle - 1);
        // 1-D factors (float-rounded cos/sin of kr*j) per angle and offset.
        int sp = span;
        std::vector<std::complex<float>> fac((size_t)n_angle * (2 * sp + 1));
        for (int a = 1; a <= n_angle; a++) {
            double kr = (double)(a - 1) * d_angle;
            for (int j = -sp; j <= sp; j++) {
                double r = (double)j;
                fac[(size_t)(a - 1) * (2 * sp + 1) + (j + sp)] =
                    std::complex<float>((float)std::cos(kr * r), (float)std::sin(kr * r));
            }
        }
        auto Ttest = [&](int j, int jj, int a, int a2) -> std::complex<double> {
            std::complex<float> x = fac[(size_t)(a - 1) * (2 * sp + 1) + (j + sp)];
            std::complex<float> y = fac[(size_t)(a2 - 1) * (2 * sp + 1) + (jj + sp)];
            // complex*4 product, computed component-wise in single precision
            volatile float ac = x.real() * y.real(), bd = x.imag() * y.imag();
            volatile float ad = x.real() * y.imag(), bc = x.imag() * y.real();
            float re = ac - bd, im = ad + bc;
            return std::complex<double>((double)re, (double)im);
        };
        double Tr_max = 0, Trr_max = 0, Trrr_max = 0, Trrrr_max = 0, Trs_max = 0, Trrs_max = 0, Trrss_max = 0;
#pragma omp parallel for reduction(max : Tr_max, Trr_max, Trrr_max, Trrrr_max, Trs_max, Trrs_max, Trrss_max) schedule(static)
        for (int angle = 1; angle <= n_angle; angle++) {
            // ks = 0 -> angle2 index 1
            std::complex<double> Tr(0, 0), Trr(0, 0), Trrr(0, 0), Trrrr(0, 0), temp;
            for (int j = -span1; j <= span1; j++) {
                temp = Ttest(j, 0, angle, 1);
                Tr = Tr + D1(j) * temp;
                Trr = Trr + D2(j) * temp;
            }
            for (int j = -span; j <= span; j++) {
                temp = Ttest(j, 0, angle, 1);
                Trrr = Trrr + D3(j) * temp;
                Trrrr = Trrrr + D4(j) * temp;
            }
            std::complex<double> c0 = Ttest(0, 0, angle, 1);  // == (1,0)
            Tr = Tr / c0; Trr = Trr / c0; Trrr = Trrr / c0; Trrrr = Trrrr / c0;
            if (std::fabs(Tr.imag()) > Tr_max) Tr_max = std::fabs(Tr.imag());
            if (std::fabs(Trr.real()) > Trr_max) Trr_max = std::fabs(Trr.real());
            if (std::fabs(Trrr.imag()) > Trrr_max) Trrr_max = std::fabs(Trrr.imag());
            if (std::fabs(Trrrr.real()) > Trrrr_max) Trrrr_max = std::fabs(Trrrr.real());
            for (int angle2 = 1; angle2 <= n_angle; angle2++) {
                std::complex<double> Trs(0, 0), Trrs(0, 0), Trrss(0, 0);
                for (int j = -span1; j <= span1; j++)
                    for (int jj = -span1; jj <= span1; jj++) {
                        std::complex<double> t = Ttest(j, jj, angle, angle2);
                        Trs = Trs + Drs(j, jj) * t;
                        Trrs = Trrs + Drrs(j, jj) * t;
                        Trrss = Trrss + Drrss(j, jj) * t;
                    }
                if (std::fabs(Trs.real()) > Trs_max) Trs_max = std::fabs(Trs.real());
                if (std::fabs(Trrs.imag()) > Trrs_max) Trrs_max = std::fabs(Trrs.imag());
                if (std::fabs(Trrss.real()) > Trrss_max) Trrss_max = std::fabs(Trrss.real());
            }
        }
        Tr_base = Tr_max; Trr_base = Trr_max; Trrr_base = Trrr_max; Trrrr_base = Trrrr_max;
        Ts_base = 0; Tss_base = 0; Tsss_base = 0; Tssss_base = 0;  // never set in the reference loop
        Trs_base = Trs_max; Trrss_base = Trrss_max; Trss_base = 0.0; Trrs_base = Trrs_max;
    }

    EigMax scaled_eig(int level) const {  // test_eigenvalues/iterate_local_time_steps preamble
        EigMax e;
        e.Ts = Tr_base / ds_grid[level];
        e.Tss = -Trr_base / ds2_grid[level];
        e.Tsss = Trrr_base / ds3_grid[level];
        e.Tssss = Trrrr_base / ds4_grid[level];
        e.Tr = Tr_base / dr_grid[level];
        e.Trr = -Trr_base / dr2_grid[level];
        e.Trrr = Trrr_base / dr3_grid[level];
        e.Trrrr = Trrrr_base / dr4_grid[level];
        e.Trs = -Trs_base / drds_grid[level];
        e.Trrss = Trrss_base / dr2ds2_grid[level];
        e.Trss = Trrs_base / drds2_grid[level];
        e.Trrs = Trrs_base / dr2ds_grid[level];
        return e;
    }

    // stability_RK4_smoother (smoother.f90:423-462 in the cat numbering: :523-562)
    void stability_RK4_smoother() {
        double Ts_max = Tr_base / ds, Tss_max = -Trr_base / ds2, Tr_max = Tr_base / dr, Trr_max = -Trr_base / dr2;
#pragma omp parallel for schedule(static)
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                double eR = std::fabs(Trr_max / sq(xr(i))) + std::fabs(Tss_max / sq(zs(k)));
                double eI = std::fabs(xrr(i) / std::pow(xr(i), 3.0)) * Tr_max + std::fabs(zss(k) / std::pow(zs(k), 3.0)) * Ts_max;
                dts_array(i, k) = 2.0 * eR / (sq(eR) + sq(eI));
            }
    }

    // stability_vis_smoother (smoother.f90:465-508)
    void stability_vis_smoother(int level) {
        double Ts_max = Tr_base / ds_grid[level], Tss_max = -Trr_base / ds2_grid[level];
        double Tr_max = Tr_base / dr_grid[level], Trr_max = -Trr_base / dr2_grid[level];
        int f = 1 << (level - 1);
        for (int i = 0; i <= nx_grid[level]; i++)
            for (int k = 1; k <= nz_grid[level] - 1; k++) {
                int i1 = i * f, k1 = k * f;
                double eR = std::fabs(Trr_max / sq(xr(i1))) + std::fabs(Tss_max / sq(zs(k1)));
                double eI = std::fabs(xrr(i1) / std::pow(xr(i1), 3.0)) * Tr_max + std::fabs(zss(k1) / std::pow(zs(k1), 3.0)) * Ts_max;
                dt_vis[level](i, k) = 2.0 * eR / (sq(eR) + sq(eI));
            }
    }

    int create(const tc_params* in) {
        p = *in;
        if (p.order != 2 && p.order != 4) return TC_ERR_UNSUPPORTED;
        if (p.grids < 2 || p.grids > 6) return TC_ERR_ARG;
        if (p.comp == 1 && (p.ntype < 1 || p.ntype > TC_MAX_TYPES)) return TC_ERR_ARG;
        if (p.tracer != 0 && p.tracer != 1) return TC_ERR_ARG;
        if (p.iterate_order != 1) return TC_ERR_UNSUPPORTED;
        if (p.torder != 2 && p.torder != 4) return TC_ERR_UNSUPPORTED;
        order = p.order;
        nx = p.nx; nz = p.nz; grids = p.grids;
        comp = p.comp;
        tracer = p.tracer;
        if (p.equalize != 0 && p.equalize != 1) return TC_ERR_ARG;
        if (p.equalize == 1 && p.comp == 0 && p.tracer == 0) return TC_ERR_ARG;
        eq_T = (p.equalize_threads > 0) ? p.equalize_threads : 1;
        if (eq_T > 1024) return TC_ERR_ARG;
        seed_ranks();
        compute_smoothing_parameters();
        multigrid_setup();
        compute_basics();
        storage();
        FD_coefficients();
        analysis = 1;
        Compute_Matrix_coarse();
        analysis = 0;
        ldab = 2 * kl + ku + 1;
        Mc.assign((size_t)ldab * ngrid_coarse, 0.0);
        Bc.assign(ngrid_coarse + 1, 0.0); RowB.assign(ngrid_coarse + 1, 0.0); IPIV.assign(ngrid_coarse + 1, 0);
        build = 0; scaling = 0;
        smooth_vis = 1;
        build_grid();
        derivative_eigenvalues();
        stability_RK4_smoother();
        for (int l = 1; l <= grids; l++) stability_vis_smoother(l);
        for (int t = 0; t < TC_MAX_TYPES; t++) { mass[t] = 0; n_comp[t] = 0; }
        return TC_OK;
    }

    // =====================================================================
    // small stencil helpers (dot_product / sum in the reference's order)
    // =====================================================================
    inline double dotx(const V1& Dc, int sp, const Arr& f, int i, int k) const {
        double s = 0.0;
        for (int j = -sp; j <= sp; j++) s = s + Dc(j) * f(i + j, k);
        return s;
    }
    inline double dotz(const V1& Dc, int sp, const Arr& f, int i, int k) const {
        double s = 0.0;
        for (int j = -sp; j <= sp; j++) s = s + Dc(j) * f(i, k + j);
        return s;
    }
    inline double sum2(const Arr& Dm, const Arr& f, int i, int k) const {
        double s = 0.0;
        for (int dk = -span1; dk <= span1; dk++)
            for (int di = -span1; di <= span1; di++) s = s + Dm(di, dk) * f(i + di, k + dk);
        return s;
    }

    // =====================================================================
    // boundary conditions
    // =====================================================================
    // enforceBCs (energy.f90:455-475)
    void enforceBCs(Arr& T0) {
        for (int i = 1; i <= span; i++)
            for (int k = 0; k <= nz; k++) { T0(-i, k) = T0(i, k); T0(nx + i, k) = T0(nx - i, k); }
        for (int k = 1; k <= span; k++)
            for (int i = -span; i <= nx + span; i++) {
                if (p.Tbot == 0) T0(i, -k) = -(T0(i, k) - 1.0) + 1.0;
                else T0(i, -k) = T0(i, k);
                T0(i, nz + k) = -T0(i, nz - k);
            }
        for (int i = -span; i <= nx + span; i++) {
            if (p.Tbot == 0) T0(i, 0) = 1.0;
            T0(i, nz) = 0.0;
        }
    }
    // enforceBCs_comp (composition.f90:792-803): the four statements run inside
    // one loop over i, so corner ghosts take partly stale values (kept).
    void enforceBCs_comp(Arr& C0) {
        for (int i = 1; i <= span; i++) {
            for (int k = 0; k <= nz; k++) { C0(-i, k) = C0(i, k); C0(nx + i, k) = C0(nx - i, k); }
            for (int ii = -span; ii <= nx + span; ii++) { C0(ii, -i) = C0(ii, i); C0(ii, nz + i) = C0(ii, nz - i); }
        }
    }
    // enforceBCs_stream (iterative_solver.f90:965-989)
    void enforceBCs_stream(int level, Arr& S0) {
        int a = nx_grid[level], b = nz_grid[level];
        for (int k = -span; k <= b + span; k++) { S0(0, k) = 0.0; S0(a, k) = 0.0; }
        for (int i = -span; i <= a + span; i++) { S0(i, 0) = 0.0; S0(i, b) = 0.0; }
        for (int i = 1; i <= span; i++)
            for (int k = 0; k <= b; k++) { S0(-i, k) = -S0(i, k); S0(a + i, k) = -S0(a - i, k); }
        if (p.Vbc == 1) {
            for (int i = 1; i <= span; i++)
                for (int ii = -span; ii <= a + span; ii++) { S0(ii, -i) = S0(ii, i); S0(ii, b + i) = S0(ii, b - i); }
        } else if (p.Vbc == 0) {
            for (int i = 1; i <= span; i++)
                for (int ii = -span; ii <= a + span; ii++) { S0(ii, -i) = -S0(ii, i); S0(ii, b + i) = -S0(ii, b - i); }
        }
    }
    // velocityBCs (composition.f90:806-836)
    void velocityBCs() {
        int si = span_interp;
        for (int i = 1; i <= si; i++) {
            for (int k = 0; k <= nz; k++) { w(-i, k) = w(i, k); w(nx + i, k) = w(nx - i, k); }
            for (int ii = 0; ii <= nx; ii++) {
                if (p.Vbc == 0) { u(ii, -i) = u(ii, i); u(ii, nz + i) = u(ii, nz - i); }
                else if (p.Vbc == 1) { u(ii, -i) = -u(ii, i); u(ii, nz + i) = -u(ii, nz - i); }
            }
        }
        for (int k = 1; k <= si; k++) {
            for (int i = -si; i <= nx + si; i++) { w(i, -k) = -w(i, k); w(i, nz + k) = -w(i, nz - k); }
            for (int kk = -si; kk <= nz + si; kk++) { u(-k, kk) = -u(k, kk); u(nx + k, kk) = -u(nx - k, kk); }
        }
        for (int k = -si; k <= nz + si; k++) { u(0, k) = 0.0; u(nx, k) = 0.0; }
        for (int i = -si; i <= nx + si; i++) { w(i, 0) = 0.0; w(i, nz) = 0.0; }
        if (p.Vbc == 1)
            for (int i = -si; i <= nx + si; i++) { u(i, 0) = 0.0; u(i, nz) = 0.0; }
    }
    // viscosityBCs_initialize / viscosityBCs (iterative_solver.f90:379-453)
    void viscosity_bcs(int level, bool initialize) {
        Arr& V = vis_grid[level];
        int a = nx_grid[level], b = nz_grid[level];
        if (level > 1) {
            Arr& F = vis_grid[level - 1];
            if (initialize)
                for (int k = 1; k <= b - 1; k++) { V(0, k) = F(0, 2 * k); V(a, k) = F(nx_grid[level - 1], 2 * k); }
            for (int i = 0; i <= a; i++) { V(i, 0) = F(2 * i, 0); V(i, b) = F(2 * i, nz_grid[level - 1]); }
        }
        for (int i = 1; i <= span; i++)
            for (int k = 0; k <= b; k++) { V(-i, k) = V(i, k); V(a + i, k) = V(a - i, k); }
        double vT2 = sq(p.visT);
        if (p.RaT != 0.0) {
            for (int k = 1; k <= span; k++)
                for (int i = -span; i <= a + span; i++) {
                    V(i, -k) = 1.0 / V(i, k) / vT2;
                    V(i, b + k) = 1.0 / V(i, b - k);
                }
        } else {
            for (int k = 1; k <= span; k++)
                for (int i = -span; i <= a + span; i++) { V(i, -k) = V(i, k); V(i, b + k) = V(i, b - k); }
        }
    }
    // load_conductivity_array (energy.f90:31-58)
    void load_conductivity_array() {
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                double c = 1.0;
                if (comp != 0)
                    for (int j = 0; j < ntype; j++) c = std::exp(-Cvis[j](i, k) * std::log(1.0 / p.conduct_factor[j]));
                conduct(i, k) = c;
            }
        for (int i = 1; i <= spanT; i++)
            for (int k = 0; k <= nz; k++) { conduct(-i, k) = conduct(i, k); conduct(nx + i, k) = conduct(nx - i, k); }
        for (int k = 1; k <= spanT; k++)
            for (int i = -spanT; i <= nx + spanT; i++) { conduct(i, -k) = conduct(i, k); conduct(i, nz + k) = conduct(i, nz - k); }
        for (int i = -span_interp; i <= nx + span_interp; i++)
            for (int k = -span_interp; k <= nz + span_interp; k++) {
                conduct_r(i, k) = dotx(D1, span1, conduct, i, k) / dr;
                conduct_s(i, k) = dotz(D1, span1, conduct, i, k) / ds;
            }
    }

    // =====================================================================
    // field smoothers
    // =====================================================================
    // smoothness (multigrid_cycle.f90:175-195)
    double smoothness(const Arr& T0) const {
        double diff = 0.0;
#pragma omp parallel for reduction(max : diff) schedule(static)
        for (int i = 0; i <= nx - 1; i++)
            for (int k = 1; k <= nz - 1; k++) {
                double c = T0(i, k);
                double a1 = std::fabs(T0(i, k - 1) - c), a2 = std::fabs(T0(i + 1, k - 1) - c);
                double a3 = std::fabs(T0(i + 1, k) - c), a4 = std::fabs(T0(i, k + 1) - c);
                double a5 = std::fabs(T0(i + 1, k + 1) - c);
                double a = std::max(std::max(std::max(std::max(a1, a2), a3), a4), a5);
                if (a > diff) diff = a;
            }
        return diff;
    }
    // smoother_space (smoother.f90:122-140)
    inline double smoother_space(int i, int k, const Arr& T0) const {
        double Tr = dotx(D1, span1, T0, i, k) / dr, Ts = dotz(D1, span1, T0, i, k) / ds;
        double Trr = dotx(D2, span1, T0, i, k) / dr2, Tss = dotz(D2, span1, T0, i, k) / ds2;
        double Tx = Tr / xr(i), Tz = Ts / zs(k);
        double Txx = (Trr - Tx * xrr(i)) / sq(xr(i));
        double Tzz = (Tss - Tz * zss(k)) / sq(zs(k));
        return Txx + Tzz;
    }
    // vis_space (smoother.f90:142-164)
    inline double vis_space(int i, int k, const Arr& T0, int level) const {
        int f = 1 << (level - 1), i1 = i * f, k1 = k * f;
        double Tr = dotx(D1, span1, T0, i, k) / dr_grid[level], Ts = dotz(D1, span1, T0, i, k) / ds_grid[level];
        double Trr = dotx(D2, span1, T0, i, k) / dr2_grid[level], Tss = dotz(D2, span1, T0, i, k) / ds2_grid[level];
        double Tx = Tr / xr(i1), Tz = Ts / zs(k1);
        double Txx = (Trr - Tx * xrr(i1)) / sq(xr(i1));
        double Tzz = (Tss - Tz * zss(k1)) / sq(zs(k1));
        return Txx + Tzz;
    }
    // smoother_time_T (smoother.f90:343-377)
    int smoother_time_T(const Arr& Tin) {
        Tvis = Tin; Tbuoy = Tin;
        if (p.RaT == 0.0) return TC_OK;
        int n = 0;
        Arr T0;
        for (;;) {
            double diff = smoothness(Tvis);
            if (diff < delta_T) { n_temp = n; break; }
            if (n >= loop_cap) return TC_ERR_LOOP_CAP;
            T0 = Tvis;
#pragma omp parallel for schedule(static)
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k <= nz; k++) {
                    double temp = smoother_space(i, k, T0);
                    double dts = dts_array(i, k) * p.courantT;
                    Tvis(i, k) = T0(i, k) + dts * temp;
                }
            enforceBCs(Tvis);
            n++;
        }
        return TC_OK;
    }
    // smoother_time (smoother.f90:287-341): C filter for every enriched type.
    int smoother_time() {
        int Niter = 10;
        double lb = -5.0, la = -1.0;
        for (int t = 0; t < ntype; t++) { Cvis[t] = Cnew[t]; Cbuoy[t] = Cnew[t]; }
        Arr T0;
        for (int t = 0; t < ntype; t++) {
            int nn = 0, trigger = 0;
            long guard = 0;
            for (;;) {
                for (int n = 1; n <= Niter; n++) {
                    double diff = smoothness(Cvis[t]);
                    if (diff < delta_C[t]) { trigger = 1; break; }
                    double c;
                    if (nn == 0) {
                        int ntemp = Niter - n + 1;
                        c = 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * pii / (double)(2 * Niter)));
                    } else c = 1.0;
                    T0 = Cvis[t];
                    Arr& Cv = Cvis[t];
#pragma omp parallel for schedule(static)
                    for (int i = 0; i <= nx; i++)
                        for (int k = 0; k <= nz; k++) {
                            double temp = smoother_space(i, k, T0);
                            double dts = dts_array(i, k) * p.courantC;
                            double v = T0(i, k) + c * dts * temp;
                            if (v < 0.0) v = 0.0;
                            if (v > 1.0) v = 1.0;
                            Cv(i, k) = v;
                        }
                    enforceBCs_comp(Cvis[t]);
                }
                if (trigger == 1) break;
                Niter = 1;
                nn++;
                if (++guard > loop_cap) return TC_ERR_LOOP_CAP;
            }
            n_comp[t] = nn;
        }
        return TC_OK;
    }

    // =====================================================================
    // viscosity and per-level coefficients
    // =====================================================================
    // visf (momentum.f90:1-30)
    double visf(int i, int k) const {
        if (p.ivis == 1) return std::exp(-Tvis(i, k) * std::log(p.visT) + (1.0 - zg(k)) * std::log(p.visP));
        if (p.ivis == 2 && comp == 1) {
            double d = 0.0;
            for (int j = 0; j < ntype; j++) d = d + Cvis[j](i, k) * std::log(p.visC[j]);
            if (p.RaT != 0.0) return std::exp(-Tvis(i, k) * std::log(p.visT) - d + (1.0 - zg(k)) * std::log(p.visP));
            return std::exp(-d + (1.0 - zg(k)) * std::log(p.visP));
        }
        if (p.ivis == 3) {
            double diffusion = std::pow(p.visT, -T(i, k));
            if (zg(k) < (1.0 - p.yield_depth) || strain(i, k) == 0.0) return diffusion;
            double plastic = (p.yield + p.yield_gradient * zg(k)) / strain(i, k);
            return 1.0 / (1.0 / diffusion + 1.0 / plastic);
        }
        if (p.ivis == -1) return std::exp((1.0 - zg(k)) * std::log(p.visP));
        return 1.0;
    }
    // compute_strain_rate_invariant (momentum.f90:32-62)
    void compute_strain_rate_invariant() {
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                double ur = dotx(D1, span1, u, i, k) / dr, us = dotz(D1, span1, u, i, k) / ds;
                double wr = dotx(D1, span1, w, i, k) / dr, ws = dotz(D1, span1, w, i, k) / ds;
                double ux = ur / xr(i), uz = us / zs(k), wx = wr / xr(i), wz = ws / zs(k);
                strain(i, k) = std::pow(0.5 * (2.0 * (sq(ux) + sq(wz)) + sq(uz + wx)), 0.5);
            }
        for (int i = 1; i <= span; i++)
            for (int k = 0; k <= nz; k++) { strain(-i, k) = strain(i, k); strain(nx + i, k) = strain(nx - i, k); }
        for (int k = 1; k <= span; k++)
            for (int i = -span; i <= nx + span; i++) { strain(i, -k) = strain(i, k); strain(i, nz + k) = strain(i, nz - k); }
    }
    // viscosity_gradients (iterative_solver.f90:290-329)
    void viscosity_gradients(int level) {
        int a = nx_grid[level], b = nz_grid[level];
        if (p.ivis == 0) {
            vis_x[level].fill(0); vis_z[level].fill(0); vis_xx[level].fill(0); vis_zz[level].fill(0); vis_xz[level].fill(0);
            return;
        }
        const Arr& V = vis_grid[level];
        int f = 1 << (level - 1);
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= a - 1; i++) {
            int ii = i * f;
            for (int k = 1; k <= b - 1; k++) {
                int kk = k * f;
                double vis_r = dotx(D1, span1, V, i, k) / dr_grid[level];
                double vis_rr = dotx(D2, span1, V, i, k) / dr2_grid[level];
                double vis_s = dotz(D1, span1, V, i, k) / ds_grid[level];
                double vis_ss = dotz(D2, span1, V, i, k) / ds2_grid[level];
                double vis_rs = sum2(Drs, V, i, k) / drds_grid[level];
                vis_x[level](i, k) = vis_r / xr(ii);
                vis_z[level](i, k) = vis_s / zs(kk);
                vis_xx[level](i, k) = (vis_rr - vis_x[level](i, k) * xrr(ii)) / sq(xr(ii));
                vis_zz[level](i, k) = (vis_ss - vis_z[level](i, k) * zss(kk)) / sq(zs(kk));
                vis_xz[level](i, k) = vis_rs / xr(ii) / zs(kk);
            }
        }
    }
    // eigI / eigR (iterative_solver.f90:750-857)
    double eigI(int level, int i, int k, const EigMax& e) const {
        int f = 1 << (level - 1), i1 = i * f, k1 = k * f;
        double Sr = e.Tr, Ss = e.Ts, Srr = 0, Sss = 0, Srrr = e.Trrr, Ssss = e.Tsss, Srrrr = 0, Sssss = 0;
        double Srs = 0, Srrs = e.Trrs, Srss = e.Trss, Srrss = 0;
        double x1 = xr(i1), x2 = xrr(i1), x3 = xrrr(i1), x4 = xrrrr(i1);
        double z1 = zs(k1), z2 = zss(k1), z3 = zsss(k1), z4 = zssss(k1);
        double Sx = Sr / x1, Sz = Ss / z1;
        double Sxx = (Srr + std::fabs(Sx * x2)) / sq(x1);
        double Szz = (Sss + std::fabs(Sz * z2)) / sq(z1);
        double Sxxx = (Srrr + std::fabs(3.0 * Sxx * x1 * x2) + std::fabs(Sx * x3)) / std::fabs(std::pow(x1, 3.0));
        double Szzz = (Ssss + std::fabs(3.0 * Szz * z1 * z2) + std::fabs(Sz * z3)) / std::fabs(std::pow(z1, 3.0));
        double Sxxxx = (Srrrr + std::fabs(6.0 * Sxxx * x2 * sq(x1)) + (std::fabs(3.0 * sq(x2) + 4.0 * x1 * x3) * std::fabs(Sxx)) + std::fabs(Sx * x4)) / std::pow(x1, 4.0);
        double Szzzz = (Sssss + std::fabs(6.0 * Szzz * z2 * sq(z1)) + (std::fabs(3.0 * sq(z2) + 4.0 * z1 * z3) * std::fabs(Szz)) + std::fabs(Sz * z4)) / std::pow(z1, 4.0);
        double Sxz = Srs / x1 / z1;
        double Sxxz = (Srrs + std::fabs(Sxz * z1 * x2)) / std::fabs(z1) / sq(x1);
        double Sxzz = (Srss + std::fabs(Sxz * x1 * z2)) / std::fabs(x1) / sq(z1);
        double Sxxzz = (Srrss + std::fabs(Sxzz * x2) * sq(z1) + std::fabs(Sxxz * z2) * sq(x1) + std::fabs(Sxz * x2 * z2)) / sq(x1 * z1);
        const Arr &V = vis_grid[level];
        double t1 = (vis_xx[level](i, k) + vis_zz[level](i, k)) * (Sxx + Szz);
        double t2 = V(i, k) * (Sxxxx + Szzzz);
        double t3 = 2.0 * V(i, k) * Sxxzz;
        double t4 = 4.0 * vis_xz[level](i, k) * Sxz;
        double t5 = 2.0 * vis_x[level](i, k) * (Sxxx + Sxzz);
        double t6 = 2.0 * vis_z[level](i, k) * (Szzz + Sxxz);
        return std::fabs(t1) + std::fabs(t2) + std::fabs(t3) + std::fabs(t4) + std::fabs(t5) + std::fabs(t6);
    }
    double eigR(int level, int i, int k, const EigMax& e) const {
        int f = 1 << (level - 1), i1 = i * f, k1 = k * f;
        double Sr = 0, Ss = 0, Srr = e.Trr, Sss = e.Tss, Srrr = 0, Ssss = 0, Srrrr = e.Trrrr, Sssss = e.Tssss;
        double Srs = e.Trs, Srrs = 0, Srss = 0, Srrss = e.Trrss;
        double x1 = xr(i1), x2 = xrr(i1), x3 = xrrr(i1), x4 = xrrrr(i1);
        double z1 = zs(k1), z2 = zss(k1), z3 = zsss(k1), z4 = zssss(k1);
        double Sx = Sr / x1, Sz = Ss / z1;
        double Sxx = (Srr - Sx * x2) / sq(x1);
        double Szz = (Sss - Sz * z2) / sq(z1);
        double Sxxx = (Srrr - 3.0 * Sxx * x1 * x2 - Sx * x3) / std::pow(x1, 3.0);
        double Szzz = (Ssss - 3.0 * Szz * z1 * z2 - Sz * z3) / std::pow(z1, 3.0);
        double Sxxxx = (Srrrr - 6.0 * Sxxx * x2 * sq(x1) - (3.0 * sq(x2) + 4.0 * x1 * x3) * Sxx - Sx * x4) / std::pow(x1, 4.0);
        double Szzzz = (Sssss - 6.0 * Szzz * z2 * sq(z1) - (3.0 * sq(z2) + 4.0 * z1 * z3) * Szz - Sz * z4) / std::pow(z1, 4.0);
        double Sxz = Srs / x1 / z1;
        double Sxxz = (Srrs - Sxz * z1 * x2) / z1 / sq(x1);
        double Sxzz = (Srss - Sxz * x1 * z2) / x1 / sq(z1);
        double Sxxzz = (Srrss - Sxzz * x2 * sq(z1) - Sxxz * z2 * sq(x1) - Sxz * x2 * z2) / sq(x1 * z1);
        const Arr &V = vis_grid[level];
        double t1 = (vis_xx[level](i, k) - vis_zz[level](i, k)) * (Sxx - Szz);
        double t2 = V(i, k) * (Sxxxx + Szzzz);
        double t3 = 2.0 * V(i, k) * Sxxzz;
        double t4 = 4.0 * vis_xz[level](i, k) * Sxz;
        double t5 = 2.0 * vis_x[level](i, k) * (Sxxx + Sxzz);
        double t6 = 2.0 * vis_z[level](i, k) * (Szzz + Sxxz);
        return -(t1 + t2 + t3 + t4 + t5 + t6);
    }
    // test_eigenvalues (iterative_solver.f90:666-698): resets ratio on every
    // level to 1e99 before filling the requested one.
    void test_eigenvalues(int level) {
        for (int l = 1; l <= grids; l++) ratio[l].fill(1.0e99);
        if (p.ivis == 0) return;
        EigMax e = scaled_eig(level);
        int a = nx_grid[level], b = nz_grid[level];
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= a - 1; i++)
            for (int k = 1; k <= b - 1; k++) {
                double eI = eigI(level, i, k, e), eR = eigR(level, i, k, e);
                ratio[level](i, k) = std::fabs(eR / eI);
            }
    }
    // iterate_local_time_steps (iterative_solver.f90:700-748), iterate_order=1
    void iterate_local_time_steps(int level) {
        EigMax e = scaled_eig(level);
        int a = nx_grid[level], b = nz_grid[level];
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= a - 1; i++)
            for (int k = 1; k <= b - 1; k++) {
                double eI = eigI(level, i, k, e);
                double eR = eigR(level, i, k, e);
                dt_stream[level](i, k) = -p.courant_stream * 2.0 * eR / (sq(eR) + sq(eI));
            }
    }
    double ratio_min(int level) {
        double m = 1.0e300;
        int a = nx_grid[level], b = nz_grid[level];
        bool first = true;
        for (int k = 1; k <= b - 1; k++)
            for (int i = 1; i <= a - 1; i++) {
                double v = ratio[level](i, k);
                if (first || v < m) { m = v; first = false; }
            }
        return m;
    }
    // smoother_vis (smoother.f90:166-263)
    int smoother_vis(int level, int interpolate) {
        int option, Niter;
        double lb, la;
        if (level == 1 && interpolate == 0) { option = 1; Niter = 6; lb = -5.0; la = -2.0; }
        else { option = 0; Niter = p.vis_iter; lb = -2.0; la = -1.0; }
        if (interpolate == 0 || level == 1) { Nvis_store = 0; nn_store = 1; }
        int a = nx_grid[level], b = nz_grid[level];
        int kmin, kmax;
        if (p.RaT == 0.0) { kmin = 0; kmax = b; } else { kmin = 1; kmax = b - 1; }
        int n = 0, trigger = 0;
        Arr T0;
        long guard = 0;
        for (;;) {
            int nn_begin = nn_store;
            for (int nn = nn_begin; nn <= Niter; nn++) {
                viscosity_gradients(level);
                test_eigenvalues(level);
                double rmin = ratio_min(level);
                if (option == 1) {
                    if ((Nvis_store >= 1 && rmin > p.eig_ratio_min) || p.ivis == 0 || n > 20) {
                        eig_fine = rmin; n_eta = n; trigger = 1; break;
                    }
                } else {
                    if (interpolate == 0) {
                        if (rmin > p.eig_ratio || p.ivis == 0) { trigger = 1; nn_store = nn; break; }
                    } else {
                        if (Nvis_store >= 1 || p.ivis == 0) { trigger = 1; break; }
                    }
                }
                int ntemp = Niter - nn + 1;
                double c = 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * pii / (double)(2 * Niter)));
                T0 = vis_grid[level];
                Arr& V = vis_grid[level];
#pragma omp parallel for schedule(static)
                for (int i = 0; i <= a; i++)
                    for (int k = kmin; k <= kmax; k++) {
                        double temp = vis_space(i, k, T0, level);
                        double dts = dt_vis[level](i, k) * 0.99;
                        V(i, k) = T0(i, k) + c * dts * temp;
                    }
                viscosity_bcs(level, false);
                if (++guard > loop_cap) return TC_ERR_LOOP_CAP;
            }
            if (trigger == 1) break;
            Nvis_store = Nvis_store + 1;
            nn_store = 1;
            if (option == 1) { nn_store = 1; Niter = 6; lb = -2.0; la = -1.0; }
            n = n + 1;
            if (++guard > loop_cap) return TC_ERR_LOOP_CAP;
        }
        return TC_OK;
    }
    // restrict / restrict_coefficients (iterative_solver.f90:596-664); the
    // corner term repeats (ii-1,kk+1) and omits (ii+1,kk-1), as in the reference.
    void restrict_arr(int level, const Arr& in, Arr& out) {
        int a = nx_grid[level], b = nz_grid[level];
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= a - 1; i++) {
            int ii = 2 * i;
            for (int k = 1; k <= b - 1; k++) {
                int kk = 2 * k;
                double corners = (in(ii - 1, kk - 1) + in(ii - 1, kk + 1) + in(ii + 1, kk + 1) + in(ii - 1, kk + 1)) / 16.0;
                double sides = (in(ii - 1, kk) + in(ii, kk - 1) + in(ii + 1, kk) + in(ii, kk + 1)) / 8.0;
                double centre = in(ii, kk) / 4.0;
                out(i, k) = corners + sides + centre;
            }
        }
    }
    // compute_viscosity (iterative_solver.f90:331-377)
    int compute_viscosity(int level) {
        int st;
        if (level == 1) {
            Arr& V = vis_grid[1];
#pragma omp parallel for schedule(static)
            for (int i = -span; i <= nx_grid[1] + span; i++)
                for (int k = -span; k <= nz_grid[1] + span; k++) V(i, k) = visf(i, k);
            st = smoother_vis(1, 0);
            if (st) return st;
        } else {
            int l1 = level - 1;
            vis_gridf[l1] = vis_grid[l1]; vis_xf[l1] = vis_x[l1]; vis_zf[l1] = vis_z[l1];
            vis_xxf[l1] = vis_xx[l1]; vis_zzf[l1] = vis_zz[l1]; vis_xzf[l1] = vis_xz[l1];
            st = smoother_vis(l1, 1);
            if (st) return st;
            restrict_arr(level, vis_grid[l1], vis_grid[level]);
            viscosity_bcs(level, true);
            if (level < grids) { st = smoother_vis(level, 0); if (st) return st; }
            else viscosity_gradients(level);
            vis_grid[l1] = vis_gridf[l1]; vis_x[l1] = vis_xf[l1]; vis_z[l1] = vis_zf[l1];
            vis_xx[l1] = vis_xxf[l1]; vis_zz[l1] = vis_zzf[l1]; vis_xz[l1] = vis_xzf[l1];
        }
        return TC_OK;
    }

    // =====================================================================
    // streamfunction operator and multigrid
    // =====================================================================
    // stream_space (iterative_solver.f90:456-561).  build=0: RHS - L S0;
    // build=1: coefficient of S(iq,kq) (times Sval) in L at (i,k).
    double stream_space(int i, int k, const Arr* S0, int level, int iq, int kq, double Sval) const {
        int f = 1 << (level - 1), i1 = i * f, k1 = k * f;
        double Sr, Ss, Srr, Sss, Srrr, Ssss, Srrrr, Sssss, Srs, Srss, Srrs, Srrss;
        if (build == 0) {
            const Arr& S = *S0;
            Sr = dotx(D1, span1, S, i, k) / dr_grid[level];
            Ss = dotz(D1, span1, S, i, k) / ds_grid[level];
            Srr = dotx(D2, span1, S, i, k) / dr2_grid[level];
            Sss = dotz(D2, span1, S, i, k) / ds2_grid[level];
            Srrr = dotx(D3, span, S, i, k) / dr3_grid[level];
            Ssss = dotz(D3, span, S, i, k) / ds3_grid[level];
            Srrrr = dotx(D4, span, S, i, k) / dr4_grid[level];
            Sssss = dotz(D4, span, S, i, k) / ds4_grid[level];
            Srs = sum2(Drs, S, i, k) / drds_grid[level];
            Srss = sum2(Drss, S, i, k) / drds2_grid[level];
            Srrs = sum2(Drrs, S, i, k) / dr2ds_grid[level];
            Srrss = sum2(Drrss, S, i, k) / dr2ds2_grid[level];
        } else {
            int di = iq - i, dk = kq - k;
            if (k == kq) {
                Sr = D1(di) * Sval / dr_grid[level]; Srr = D2(di) * Sval / dr2_grid[level];
                Srrr = D3(di) * Sval / dr3_grid[level]; Srrrr = D4(di) * Sval / dr4_grid[level];
            } else { Sr = 0; Srr = 0; Srrr = 0; Srrrr = 0; }
            if (i == iq) {
                Ss = D1(dk) * Sval / ds_grid[level]; Sss = D2(dk) * Sval / ds2_grid[level];
                Ssss = D3(dk) * Sval / ds3_grid[level]; Sssss = D4(dk) * Sval / ds4_grid[level];
            } else { Ss = 0; Sss = 0; Ssss = 0; Sssss = 0; }
            Srs = Drs(di, dk) * Sval / drds_grid[level];
            Srss = Drss(di, dk) * Sval / drds2_grid[level];
            Srrs = Drrs(di, dk) * Sval / dr2ds_grid[level];
            Srrss = Drrss(di, dk) * Sval / dr2ds2_grid[level];
        }
        double x1 = xr(i1), x2 = xrr(i1), x3 = xrrr(i1), x4 = xrrrr(i1);
        double z1 = zs(k1), z2 = zss(k1), z3 = zsss(k1), z4 = zssss(k1);
        double Sx = Sr / x1, Sz = Ss / z1;
        double Sxx = (Srr - Sx * x2) / sq(x1);
        double Szz = (Sss - Sz * z2) / sq(z1);
        double Sxxx = (Srrr - 3.0 * Sxx * x1 * x2 - Sx * x3) / std::pow(x1, 3.0);
        double Szzz = (Ssss - 3.0 * Szz * z1 * z2 - Sz * z3) / std::pow(z1, 3.0);
        double Sxxxx = (Srrrr - 6.0 * Sxxx * x2 * sq(x1) - (3.0 * sq(x2) + 4.0 * x1 * x3) * Sxx - Sx * x4) / std::pow(x1, 4.0);
        double Szzzz = (Sssss - 6.0 * Szzz * z2 * sq(z1) - (3.0 * sq(z2) + 4.0 * z1 * z3) * Szz - Sz * z4) / std::pow(z1, 4.0);
        double Sxz = Srs / x1 / z1;
        double Sxxz = (Srrs - Sxz * z1 * x2) / z1 / sq(x1);
        double Sxzz = (Srss - Sxz * x1 * z2) / x1 / sq(z1);
        double Sxxzz = (Srrss - Sxzz * x2 * sq(z1) - Sxxz * z2 * sq(x1) - Sxz * x2 * z2) / sq(x1 * z1);
        const Arr& V = vis_grid[level];
        double t1, t2, t3, t4, t5, t6;
        if (p.ivis == 0) {
            t1 = 0.0; t2 = V(i, k) * (Sxxxx + Szzzz); t3 = 2.0 * V(i, k) * Sxxzz; t4 = 0.0; t5 = 0.0; t6 = 0.0;
        } else {
            t1 = (vis_xx[level](i, k) - vis_zz[level](i, k)) * (Sxx - Szz);
            t2 = V(i, k) * (Sxxxx + Szzzz);
            t3 = 2.0 * V(i, k) * Sxxzz;
            t4 = 4.0 * vis_xz[level](i, k) * Sxz;
            t5 = 2.0 * vis_x[level](i, k) * (Sxxx + Sxzz);
            t6 = 2.0 * vis_z[level](i, k) * (Szzz + Sxxz);
        }
        if (build == 0) {
            if (scaling == 0) return -(t1 + t2 + t3 + t4 + t5 + t6 - RHS[level](i, k));
            return t1 + t2 + t3 + t4 + t5 + t6;
        }
        return t1 + t2 + t3 + t4 + t5 + t6;
    }
    // compute_RHS (iterative_solver.f90:563-594)
    void compute_RHS(int level) {
        if (level == 1) {
            Arr& R = RHS[1];
#pragma omp parallel for schedule(static)
            for (int i = 1; i <= nx_grid[1] - 1; i++)
                for (int k = 1; k <= nz_grid[1] - 1; k++) {
                    R(i, k) = 0.0;
                    if (p.RaT != 0.0) {
                        double Tr = dotx(D1, span1, Tbuoy, i, k) / dr;
                        double Tx = Tr / xr(i);
                        R(i, k) = p.RaT * Tx;
                    }
                    if (comp == 1)
                        for (int j = 0; j < ntype; j++) {
                            double Cr = dotx(D1, span1, Cbuoy[j], i, k) / dr;
                            double Cx = Cr / xr(i);
                            R(i, k) = R(i, k) - p.RaC[j] * Cx;
                        }
                }
        } else {
            restrict_arr(level, residual, RHS[level]);
        }
    }
    // compute_reference_residual (iterative_solver.f90:281-288)
    void compute_reference_residual(int level) {
        double s = 0.0;
        int a = nx_grid[level], b = nz_grid[level];
        for (int k = 1; k <= b - 1; k++)
            for (int i = 1; i <= a - 1; i++) s = s + std::fabs(RHS[level](i, k));
        res_ref[level] = s / (double)(a - 2) / (double)(b - 2);
    }
    // compute_residual (iterative_solver.f90:258-279)
    int compute_residual(int level, const Arr& sol, int pidx) {
        int a = nx_grid[level], b = nz_grid[level];
#pragma omp parallel for schedule(static)
        for (int i = 1; i <= a - 1; i++)
            for (int k = 1; k <= b - 1; k++) residual(i, k) = stream_space(i, k, &sol, level, 0, 0, 0.0);
        double s = 0.0;
        for (int k = 1; k <= b - 1; k++)
            for (int i = 1; i <= a - 1; i++) s = s + std::fabs(residual(i, k));
        residual_mag[pidx] = s / (double)(a - 1) / (double)(b - 1);
        if (level == 1 && residual_mag[pidx] > 1.0e10 * res_ref[level]) return TC_ERR_MG_RESIDUAL;
        return TC_OK;
    }
    // iterate_stream (iterative_solver.f90:860-963), iterate_order=1
    int iterate_stream(int level, int Niter, int dir, int pidx) {
        int a = nx_grid[level], b = nz_grid[level];
        Arr c; c.alloc(1, a - 1, 1, b - 1);
        Arr S0;
        for (int n = 1; n <= Niter; n++) {
            double ntemp = (double)(Niter - n + 1);
            double la = -1.0;
            double temp = std::cos((2.0 * ntemp - 1.0) * pii / (double)(2 * Niter));
            const Arr& R = ratio[level];
            for (int i = 1; i <= a - 1; i++)
                for (int k = 1; k <= b - 1; k++) {
                    double lb;
                    double rr = R(i, k);
                    if (rr > 1.0e99) lb = -2.0;
                    else lb = -2.0 * sq(rr) / (1.0 + sq(rr));
                    c(i, k) = 2.0 / (-lb - la + (lb - la) * temp);
                }
            if (dir == 1) c.fill(1.0);
            S0 = error[level];
            Arr& E = error[level];
#pragma omp parallel for schedule(static)
            for (int i = 1; i <= a - 1; i++)
                for (int k = 1; k <= b - 1; k++) {
                    double t = stream_space(i, k, &S0, level, 0, 0, 0.0);
                    E(i, k) = S0(i, k) + c(i, k) * dt_stream[level](i, k) * t;
                }
            enforceBCs_stream(level, E);
        }
        return compute_residual(level, error[level], pidx);
    }
    // prolong (iterative_solver.f90:175-233)
    void prolong(int lc) {
        int lf = lc - 1;
        Arr& F = error[lf];
        const Arr& C = error[lc];
        for (int i = 1; i <= nx_grid[lc] - 1; i++)
            for (int k = 1; k <= nz_grid[lc] - 1; k++) F(2 * i, 2 * k) = F(2 * i, 2 * k) + C(i, k);
        for (int i = 2; i <= nx_grid[lf] - 2; i += 2)
            for (int k = 1; k <= nz_grid[lf] - 1; k += 2)
                F(i, k) = F(i, k) + (C(i / 2, (k - 1) / 2) + C(i / 2, (k + 1) / 2)) / 2.0;
        for (int k = 2; k <= nz_grid[lf] - 2; k += 2)
            for (int i = 1; i <= nx_grid[lf] - 1; i += 2)
                F(i, k) = F(i, k) + (C((i - 1) / 2, k / 2) + C((i + 1) / 2, k / 2)) / 2.0;
        for (int i = 1; i <= nx_grid[lf] - 1; i += 2)
            for (int k = 1; k <= nz_grid[lf] - 1; k += 2)
                F(i, k) = F(i, k) + (C((i - 1) / 2, (k - 1) / 2) + C((i + 1) / 2, (k - 1) / 2) +
                                     C((i + 1) / 2, (k + 1) / 2) + C((i - 1) / 2, (k + 1) / 2)) / 4.0;
        enforceBCs_stream(lf, F);
    }
    // pf_coarse / indices_coarse with Database=2 (iterative_solver.f90:991-1024)
    int pf_coarse(int ip, int kp) const { int N = nz_grid[grids] + 1; return N * ip + kp + 1; }
    void indices_coarse(int pp, int& ip, int& kp) const {
        int N = nz_grid[grids] + 1;
        kp = pp - N * ((pp - 1) / N) - 1;
        ip = (pp - 1) / N;
    }
    inline double& MC(int r, int c) { return Mc[(size_t)(r - 1) + (size_t)(c - 1) * ldab]; }
    // Compute_Matrix_coarse (iterative_solver.f90:1026-1179) incl. DGBEQU row scaling.
    void Compute_Matrix_coarse() {
        int nxc = nx_grid[grids], nzc = nz_grid[grids];
        std::vector<int> limit(2 * span + 1);
        auto LIM = [&](int j) -> int& { return limit[j + span]; };
        LIM(-span) = 0;
        for (int j = -span1; j <= -1; j++) LIM(j) = span1;
        LIM(0) = span;
        for (int j = 1; j <= span1; j++) LIM(j) = span1;
        LIM(span) = 0;
        if (analysis == 1) {
            ku = 0; kl = 0;
            for (int pp = 1; pp <= ngrid_coarse; pp++) {
                int ip, kp; indices_coarse(pp, ip, kp);
                for (int j = -span; j <= span; j++) {
                    int iq = j + ip;
                    if (iq > 0 && iq < nxc)
                        for (int kq = -LIM(j) + kp; kq <= kp + LIM(j); kq++)
                            if (kq > 0 && kq < nzc) {
                                int q = pf_coarse(iq, kq), t = q - pp;
                                if (t > ku) ku = t;
                                if (-t > kl) kl = -t;
                            }
                }
            }
            return;
        }
        int kv1 = kl + ku + 1;
        build = 1;
        std::fill(Mc.begin(), Mc.end(), 0.0);
        for (int pp = 1; pp <= ngrid_coarse; pp++) {
            int ip, kp; indices_coarse(pp, ip, kp);
            if (ip > 0 && ip < nxc && kp > 0 && kp < nzc)
                for (int j = -span; j <= span; j++) {
                    int iq = j + ip;
                    if (iq >= 0 && iq <= nxc)
                        for (int kq = -LIM(j) + kp; kq <= kp + LIM(j); kq++)
                            if (kq >= 0 && kq <= nzc) {
                                int q = pf_coarse(iq, kq);
                                MC(kv1 + pp - q, q) = stream_space(ip, kp, nullptr, grids, iq, kq, 1.0);
                            }
                }
        }
        for (int pp = 1; pp <= ngrid_coarse; pp++) {
            int ip, kp; indices_coarse(pp, ip, kp);
            if (ip > 0 && ip < nxc && kp > 0 && kp < nzc)
                for (int j = -span; j <= span; j++) {
                    int iq = j + ip;
                    for (int kq = -LIM(j) + kp; kq <= kp + LIM(j); kq++) {
                        if (iq < 0 || iq > nxc || kq < 0 || kq > nzc) {
                            int iiq, kkq; double xval, zval;
                            if (iq < 0) { iiq = -iq; xval = -1.0; }
                            else if (iq > nxc) { iiq = 2 * nxc - iq; xval = -1.0; }
                            else { iiq = iq; xval = 1.0; }
                            if (kq < 0) { kkq = -kq; zval = (p.Vbc == 0) ? -1.0 : 1.0; }
                            else if (kq > nzc) { kkq = 2 * nzc - kq; zval = (p.Vbc == 0) ? -1.0 : 1.0; }
                            else { kkq = kq; zval = 1.0; }
                            double Sval = xval * zval;
                            int q = pf_coarse(iiq, kkq);
                            MC(kv1 + pp - q, q) = MC(kv1 + pp - q, q) + stream_space(ip, kp, nullptr, grids, iq, kq, Sval);
                        }
                    }
                }
        }
        for (int kp = 0; kp <= nzc; kp++) { MC(kv1, pf_coarse(0, kp)) = 1.0; MC(kv1, pf_coarse(nxc, kp)) = 1.0; }
        for (int ip = 0; ip <= nxc; ip++) { MC(kv1, pf_coarse(ip, 0)) = 1.0; MC(kv1, pf_coarse(ip, nzc)) = 1.0; }
        // DGBEQU row factors on rows kl+1..2kl+ku+1 (band without fill rows)
        int n = ngrid_coarse;
        for (int i = 1; i <= n; i++) RowB[i] = 0.0;
        for (int j = 1; j <= n; j++)
            for (int i = std::max(j - ku, 1); i <= std::min(j + kl, n); i++)
                RowB[i] = std::max(RowB[i], std::fabs(MC(kv1 + i - j, j)));
        const double smlnum = 2.2250738585072014e-308, bignum = 1.0 / smlnum;
        for (int i = 1; i <= n; i++) RowB[i] = 1.0 / std::min(std::max(RowB[i], smlnum), bignum);
        for (int q = 1; q <= n; q++)
            for (int pp = std::max(1, q - kl); pp <= std::min(n, q + ku); pp++) MC(kv1 + pp - q, q) = RowB[pp] * MC(kv1 + pp - q, q);
        build = 0;
    }
    // DGBTRF via the unblocked dgbtf2 algorithm (LAPACK 3.x).
    int dgbtrf() {
        int n = ngrid_coarse, m = n, KV = ku + kl, info = 0;
        auto AB = [&](int r, int c) -> double& { return MC(r, c); };
        for (int j = ku + 2; j <= std::min(KV, n); j++)
            for (int i = KV - j + 2; i <= kl; i++) AB(i, j) = 0.0;
        int JU = 1;
        for (int j = 1; j <= std::min(m, n); j++) {
            if (j + KV <= n)
                for (int i = 1; i <= kl; i++) AB(i, j + KV) = 0.0;
            int KM = std::min(kl, m - j);
            int JP = 1; double amax = std::fabs(AB(KV + 1, j));
            for (int t = 2; t <= KM + 1; t++) { double v = std::fabs(AB(KV + t, j)); if (v > amax) { amax = v; JP = t; } }
            IPIV[j] = JP + j - 1;
            if (AB(KV + JP, j) != 0.0) {
                JU = std::max(JU, std::min(j + ku + JP - 1, n));
                if (JP != 1)
                    for (int c = 0; c <= JU - j; c++) std::swap(AB(KV + JP - c, j + c), AB(KV + 1 - c, j + c));
                if (KM > 0) {
                    double rcp = 1.0 / AB(KV + 1, j);
                    for (int t = 1; t <= KM; t++) AB(KV + 1 + t, j) = rcp * AB(KV + 1 + t, j);
                    if (JU > j)
                        for (int c = 1; c <= JU - j; c++) {
                            double temp = -AB(KV + 1 - c, j + c);  // alpha*y(j), alpha=-1
                            if (temp != 0.0)
                                for (int t = 1; t <= KM; t++) AB(KV + 1 + t - c, j + c) = AB(KV + 1 + t - c, j + c) + AB(KV + 1 + t, j) * temp;
                        }
                }
            } else if (info == 0) info = j;
        }
        return info;
    }
    // DGBTRS('N', NRHS=1) via dger + dtbsv (LAPACK 3.x).
    void dgbtrs(std::vector<double>& B) {
        int n = ngrid_coarse, KD = ku + kl + 1;
        auto AB = [&](int r, int c) -> double& { return MC(r, c); };
        if (kl > 0)
            for (int j = 1; j <= n - 1; j++) {
                int LM = std::min(kl, n - j);
                int L = IPIV[j];
                if (L != j) std::swap(B[L], B[j]);
                double temp = -B[j];
                if (temp != 0.0)
                    for (int t = 1; t <= LM; t++) B[j + t] = B[j + t] + AB(KD + t, j) * temp;
            }
        int K = kl + ku;  // dtbsv upper, non-unit, bandwidth K, diagonal in row K+1
        for (int j = n; j >= 1; j--) {
            if (B[j] != 0.0) {
                int L = K + 1 - j;
                B[j] = B[j] / AB(K + 1, j);
                double temp = B[j];
                for (int i = j - 1; i >= std::max(1, j - K); i--) B[i] = B[i] - temp * AB(L + i, j);
            }
        }
    }
    void Compute_coarse_vector() {
        for (int i = 1; i <= ngrid_coarse; i++) Bc[i] = 0.0;
        for (int i = 1; i <= nx_grid[grids] - 1; i++)
            for (int k = 1; k <= nz_grid[grids] - 1; k++) {
                int pp = pf_coarse(i, k);
                Bc[pp] = RHS[grids](i, k) * RowB[pp];
            }
    }
    void Stream_grid_coarse() {
        for (int pp = 1; pp <= ngrid_coarse; pp++) {
            int ip, kp; indices_coarse(pp, ip, kp);
            error[grids](ip, kp) = Bc[pp];
        }
    }
    int last_cycles = 0;
    int cycles_acc = 0;
    // level-1 residual ratio after each level-1 visit of the last multigrid
    // call (the quantity the convergence test compares with the tolerance)
    std::vector<double> res_trace;
    // multigrid (iterative_solver.f90:79-173)
    int multigrid() {
        int st;
        res_trace.clear();
        error[1] = SF;
        compute_RHS(1);
        compute_reference_residual(1);
        if (p.non_Newtonian == 0) {
            for (int l = 1; l <= grids; l++) { st = compute_viscosity(l); if (st) return st; }
            if (time == 0.0 || p.ivis > 0) {
                Compute_Matrix_coarse();
                if (dgbtrf() != 0) return TC_ERR_SINGULAR;
            }
            for (int l = 1; l <= grids; l++) iterate_local_time_steps(l);
        }
        int q = 1;
        for (;;) {
            if (p.non_Newtonian == 1) {
                SF = error[1];
                compute_velocities();
                compute_strain_rate_invariant();
                for (int l = 1; l <= grids; l++) {
                    st = compute_viscosity(l); if (st) return st;
                    iterate_local_time_steps(l);
                }
                Compute_Matrix_coarse();
                if (dgbtrf() != 0) return TC_ERR_SINGULAR;
            }
            bool conv = false;
            for (int pp = 1; pp <= nsteps; pp++) {
                int level = multi[pp];
                int dir = (multi[pp + 1] > multi[pp]) ? 0 : 1;
                if (multi[pp - 1] < multi[pp]) {
                    if (p.mg_zero_coarse && level > 1 && level < grids) error[level].fill(0.0);
                    compute_RHS(level);
                    if (pp <= grids && q == 1) compute_reference_residual(level);
                }
                if (level < grids) {
                    st = iterate_stream(level, p.Nmulti, dir, pp);
                    if (getenv("TCO_DEBUG")) fprintf(stderr, "q=%d p=%d level=%d dir=%d res=%.6e ref=%.6e\n", q, pp, level, dir, residual_mag[pp], res_ref[level]);
                    if (st) return st;
                } else {
                    Compute_coarse_vector();
                    dgbtrs(Bc);
                    Stream_grid_coarse();
                    enforceBCs_stream(level, error[level]);
                }
                if (level == 1) {
                    if (p.non_Newtonian == 1) {
                        SF = error[1];
                        compute_velocities();
                        compute_strain_rate_invariant();
                        st = compute_viscosity(1); if (st) return st;
                        st = compute_residual(1, error[1], pp); if (st) return st;
                    }
                    res_trace.push_back(residual_mag[1] / res_ref[1]);
                    if (residual_mag[1] / res_ref[1] <= p.tolerance) { conv = true; break; }
                }
                if (multi[pp + 1] < multi[pp]) prolong(level);
            }
            if (conv || residual_mag[1] / res_ref[1] <= p.tolerance) break;
            q = q + 1;
            if (q > p.max_cycles) { last_cycles = q; return TC_ERR_MG_CYCLES; }
        }
        SF = error[1];
        last_cycles = q;
        cycles_acc += q;
        return TC_OK;
    }

    // =====================================================================
    // velocities, tracers, composition
    // =====================================================================
    // compute_velocities (momentum.f90:532-551)
    void compute_velocities() {
        u.fill(0.0); w.fill(0.0);
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                double SFr = dotx(D1, span1, SF, i, k) / dr;
                double SFs = dotz(D1, span1, SF, i, k) / ds;
                double SFx = SFr / xr(i), SFz = SFs / zs(k);
                u(i, k) = SFz;
                w(i, k) = -SFx;
            }
        velocityBCs();
    }
    // compute_derivatives (composition.f90:900-919)
    void compute_derivatives(const Arr& f, std::vector<Arr>& DERr) {
        int si = span_interp;
        for (int jj = 1; jj <= order - 1; jj++)
            for (int k = -si; k <= nz + si; k++)
                for (int i = 0; i <= nx; i++) {
                    double s = 0.0;
                    for (int j = -si; j <= si; j++) s = s + D[jj](j) * f(i + j, k);
                    DERr[jj](i, k) = s / dr_power[jj];
                }
    }
    // interpolate (composition.f90:838-898)
    double interpolate(double r, double s, const std::vector<Arr>& DERr, const Arr& f) const {
        int si = span_interp;
        int i = (int)(r / dr);
        int k = (int)(s / ds);
        double hr = r - (double)i * dr;
        double fR[16];  // index jj+si, jj=-si..si+1
        if (hr <= dro2) {
            for (int jj = -si; jj <= si + 1; jj++) fR[jj + si] = f(i, k + jj);
            for (int j = 1; j <= order - 1; j++) {
                double a1 = pw(hr, j) / factorial[j];
                for (int jj = -si; jj <= si + 1; jj++) fR[jj + si] = fR[jj + si] + DERr[j](i, k + jj) * a1;
            }
        } else {
            hr = dr - hr;
            for (int jj = -si; jj <= si + 1; jj++) fR[jj + si] = f(i + 1, k + jj);
            for (int j = 1; j <= order - 1; j++) {
                double a1 = pw(-hr, j) / factorial[j];
                for (int jj = -si; jj <= si + 1; jj++) fR[jj + si] = fR[jj + si] + DERr[j](i + 1, k + jj) * a1;
            }
        }
        double hs = s - (double)k * ds;
        double DERs[16];
        double fin;
        if (hs <= dso2) {
            for (int jj = 1; jj <= order - 1; jj++) {
                double t = 0.0;
                for (int j = -si; j <= si; j++) t = t + D[jj](j) * fR[0 + j + si];
                DERs[jj] = t / ds_power[jj];
            }
            fin = fR[0 + si];
            for (int j = 1; j <= order - 1; j++) fin = fin + DERs[j] * (pw(hs, j) / factorial[j]);
        } else {
            hs = ds - hs;
            for (int jj = 1; jj <= order - 1; jj++) {
                double t = 0.0;
                for (int j = -si; j <= si; j++) t = t + D[jj](j) * fR[1 + j + si];
                DERs[jj] = t / ds_power[jj];
            }
            fin = fR[1 + si];
            for (int j = 1; j <= order - 1; j++) fin = fin + DERs[j] * (pw(-hs, j) / factorial[j]);
        }
        return fin;
    }
    // tracers_to_corners (composition.f90:669-790).  With temperature tracers
    // (Tt != nullptr) the per-volume sums of Ttr are exact: every Ttr enters
    // as a 128-bit fixed-point integer (tracer_fixq) and the sum is rounded
    // once (tracer_fixd), so the result does not depend on the summation
    // order (the reference's depends on its OpenMP thread count).
    int tracers_to_corners(const std::vector<double>& rr, const std::vector<double>& ss, const double* Tt = nullptr,
                           const Arr* T0 = nullptr) {
        if (Tt) Tratio = *T0;  // empty volumes keep T0
        for (int t = 0; t <= ntype; t++) count_type[t].fill(0);
        int nth = 1;
#ifdef _OPENMP
        nth = omp_get_max_threads();
#endif
        int bad = 0;
        size_t plane = count_type[0].v.size();
        std::vector<int> work((size_t)nth * (ntype + 1) * plane, 0);
#pragma omp parallel reduction(| : bad)
        {
            int rank = 0;
#ifdef _OPENMP
            rank = omp_get_thread_num();
#endif
            int* my = &work[(size_t)rank * (ntype + 1) * plane];
#pragma omp for schedule(static)
            for (long id = 0; id < ntr; id++) {
                double r = rr[id], s = ss[id];
                int i = (int)std::lround(r / dr);
                int k = (int)std::lround(s / ds);
                if (r <= 0.0 || r >= p.aspect || s <= 0.0 || s >= 1.0) { bad = 1; continue; }
                int t = Ttype[id];
                my[(size_t)t * plane + (size_t)(i + span) + (size_t)(k + span) * count_type[0].ni] += 1;
            }
        }
        if (bad) return TC_ERR_TRACER_OUTSIDE;
        std::vector<__int128> tsum;
        if (Tt) {
            tsum.assign((size_t)(nx + 1) * (nz + 1), 0);
            for (long id = 0; id < ntr; id++) {
                int i = (int)std::lround(rr[id] / dr);
                int k = (int)std::lround(ss[id] / ds);
                tsum[(size_t)i + (size_t)k * (nx + 1)] += tracer_fixq(Tt[id]);
            }
        }
        for (int r = 0; r < nth; r++)
            for (int t = 0; t <= ntype; t++) {
                int* src = &work[((size_t)r * (ntype + 1) + t) * plane];
                for (size_t x = 0; x < plane; x++) count_type[t].v[x] += src[x];
            }
        for (int t = 0; t <= ntype; t++) {
            IArr& C = count_type[t];
            for (int i = 1; i <= span; i++)
                for (int k = 0; k <= nz; k++) { C(-i, k) = C(i, k); C(nx + i, k) = C(nx - i, k); }
            for (int k = 1; k <= span; k++)
                for (int i = 0; i <= nx; i++) { C(i, -k) = C(i, k); C(i, nz + k) = C(i, nz - k); }
        }
        nempty.fill(0);
        for (size_t x = 0; x < nempty.v.size(); x++) {
            int s = 0;
            for (int t = 0; t <= ntype; t++) s += count_type[t].v[x];
            nempty.v[x] = s;
        }
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                int ne = nempty(i, k);
                if (ne > 0)
                    for (int t = 1; t <= ntype; t++) {
                        int ct = count_type[t](i, k);
                        double& C = Cnew[t - 1](i, k);
                        if (ct == ne) C = 1.0;
                        else if (ct == 0) C = 0.0;
                        else C = (double)ct / (double)ne;
                    }
                if (Tt && ne > 0) Tratio(i, k) = tracer_fixd(tsum[(size_t)i + (size_t)k * (nx + 1)]) / (double)ne;
            }
        if (comp == 1) {
            for (int t = 0; t < ntype; t++) enforceBCs_comp(Cnew[t]);
            if (smooth_vis == 1) { int st = smoother_time(); if (st) return st; }
        }
        if (Tt) {
            enforceBCs(Tratio);
            if (smooth_vis == 1) { int st = smoother_time_T(Tratio); if (st) return st; }
        }
        load_conductivity_array();
        return TC_OK;
    }

    // extendT (energy.f90:478-499): Textend for the tracers' conduction term
    void extendT(const Arr& T0) {
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) Textend(i, k) = T0(i, k);
        for (int i = 1; i <= spanT; i++)
            for (int k = 0; k <= nz; k++) { Textend(-i, k) = Textend(i, k); Textend(nx + i, k) = Textend(nx - i, k); }
        for (int k = 1; k <= spanT; k++)
            for (int i = -spanT; i <= nx + spanT; i++) {
                if (p.Tbot == 0) Textend(i, -k) = -(Textend(i, k) - 1.0) + 1.0;
                else if (p.Tbot == 1) Textend(i, -k) = Textend(i, k);
                Textend(i, nz + k) = -Textend(i, nz - k);
            }
        if (p.Tbot == 0)
            for (int i = -spanT; i <= nx + spanT; i++) Textend(i, 0) = 1.0;
        for (int i = -spanT; i <= nx + spanT; i++) Textend(i, nz) = 0.0;
    }
    // tracer_space (energy.f90:82-100): energy_space without advection, on Textend
    double tracer_space(int i, int k) const {
        double Tr = dotx(D1, span1, Textend, i, k) / dr, Ts = dotz(D1, span1, Textend, i, k) / ds;
        double Trr = dotx(D2, span1, Textend, i, k) / dr2, Tss = dotz(D2, span1, Textend, i, k) / ds2;
        double kx = conduct_r(i, k) / xr(i), kz = conduct_s(i, k) / zs(k);
        double Tx = Tr / xr(i), Tz = Ts / zs(k);
        double Txx = (Trr - Tx * xrr(i)) / sq(xr(i));
        double Tzz = (Tss - Tz * zss(k)) / sq(zs(k));
        return conduct(i, k) * (Txx + Tzz) + (kx * Tx + kz * Tz) + heating(i, k);
    }
    // load_tracer_space_array (energy.f90:102-115) + compute_derivatives of it
    void load_tracer_space_array() {
        extendT(Tratio);
        for (int i = -span_interp; i <= nx + span_interp; i++)
            for (int k = -span_interp; k <= nz + span_interp; k++) tsa(i, k) = tracer_space(i, k);
        compute_derivatives(tsa, DERr_tracer);
    }

    // =====================================================================
    // energy equation and time step
    // =====================================================================
    double heating(int i, int k) const {
        if (comp == 0) return p.H;
        double s = 0.0;
        for (int j = 0; j < ntype; j++) s = s + Cvis[j](i, k);
        double h = p.H * (1.0 - s);
        for (int j = 0; j < ntype; j++) h = p.Htype[j] * Cvis[j](i, k) + h;
        return h;
    }
    // energy_space (energy.f90:60-80)
    double energy_space(int i, int k, const Arr& T0) const {
        double Tr = dotx(D1, span1, T0, i, k) / dr, Ts = dotz(D1, span1, T0, i, k) / ds;
        double Trr = dotx(D2, span1, T0, i, k) / dr2, Tss = dotz(D2, span1, T0, i, k) / ds2;
        double kx = conduct_r(i, k) / xr(i), kz = conduct_s(i, k) / zs(k);
        double Tx = Tr / xr(i), Tz = Ts / zs(k);
        double Txx = (Trr - Tx * xrr(i)) / sq(xr(i));
        double Tzz = (Tss - Tz * zss(k)) / sq(zs(k));
        return conduct(i, k) * (Txx + Tzz) + (kx * Tx + kz * Tz) - u(i, k) * Tx - w(i, k) * Tz + heating(i, k);
    }
    // stability_RK4 (energy.f90:600-646), tracer=0
    int stability_RK4() {
        double Ts_max = Tr_base / ds, Tr_max = Tr_base / dr;
        double Tss_max = -Trr_base / ds2, Trr_max = -Trr_base / dr2;
        if (p.RaT != 0.0) {
            double eA_max = 0.0, eD_max = 0.0;
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k <= nz; k++) {
                    double eA = std::fabs(-(conduct(i, k) * xrr(i) / std::pow(xr(i), 3.0)) - u(i, k) / xr(i) + conduct_r(i, k) / sq(xr(i))) * Tr_max +
                                std::fabs(-(conduct(i, k) * zss(k) / std::pow(zs(k), 3.0)) - w(i, k) / zs(k) + conduct_s(i, k) / sq(zs(k))) * Ts_max;
                    double eD = conduct(i, k) * (std::fabs(Trr_max / sq(xr(i))) + std::fabs(Tss_max / sq(zs(k))));
                    if (eA > eA_max) eA_max = eA;
                    if (eD > eD_max) eD_max = eD;
                }
            double dtA, dtD;
            if (p.torder == 2) {
                if (eA_max >= eD_max) return TC_ERR_RK2_STABILITY;
                dtA = 1.0 / eA_max; dtD = 2.0 / eD_max;
            } else {
                dtA = 2.8 / eA_max; dtD = 2.8 / eD_max;
            }
            if (eA_max == 0.0) dt = dtD;
            else dt = 1.0 / (1.0 / dtA + 1.0 / dtD);
        } else dt = p.dt_manual;
        dt = p.courant * dt;
        return TC_OK;
    }
    int update_velocities() {  // momentum.f90:64-76 (iterate=1)
        int st = multigrid();
        if (st) return st;
        compute_velocities();
        return TC_OK;
    }
    void energy_stage(const Arr& Tin, int stage, double factor, const Arr& T0, Arr& Tout) {
        // stage 1: T=temp; Tout=T0+factor*temp.  stages 2,3: T=T+2*temp; Tout=T0+factor*temp.
        // stage 4: T = T0 + (dt/6)*(T+temp).
#pragma omp parallel for schedule(static)
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                double temp = energy_space(i, k, Tin);
                if (stage == 1) { T(i, k) = temp; Tout(i, k) = T0(i, k) + factor * temp; }
                else if (stage == 4) { T(i, k) = T0(i, k) + factor * (T(i, k) + temp); }
                else { T(i, k) = T(i, k) + 2.0 * temp; Tout(i, k) = T0(i, k) + factor * temp; }
            }
    }
    // =====================================================================
    // tracer repositioning, TRA (composition.f90:7-580)
    // =====================================================================
    // initial mzran seeds of each OpenMP thread (basics.f90:198-212)
    void seed_ranks() {
        sd_i.assign(eq_T, 0); sd_j.assign(eq_T, 0); sd_k.assign(eq_T, 0); sd_n.assign(eq_T, 0);
        sd_i[0] = 521288629; sd_j[0] = 362436069; sd_k[0] = 16163801; sd_n[0] = 1131199299;
        for (int j = 1; j < eq_T; j++) {
            int32_t r = sd_i[j - 1] - sd_k[j - 1];
            if (r < 0) r += 2147483579;
            sd_i[j] = sd_j[j - 1];
            sd_j[j] = sd_k[j - 1];
            sd_k[j] = r;
            sd_n[j] = (int32_t)(69069u * (uint32_t)sd_n[j - 1] + 1013904243u);
        }
    }
    // mzran (composition.f90:7-20); 32-bit integers wrap
    double mzran(int rank) {
        int32_t r = sd_i[rank] - sd_k[rank];
        if (r < 0) r += 2147483579;
        sd_i[rank] = sd_j[rank];
        sd_j[rank] = sd_k[rank];
        sd_k[rank] = r;
        sd_n[rank] = (int32_t)(69069u * (uint32_t)sd_n[rank] + 1013904243u);
        r = (int32_t)((uint32_t)r + (uint32_t)sd_n[rank]);
        return 0.5 + (0.2328306e-9) * (double)r;
    }
    // shuffle_serial (composition.f90:22-34) on a(istart:N), `a` indexed absolutely
    void shuffle_serial(int* a, int istart, int N, int rank) {
        for (int i = istart; i <= N - 1; i++) {
            const double ran = mzran(rank);
            const int r = (int)std::floor(ran * (double)(N - i)) + i + 1;
            std::swap(a[i], a[r]);
        }
    }
    // iterations of thread t in a static-schedule OpenMP loop over N iterations
    void omp_static(int N, int t, int& lo, int& cnt) const {
        const int q = N / eq_T, r = N % eq_T;
        if (t < r) { cnt = q + 1; lo = t * cnt; } else { cnt = q; lo = t * q + r; }
    }
    int minval_masked(const std::vector<int>& nex, int t, bool use_type) const {
        int m = 2147483647;  // Fortran minval of an empty selection: HUGE
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                const int v = nex[(size_t)i * (nz + 1) + k];
                if (v > 0) continue;
                if (use_type) {
                    if (t == 0) {
                        double sC = 0.0;
                        for (int j = 0; j < ntype; j++) sC = sC + Cnew[j](i, k);
                        if (sC != 0.0) continue;
                    } else if (Cnew[t - 1](i, k) != 1.0) continue;
                }
                m = std::min(m, v);
            }
        return m;
    }
    int maxloc_type(int i, int k) {
        int best = 0;
        for (int t = 1; t <= ntype; t++)
            if (count_type[t](i, k) > count_type[best](i, k)) best = t;
        return best;
    }
    // equalize_tracers (composition.f90:83-580) with eq_T OpenMP threads
    int equalize_tracers() {
        const int NT = ntype + 1, NR = eq_T;
        const size_t ncell = (size_t)(nx + 1) * (nz + 1);
        auto C = [&](int i, int k) { return (size_t)i * (nz + 1) + k; };
        std::vector<long> Nideal(NT, 0);
        if (comp == 1) {
            long s = 0;
            for (int t = 1; t <= ntype; t++) { Nideal[t] = std::lround(Cinit[t - 1] * (double)ntr); s += Nideal[t]; }
            Nideal[0] = ntr - s;
        } else Nideal[0] = ntr;
        // ---- excess tracers per corner volume ----
        std::vector<int> nex(ncell, 0), tpc_type(NT, 0);
        if (comp == 0) {
            tpc_type[0] = p.tpc;
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k <= nz; k++) nex[C(i, k)] = (nempty(i, k) > 0) ? nempty(i, k) - p.tpc : 0;
        } else {
            for (int t = 0; t <= ntype; t++) {
                long cnt = 0, sum = 0;
                for (int i = 0; i <= nx; i++)
                    for (int k = 0; k <= nz; k++) {
                        bool m;
                        if (t == 0) {
                            double sC = 0.0;
                            for (int j = 0; j < ntype; j++) sC = sC + Cnew[j](i, k);
                            m = (sC == 0.0);
                        } else m = (Cnew[t - 1](i, k) == 1.0);
                        if (m) { cnt++; sum += count_type[t](i, k); }
                    }
                tpc_type[t] = (cnt > 0) ? (int)std::lround((double)sum / (double)cnt) : 0;
            }
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k <= nz; k++) {
                    nex[C(i, k)] = 0;
                    for (int t = 0; t <= ntype; t++) {
                        bool all = true;
                        for (int a = -1; a <= 1 && all; a++)
                            for (int b = -1; b <= 1 && all; b++)
                                if (count_type[t](i + a, k + b) != nempty(i + a, k + b)) all = false;
                        if (all && nempty(i, k) > 0) { nex[C(i, k)] = nempty(i, k) - tpc_type[t]; break; }
                    }
                }
        }
        long nfree = 0;
        bool allzero = true;
        for (size_t c = 0; c < ncell; c++) { if (nex[c] > 0) nfree += nex[c]; if (nex[c] != 0) allzero = false; }
        eq_row.clear();
        if (allzero) return TC_OK;
        nequalize++;
        // ---- tracer ids by corner volume, ascending, then shuffled ----
        std::vector<long> off(ncell + 1, 0);
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) off[C(i, k) + 1] = nempty(i, k);
        for (size_t c = 0; c < ncell; c++) off[c + 1] += off[c];
        std::vector<int> ids((size_t)off[ncell] + 1, 0), counter(ncell, 0);
        for (long id = 0; id < ntr; id++) {
            const int i = (int)std::lround(rtr[id] / dr), k = (int)std::lround(str[id] / ds);
            const size_t c = C(i, k);
            counter[c]++;
            ids[(size_t)off[c] + counter[c] - 1] = (int)id + 1;  // Fortran ids
        }
        auto list = [&](size_t c) { return &ids[(size_t)off[c]] - 1; };  // list(c)[1..counter]
        for (int t = 0; t < NR; t++) {
            int lo, cnt;
            omp_static(nx + 1, t, lo, cnt);
            for (int i = lo; i < lo + cnt; i++)
                for (int k = 0; k <= nz; k++) shuffle_serial(list(C(i, k)), 1, counter[C(i, k)], t);
        }
        // ---- temperature interpolant (temperature tracers) ----
        Arr Tdumb;
        std::vector<Arr> DERr_T;
        if (tracer == 1) {
            extendT(Tratio);
            const int si = span_interp;
            Tdumb.alloc(-si, nx + si, -si, nz + si);
            for (int i = -si; i <= nx + si; i++)
                for (int k = -si; k <= nz + si; k++) Tdumb(i, k) = Textend(i, k);
            DERr_T.assign(order, Arr());
            for (int j = 1; j <= order - 1; j++) DERr_T[j].alloc(0, nx, -si, nz + si);
            compute_derivatives(Tdumb, DERr_T);
        }
        // ---- donor tracers ----
        const size_t cap = (size_t)nfree + 1;
        std::vector<int> donor((size_t)NR * NT * cap, 0);
        auto D = [&](int rank, int t) { return &donor[((size_t)rank * NT + t) * cap]; };  // D(rank,t)[1..]
        std::vector<int> isv((size_t)NR * NT, 0), isv2;
        auto IS = [&](int rank, int t) -> int& { return isv[(size_t)rank * NT + t]; };
        auto take = [&](size_t c, int rank, bool near_wall_only, bool near_wall) {
            if (nex[c] <= 0) return;
            for (int q = 1; q <= counter[c]; q++) {
                const int ID = list(c)[q];
                const double r = rtr[ID - 1], sv = str[ID - 1];
                const bool nw = (sv < dist_s) || (sv > 1.0 - dist_s) || (r < dist_r) || (r > p.aspect - dist_r);
                if (near_wall_only && nw != near_wall) continue;
                const int t = Ttype[ID - 1];
                IS(rank, t) = IS(rank, t) + 1;
                D(rank, t)[IS(rank, t)] = ID;
                nex[c] = nex[c] - 1;
                if (nex[c] == 0) break;
            }
        };
        auto edges = [&](bool near_wall) {
            for (int i = 0; i <= nx; i += nx) {  // left and right columns, split over k
                for (int t = 0; t < NR; t++) {
                    int lo, cnt;
                    omp_static(nz + 1, t, lo, cnt);
                    for (int k = lo; k < lo + cnt; k++) take(C(i, k), t, true, near_wall);
                }
                if (nx == 0) break;
            }
            for (int k = 0; k <= nz; k += nz) {  // bottom and top rows, corners done, split over i
                for (int t = 0; t < NR; t++) {
                    int lo, cnt;
                    omp_static(nx - 1, t, lo, cnt);
                    for (int i = 1 + lo; i < 1 + lo + cnt; i++) take(C(i, k), t, true, near_wall);
                }
                if (nz == 0) break;
            }
        };
        edges(true);
        for (int t = 0; t < NR; t++)
            for (int tt = 0; tt < NT; tt++) shuffle_serial(D(t, tt), 1, IS(t, tt), t);
        isv2 = isv;
        edges(false);
        for (int t = 0; t < NR; t++) {  // interior volumes, split over i
            int lo, cnt;
            omp_static(nx - 1, t, lo, cnt);
            for (int i = 1 + lo; i < 1 + lo + cnt; i++)
                for (int k = 1; k <= nz - 1; k++) take(C(i, k), t, false, false);
        }
        std::vector<int> nfree_rank = isv;  // count(donor > 0) per rank and type
        long found = 0;
        for (int v : nfree_rank) found += v;
        if (found != nfree) return TC_ERR_EQUALIZE;
        for (int t = 0; t < NR; t++)
            for (int tt = 0; tt < NT; tt++)
                shuffle_serial(D(t, tt), isv2[(size_t)t * NT + tt] + 1, IS(t, tt), t);
        // ---- lottery: donors to the poorest volumes ----
        std::vector<int> nx_loop(nx + 1), nz_loop(nz + 1);
        for (int i = 0; i <= nx; i++) nx_loop[i] = i;
        for (int k = 0; k <= nz; k++) nz_loop[k] = k;
        std::fill(isv.begin(), isv.end(), 0);
        std::vector<long> tcount(NT, 0);
        auto count_all = [&]() {
            for (int t = 0; t < NT; t++) {
                long s = 0;
                for (int i = 0; i <= nx; i++)
                    for (int k = 0; k <= nz; k++) s += count_type[t](i, k);
                tcount[t] = s;
            }
        };
        auto all_ideal = [&]() { for (int t = 0; t < NT; t++) if (tcount[t] != Nideal[t]) return false; return true; };
        std::vector<int> minex(NT, 0);
        auto minexcess = [&](bool reference_typo) {
            minex[0] = (tpc_type[0] > 0) ? minval_masked(nex, 0, comp == 1) : 0;
            for (int t = 1; t <= ntype; t++)
                minex[t] = ((reference_typo ? tpc_type[0] : tpc_type[t]) > 0) ? minval_masked(nex, t, true) : 0;
        };
        auto place = [&](int rank, int t, int i, int k) -> int {
            const double r = dr * (double)i, sv = ds * (double)k;
            double pr = mzran(rank), ps = mzran(rank);
            pr = (pr - 0.5) * dr;
            ps = (ps - 0.5) * ds;
            IS(rank, t) = IS(rank, t) + 1;
            const int ID = D(rank, t)[IS(rank, t)];
            double& R = rtr[ID - 1];
            double& S = str[ID - 1];
            R = r + pr;
            S = sv + ps;
            if (R <= 0.0) R = dist_r;
            if (R >= p.aspect) R = p.aspect - dist_r;
            if (S <= 0.0) S = dist_s;
            if (S >= 1.0) S = 1.0 - dist_s;
            return ID;
        };
        long sum_nfree = 0;
        for (int v : nfree_rank) sum_nfree += v;
        auto sum_isv = [&]() { long s = 0; for (int v : isv) s += v; return s; };
        int escape = 0;
        count_all();
        if (all_ideal()) escape = 1;
        int tt_priv[1024];  // each thread's private tt keeps its value across cells and passes
        for (int t = 0; t < NR; t++) tt_priv[t] = 0;
        for (;;) {
            if (escape == 0) { count_all(); if (all_ideal()) escape = 1; }
            minexcess(false);
            bool allz = true;
            for (int t = 0; t < NT; t++) if (minex[t] != 0) allz = false;
            if (allz) break;
            if (sum_isv() >= nfree) break;
            isv2 = isv;
            shuffle_serial(nx_loop.data(), 0, nx, 0);
            shuffle_serial(nz_loop.data(), 0, nz, 0);
            for (int rank = 0; rank < NR; rank++) {
                int lo, cnt;
                omp_static(nx + 1, rank, lo, cnt);
                for (int ii = lo; ii < lo + cnt; ii++) {
                    const int i = nx_loop[ii];
                    for (int kk = 0; kk <= nz; kk++) {
                        const int k = nz_loop[kk];
                        const int type_save = maxloc_type(i, k);
                        int& tt = tt_priv[rank];
                        if (escape == 0) {
                            for (int q = 0; q < NT; q++) if (tcount[q] > Nideal[q]) { tt = q; break; }
                        } else tt = type_save;
                        const size_t c = C(i, k);
                        if (nex[c] == minex[type_save] && IS(rank, tt) < nfree_rank[(size_t)rank * NT + tt] && nex[c] < 0) {
                            const int ID = place(rank, tt, i, k);
                            if (comp == 1) Ttype[ID - 1] = type_save;
                            count_type[tt](i, k) = count_type[tt](i, k) - 1;
                            count_type[Ttype[ID - 1]](i, k) = count_type[Ttype[ID - 1]](i, k) + 1;
                            nex[c] = nex[c] + 1;
                        }
                    }
                }
            }
            if (isv == isv2) break;
        }
        // ---- remaining donors in serial, alternating between ranks ----
        int rk = 0;
        for (;;) {
            minexcess(true);
            bool allz = true;
            for (int t = 0; t < NT; t++) if (minex[t] != 0) allz = false;
            if (allz) break;
            if (sum_isv() >= nfree) break;
            isv2 = isv;
            rk = 0;
            shuffle_serial(nx_loop.data(), 0, nx, 0);
            shuffle_serial(nz_loop.data(), 0, nz, 0);
            for (int ii = 0; ii <= nx; ii++) {
                const int i = nx_loop[ii];
                for (int kk = 0; kk <= nz; kk++) {
                    const int k = nz_loop[kk];
                    const int tt = maxloc_type(i, k);
                    long used = 0, avail = 0;
                    for (int q = 0; q < NR; q++) { used += IS(q, tt); avail += nfree_rank[(size_t)q * NT + tt]; }
                    const size_t c = C(i, k);
                    if (nex[c] == minex[tt] && used < avail && nex[c] < 0) {
                        for (;;) {
                            rk = rk + 1;
                            if (rk == NR) rk = 0;
                            if (IS(rk, tt) < nfree_rank[(size_t)rk * NT + tt]) break;
                        }
                        const int ID = place(rk, tt, i, k);
                        if (comp == 1) Ttype[ID - 1] = maxloc_type(i, k);
                        nex[c] = nex[c] + 1;
                    }
                }
            }
            if (isv == isv2) break;
        }
        // ---- temperatures of the moved tracers ----
        if (tracer == 1)
            for (int t = 0; t < NR; t++)
                for (int tt = 0; tt < NT; tt++)
                    for (int q = 1; q <= IS(t, tt); q++) {
                        const int ID = D(t, tt)[q];
                        Ttr[ID - 1] = interpolate(rtr[ID - 1], str[ID - 1], DERr_T, Tdumb);
                    }
        // ---- the equalize.dat row (composition.f90:545-574) ----
        if (comp == 0) minex[0] = minval_masked(nex, 0, false);
        else for (int t = 0; t <= ntype; t++) minex[t] = minval_masked(nex, t, true);
        long deficit = 0;
        for (size_t c = 0; c < ncell; c++) if (nex[c] <= 0) deficit += nex[c];
        eq_row.clear();
        eq_row.push_back(NT);
        for (int t = 0; t < NT; t++) eq_row.push_back(comp == 0 ? p.tpc : tpc_type[t]);
        for (int t = 0; t < NT; t++) eq_row.push_back(minex[t]);
        eq_row.push_back(deficit);
        eq_row.push_back(sum_isv());
        eq_row.push_back(nfree);
        count_all();
        for (int t = 0; t < NT; t++) eq_row.push_back(tcount[t]);
        (void)sum_nfree;
        smooth_vis = 0;
        int st = tracers_to_corners(rtr, str, tracer == 1 ? Ttr.data() : nullptr, &T);
        smooth_vis = 1;
        return st;
    }

    // energy_time (energy.f90:117-453) for comp = 0 or 1, tracer = 0 or 1,
    // local_time = 0, equalize = 0.
    int energy_time() {
        int st = stability_RK4();
        if (st) return st;
        if (p.equalize == 1) { st = equalize_tracers(); if (st) return st; }
        std::vector<Arr> C0 = Cnew;
        const bool tt = (tracer == 1);
        const bool trc = (comp == 1) || tt;
        const bool rat = (p.RaT != 0.0);
        Arr T0 = tt ? Tratio : T;
        Arr T1 = T, T2 = T;
        if (tt) Ttr0 = Ttr;
        if (trc) { rtr0 = rtr; str0 = str; }
        auto derivs = [&]() { compute_derivatives(u, DERr_u); compute_derivatives(w, DERr_w); };
        // tracers_to_corners of a stage with temperature tracers, then tracer_space
        auto t2c_T = [&](const std::vector<double>& rr, const std::vector<double>& ss, const std::vector<double>& Tt,
                         bool reset_C) -> int {
            if (reset_C && comp == 1) Cnew = C0;
            int s2 = tracers_to_corners(rr, ss, Tt.data(), &T0);
            if (s2) return s2;
            load_tracer_space_array();
            return TC_OK;
        };
        // ---- stage 1 ----
        if (rat) {
            if (tt) load_tracer_space_array();
            else { energy_stage(T0, 1, 0.5 * dt, T0, T1); enforceBCs(T1); }
        }
        if (trc) {
            derivs();
            double dtstage = (p.torder == 2) ? dt : 0.5 * dt;
#pragma omp parallel for schedule(static)
            for (long id = 0; id < ntr; id++) {
                double tr = tr_vel(rtr0[id], str0[id]);
                double ts = ts_vel(rtr0[id], str0[id]);
                rtr[id] = tr; str[id] = ts;
                double tT = 0.0;
                if (tt) { tT = interpolate(rtr0[id], str0[id], DERr_tracer, tsa); Ttr[id] = tT; }
                rtr1[id] = rtr0[id] + dtstage * tr;
                str1[id] = str0[id] + dtstage * ts;
                if (tt) Ttr1[id] = Ttr0[id] + dtstage * tT;
            }
        }
        // ---- stage 2 ----
        if (tt) { st = t2c_T(rtr1, str1, Ttr1, false); if (st) return st; }
        if (p.RK_update == 1) {
            if (comp == 1 && !tt) { st = tracers_to_corners(rtr1, str1); if (st) return st; }
            if (!tt) { st = smoother_time_T(T1); if (st) return st; }
            st = update_velocities(); if (st) return st;
            if (trc) derivs();
        }
        if (rat && !tt) {
            energy_stage(T1, 2, 0.5 * dt, T0, T2);
            enforceBCs(T2);
        }
        if (trc) {
            double dtstage = 0.5 * dt;
#pragma omp parallel for schedule(static)
            for (long id = 0; id < ntr; id++) {
                double tr = tr_vel(rtr1[id], str1[id]);
                double ts = ts_vel(rtr1[id], str1[id]);
                double tT = tt ? interpolate(rtr1[id], str1[id], DERr_tracer, tsa) : 0.0;
                if (p.torder == 2) {
                    rtr[id] = rtr[id] + tr; str[id] = str[id] + ts;
                    if (tt) Ttr[id] = Ttr[id] + tT;
                    rtr[id] = rtr0[id] + dtstage * rtr[id];
                    str[id] = str0[id] + dtstage * str[id];
                    if (tt) Ttr[id] = Ttr0[id] + dtstage * Ttr[id];
                } else {
                    rtr[id] = rtr[id] + 2.0 * tr; str[id] = str[id] + 2.0 * ts;
                    if (tt) Ttr[id] = Ttr[id] + 2.0 * tT;
                    rtr2[id] = rtr0[id] + dtstage * tr;
                    str2[id] = str0[id] + dtstage * ts;
                    if (tt) Ttr2[id] = Ttr0[id] + dtstage * tT;
                }
            }
        }
        if (p.torder >= 3) {
            // ---- stage 3 ----
            if (tt) { st = t2c_T(rtr2, str2, Ttr2, true); if (st) return st; }
            if (p.RK_update == 1) {
                if (comp == 1 && !tt) { Cnew = C0; st = tracers_to_corners(rtr2, str2); if (st) return st; }
                if (!tt) { st = smoother_time_T(T2); if (st) return st; }
                st = update_velocities(); if (st) return st;
                if (trc) derivs();
            }
            if (rat && !tt) {
                energy_stage(T2, 3, dt, T0, T1);
                enforceBCs(T1);
            }
            if (trc) {
                double dtt = dt;
#pragma omp parallel for schedule(static)
                for (long id = 0; id < ntr; id++) {
                    double tr = tr_vel(rtr2[id], str2[id]);
                    rtr[id] = rtr[id] + 2.0 * tr;
                    rtr1[id] = rtr0[id] + dtt * tr;
                    double ts = ts_vel(rtr2[id], str2[id]);
                    str[id] = str[id] + 2.0 * ts;
                    str1[id] = str0[id] + dtt * ts;
                    if (tt) {
                        double tT = interpolate(rtr2[id], str2[id], DERr_tracer, tsa);
                        Ttr[id] = Ttr[id] + 2.0 * tT;
                        Ttr1[id] = Ttr0[id] + dtt * tT;
                    }
                }
            }
            // ---- stage 4 ----
            if (tt) { st = t2c_T(rtr1, str1, Ttr1, true); if (st) return st; }
            if (p.RK_update == 1) {
                if (comp == 1 && !tt) { Cnew = C0; st = tracers_to_corners(rtr1, str1); if (st) return st; }
                if (!tt) { st = smoother_time_T(T1); if (st) return st; }
                st = update_velocities(); if (st) return st;
                if (trc) derivs();
            }
            if (rat && !tt) {
                energy_stage(T1, 4, dt / 6.0, T0, T1);
                enforceBCs(T);
            }
            if (trc) {
                double dto6 = dt / 6.0;
#pragma omp parallel for schedule(static)
                for (long id = 0; id < ntr; id++) {
                    double tr = tr_vel(rtr1[id], str1[id]);
                    rtr[id] = rtr0[id] + dto6 * (rtr[id] + tr);
                    double ts = ts_vel(rtr1[id], str1[id]);
                    str[id] = str0[id] + dto6 * (str[id] + ts);
                    if (tt) {
                        double tT = interpolate(rtr1[id], str1[id], DERr_tracer, tsa);
                        Ttr[id] = Ttr0[id] + dto6 * (Ttr[id] + tT);
                    }
                }
            }
        }
        // ---- wrap up ----
        if (comp == 1) Cnew = C0;
        if (trc) { st = tracers_to_corners(rtr, str, tt ? Ttr.data() : nullptr, &T0); if (st) return st; }
        if (tt) T = Tratio;
        else { st = smoother_time_T(T); if (st) return st; }
        return TC_OK;
    }

    // =====================================================================
    // stats (basics.f90:236-403)
    // =====================================================================
    double integrate1Dx_row(const std::vector<double>& f) const {  // f(0:nx)
        double fint = 0.0;
        for (int i = 0; i <= nx - 1; i++) fint = fint + 0.5 * (f[i] * xr(i) + f[i + 1] * xr(i + 1)) * dr;
        return fint;
    }
    double integrate1Dz_col(const std::vector<double>& f, int kstart) const {
        double fint = 0.0;
        for (int k = kstart; k <= nz - 1; k++) fint = fint + 0.5 * (f[k] * zs(k) + f[k + 1] * zs(k + 1)) * ds;
        return fint;
    }
    template <class F>
    double integrate2D(F f, int kstart = 0) const {
        std::vector<double> fintx(nz + 1), row(nx + 1);
        for (int k = 0; k <= nz; k++) {
            for (int i = 0; i <= nx; i++) row[i] = f(i, k);
            fintx[k] = integrate1Dx_row(row);
        }
        return integrate1Dz_col(fintx, kstart);
    }
    void stats(tc_stats_row* row) {
        std::memset(row, 0, sizeof(*row));
        vis = vis_grid[1];
        compute_strain_rate_invariant();
        double strain_max = -1e300;
        for (int i = 0; i <= nx; i++) strain_max = std::max(strain_max, strain(i, nz));
        if (comp == 1) {
            for (int t = 0; t < ntype; t++) {
                const Arr& C = Cnew[t];
                row->Cavg[t] = integrate2D([&](int i, int k) { return C(i, k); }) / p.aspect;
            }
            if (tstep == 0) {
                for (int k = 0; k <= nz; k++) if (zgrid(ds * (double)k) <= p.dent) kent = k;
                for (int t = 0; t < ntype; t++) mass[t] = row->Cavg[t];
            }
            for (int t = 0; t < ntype; t++) {
                const Arr& C = Cnew[t];
                double fint = integrate2D([&](int i, int k) { return C(i, k); }, kent);
                row->ent[t] = fint / p.aspect / mass[t];
            }
        }
        if (comp == 1 || tracer == 1) {
            int empty = 0, mn = 1 << 30, mx = -(1 << 30);
            for (int i = 0; i <= nx; i++)
                for (int k = 0; k <= nz; k++) {
                    int v = nempty(i, k);
                    if (v == 0) empty++;
                    mn = std::min(mn, v); mx = std::max(mx, v);
                }
            row->empty_cells = empty; row->tracer_min = mn; row->tracer_max = mx;
        }
        double vrms = std::pow(integrate2D([&](int i, int k) { return sq(u(i, k)) + sq(w(i, k)); }) / p.aspect, 0.5);
        std::vector<double> rowv(nx + 1);
        for (int i = 0; i <= nx; i++) rowv[i] = sq(u(i, nz)) + sq(w(i, nz));
        double mobility = std::pow(integrate1Dx_row(rowv) / p.aspect, 0.5) / vrms;
        row->vrms = vrms; row->mobility = mobility; row->strain_max = strain_max;
        if (p.RaT != 0.0) {
            row->Tavg = integrate2D([&](int i, int k) { return T(i, k); }) / p.aspect;
            row->RaT_avg = integrate2D([&](int i, int k) { return p.RaT / conduct(i, k) / vis(i, k); }) / p.aspect;
            std::vector<double> a(nx + 1), b(nx + 1), c(nx + 1);
            for (int i = 0; i <= nx; i++) {
                double Tz_surf = dotz(D1, span1, T, i, nz) / ds / zs(nz);
                double Tz_bot = dotz(D1, span1, T, i, 0) / ds / zs(0);
                a[i] = -conduct(i, nz) * Tz_surf;
                b[i] = T(i, 0);
                c[i] = -conduct(i, 0) * Tz_bot;
            }
            row->Nu = integrate1Dx_row(a) / integrate1Dx_row(b);
            row->Nu_bot = integrate1Dx_row(c) / p.aspect;
            row->q1 = -(conduct(0, nz) * dotz(D1, span1, T, 0, nz)) / ds / zs(nz);
            row->q2 = -(conduct(nx, nz) * dotz(D1, span1, T, nx, nz)) / ds / zs(nz);
            row->q3 = -(conduct(nx, 0) * dotz(D1, span1, T, nx, 0)) / ds / zs(0);
            row->q4 = -(conduct(0, 0) * dotz(D1, span1, T, 0, 0)) / ds / zs(0);
        }
        row->time = time;
        row->tstep = tstep;
        row->n_eta = n_eta; row->n_temp = n_temp; row->eig_fine = eig_fine;
        if (time == 0.0 && p.equalize == 1)
            for (int t = 0; t < ntype; t++) Cinit[t] = row->Cavg[t];
        for (int t = 0; t < TC_MAX_TYPES; t++) row->n_comp[t] = n_comp[t];
    }

    // =====================================================================
    // state I/O
    // =====================================================================
    int upload(const double* Tin, const double* Cin, const double* SFin, const double* rin, const double* sin,
               const int32_t* tin, long n, const double* Ttr_in = nullptr) {
        if (!Tin || !SFin) return TC_ERR_ARG;
        if (comp == 1 && (n != ntr || !rin || !sin || !tin)) return TC_ERR_ARG;
        if (tracer == 1 && (n != ntr || !rin || !sin || !Ttr_in)) return TC_ERR_ARG;
        std::memcpy(T.v.data(), Tin, T.v.size() * sizeof(double));
        std::memcpy(SF.v.data(), SFin, SF.v.size() * sizeof(double));
        size_t plane = T.v.size();
        for (int t = 0; t < ntype; t++) {
            if (Cin) for (size_t x = 0; x < plane; x++) Cnew[t].v[x] = Cin[x * ntype + t];
            else Cnew[t].fill(0.0);
        }
        enforceBCs(T);
        enforceBCs_stream(1, SF);
        for (int t = 0; t < ntype; t++) enforceBCs_comp(Cnew[t]);
        for (int l = 2; l <= grids; l++) error[l].fill(0.0);
        int st;
        if (comp == 1 || tracer == 1) {
            std::memcpy(rtr.data(), rin, ntr * sizeof(double));
            std::memcpy(str.data(), sin, ntr * sizeof(double));
            for (long i = 0; i < ntr; i++) Ttype[i] = (comp == 1) ? tin[i] : 0;
            if (tracer == 1) std::memcpy(Ttr.data(), Ttr_in, ntr * sizeof(double));
            smooth_vis = 0;
            st = tracers_to_corners(rtr, str, tracer == 1 ? Ttr.data() : nullptr, &T);
            smooth_vis = 1;
            if (st) return st;
        }
        st = smoother_time_T(T); if (st) return st;
        if (comp != 0) { st = smoother_time(); if (st) return st; }
        load_conductivity_array();
        uploaded = true;
        return TC_OK;
    }
    void download(double* Tout, double* Cout, double* SFout, double* rout, double* sout, int32_t* tout) {
        if (Tout) std::memcpy(Tout, T.v.data(), T.v.size() * sizeof(double));
        if (SFout) std::memcpy(SFout, SF.v.data(), SF.v.size() * sizeof(double));
        if (Cout) {
            size_t plane = T.v.size();
            for (int t = 0; t < ntype; t++)
                for (size_t x = 0; x < plane; x++) Cout[x * ntype + t] = Cnew[t].v[x];
        }
        if (comp == 1 || tracer == 1) {
            if (rout) std::memcpy(rout, rtr.data(), ntr * sizeof(double));
            if (sout) std::memcpy(sout, str.data(), ntr * sizeof(double));
            if (tout) for (long i = 0; i < ntr; i++) tout[i] = Ttype[i];
        }
    }

    // field access for tests: returns pointer to the storage of a named field
    Arr* field(const char* name, int level, int type) {
        std::string s(name);
        auto L = [&](std::vector<Arr>& v) -> Arr* { return (level >= 1 && level < (int)v.size()) ? &v[level] : nullptr; };
        auto Ty = [&](std::vector<Arr>& v) -> Arr* { return (type >= 1 && type <= (int)v.size()) ? &v[type - 1] : nullptr; };
        if (s == "T") return &T;
        if (s == "SF") return &SF;
        if (s == "Tvis") return &Tvis;
        if (s == "Tbuoy") return &Tbuoy;
        if (s == "u") return &u;
        if (s == "w") return &w;
        if (s == "vis") return &vis;
        if (s == "strain") return &strain;
        if (s == "conduct") return &conduct;
        if (s == "conduct_r") return &conduct_r;
        if (s == "conduct_s") return &conduct_s;
        if (s == "dts_array") return &dts_array;
        if (s == "residual") return &residual;
        if (s == "Tratio") return tracer == 1 ? &Tratio : nullptr;
        if (s == "Textend") return tracer == 1 ? &Textend : nullptr;
        if (s == "tracer_space_array") return tracer == 1 ? &tsa : nullptr;
        if (s == "Cnew") return Ty(Cnew);
        if (s == "Cvis") return Ty(Cvis);
        if (s == "Cbuoy") return Ty(Cbuoy);
        if (s == "dt_vis") return L(dt_vis);
        if (s == "error") return L(error);
        if (s == "vis_grid") return L(vis_grid);
        if (s == "vis_x") return L(vis_x);
        if (s == "vis_z") return L(vis_z);
        if (s == "vis_xx") return L(vis_xx);
        if (s == "vis_zz") return L(vis_zz);
        if (s == "vis_xz") return L(vis_xz);
        if (s == "RHS") return L(RHS);
        if (s == "dt_stream") return L(dt_stream);
        if (s == "ratio") return L(ratio);
        if (s == "DERr_u") return (level >= 1 && level < (int)DERr_u.size()) ? &DERr_u[level] : nullptr;
        if (s == "DERr_w") return (level >= 1 && level < (int)DERr_w.size()) ? &DERr_w[level] : nullptr;
        return nullptr;
    }
};

}  // namespace

// ===========================================================================
// C API (prefix tco_, same meaning as the tc_ functions of tracer_gpu.h)
// ===========================================================================
extern "C" {

int tco_create(const tc_params* p, void** out) {
    if (!p || !out) return TC_ERR_ARG;
    Oracle* o = new Oracle();
    int st = o->create(p);
    if (st) { delete o; *out = nullptr; return st; }
    *out = o;
    return TC_OK;
}
int tco_destroy(void* h) { delete (Oracle*)h; return TC_OK; }
int tco_get_info(void* h, tc_info* info) {
    Oracle* o = (Oracle*)h;
    std::memset(info, 0, sizeof(*info));
    info->nx = o->nx; info->nz = o->nz; info->span = o->span; info->span_interp = o->span_interp;
    info->grids = o->grids; info->nsteps = o->nsteps; info->ntr = o->ntr;
    info->ngrid_coarse = o->ngrid_coarse; info->kl = o->kl; info->ku = o->ku;
    for (int l = 1; l <= o->grids && l <= 8; l++) { info->nx_grid[l - 1] = o->nx_grid[l]; info->nz_grid[l - 1] = o->nz_grid[l]; }
    info->dr = o->dr; info->ds = o->ds;
    return TC_OK;
}
int tco_upload_state(void* h, const double* T, const double* C, const double* SF, const double* r,
                     const double* s, const int32_t* tt, int64_t n) {
    return ((Oracle*)h)->upload(T, C, SF, r, s, tt, (long)n);
}
int tco_upload_state_ex(void* h, const double* T, const double* C, const double* SF, const double* r,
                        const double* s, const int32_t* tt, const double* Ttr, int64_t n) {
    return ((Oracle*)h)->upload(T, C, SF, r, s, tt, (long)n, Ttr);
}
// the last equalize.dat row: n = ntype+1, then tpc_type[n], minexcess[n],
// sum of deficits, tracers moved, nfree, count_display[n]; *len = 0 if the
// last call found nothing to move
int tco_equalize_row(void* h, int64_t* out, int32_t cap, int32_t* len) {
    Oracle* o = (Oracle*)h;
    if (!len || (int32_t)o->eq_row.size() > cap) return TC_ERR_ARG;
    for (size_t q = 0; q < o->eq_row.size(); q++) out[q] = o->eq_row[q];
    *len = (int32_t)o->eq_row.size();
    return TC_OK;
}
int tco_download_ttr(void* h, double* out) {
    Oracle* o = (Oracle*)h;
    if (o->tracer != 1 || !out) return TC_ERR_ARG;
    std::memcpy(out, o->Ttr.data(), o->ntr * sizeof(double));
    return TC_OK;
}
int tco_download_state(void* h, double* T, double* C, double* SF, double* r, double* s, int32_t* tt) {
    ((Oracle*)h)->download(T, C, SF, r, s, tt);
    return TC_OK;
}
int tco_set_clock(void* h, int32_t tstep, double time) {
    Oracle* o = (Oracle*)h; o->tstep = tstep; o->time = time; return TC_OK;
}
// W-cycle cap of later multigrid calls (tests that step a solve cycle by cycle)
int tco_set_max_cycles(void* h, int32_t n) {
    if (n < 1) return TC_ERR_ARG;
    ((Oracle*)h)->p.max_cycles = n;
    return TC_OK;
}
// copies up to cap entries of the last multigrid call's residual trace; returns its length
int tco_residual_trace(void* h, double* out, int32_t cap) {
    const Oracle* o = (const Oracle*)h;
    const int n = (int)o->res_trace.size();
    for (int i = 0; i < n && i < cap; i++) out[i] = o->res_trace[i];
    return n;
}
int tco_multigrid(void* h, int32_t* cycles) {
    Oracle* o = (Oracle*)h;
    int st = o->multigrid();
    if (cycles) *cycles = o->last_cycles;
    return st;
}
int tco_compute_velocities(void* h) { ((Oracle*)h)->compute_velocities(); return TC_OK; }
int tco_stats(void* h, tc_stats_row* row) { ((Oracle*)h)->stats(row); return TC_OK; }
int tco_energy_time(void* h, double* dt) {
    Oracle* o = (Oracle*)h;
    int st = o->energy_time();
    if (dt) *dt = o->dt;
    return st;
}
int tco_step(void* h, tc_stats_row* row, int32_t* cycles, double* dt_out) {
    Oracle* o = (Oracle*)h;
    o->cycles_acc = 0;
    int st = o->multigrid();
    if (cycles) *cycles = o->last_cycles;
    if (st) return st;
    o->compute_velocities();
    tc_stats_row tmp;
    o->stats(row ? row : &tmp);
    st = o->energy_time();
    if (cycles) *cycles = o->cycles_acc;
    if (st) return st;
    if (dt_out) *dt_out = o->dt;
    o->time = o->time + o->dt;
    o->tstep += 1;
    return TC_OK;
}
int tco_tracers_to_corners(void* h, const double* r, const double* s) {
    Oracle* o = (Oracle*)h;
    std::vector<double> rr(r, r + o->ntr), ss(s, s + o->ntr);
    return o->tracers_to_corners(rr, ss);
}
int tco_download_counts(void* h, int32_t* out) {
    Oracle* o = (Oracle*)h;
    size_t plane = o->count_type.empty() ? 0 : o->count_type[0].v.size();
    for (int t = 0; t <= o->ntype; t++)
        for (size_t x = 0; x < plane; x++) out[x * (o->ntype + 1) + t] = o->count_type[t].v[x];
    return TC_OK;
}
int tco_download_nempty(void* h, int32_t* out) {
    Oracle* o = (Oracle*)h;
    for (size_t x = 0; x < o->nempty.v.size(); x++) out[x] = o->nempty.v[x];
    return TC_OK;
}
// --- granular hooks used by the tests ---
int tco_field_shape(void* h, const char* name, int level, int type, int32_t* bounds4) {
    Arr* a = ((Oracle*)h)->field(name, level, type);
    if (!a) return TC_ERR_ARG;
    bounds4[0] = a->i0; bounds4[1] = a->i0 + a->ni - 1; bounds4[2] = a->k0; bounds4[3] = a->k0 + a->nk - 1;
    return TC_OK;
}
int tco_get_field(void* h, const char* name, int level, int type, double* out) {
    Arr* a = ((Oracle*)h)->field(name, level, type);
    if (!a) return TC_ERR_ARG;
    std::memcpy(out, a->v.data(), a->v.size() * sizeof(double));
    return TC_OK;
}
int tco_set_field(void* h, const char* name, int level, int type, const double* in) {
    Arr* a = ((Oracle*)h)->field(name, level, type);
    if (!a) return TC_ERR_ARG;
    std::memcpy(a->v.data(), in, a->v.size() * sizeof(double));
    return TC_OK;
}
int tco_compute_strain(void* h) { ((Oracle*)h)->compute_strain_rate_invariant(); return TC_OK; }
int tco_compute_viscosity(void* h, int level) { return ((Oracle*)h)->compute_viscosity(level); }
int tco_compute_rhs(void* h, int level) { ((Oracle*)h)->compute_RHS(level); return TC_OK; }
int tco_reference_residual(void* h, int level, double* out) {
    Oracle* o = (Oracle*)h; o->compute_reference_residual(level); *out = o->res_ref[level]; return TC_OK;
}
// residual of error(level) (after error(1) := SF when level==1 and from_sf)
int tco_residual(void* h, int level, int from_sf, double* out) {
    Oracle* o = (Oracle*)h;
    if (level == 1 && from_sf) o->error[1] = o->SF;
    int st = o->compute_residual(level, o->error[level], 1);
    *out = o->residual_mag[1];
    return st;
}
int tco_local_time_steps(void* h, int level) { ((Oracle*)h)->iterate_local_time_steps(level); return TC_OK; }
int tco_smoother_time_T(void* h) { Oracle* o = (Oracle*)h; return o->smoother_time_T(o->T); }
int tco_scalars(void* h, double* out8) {
    Oracle* o = (Oracle*)h;
    out8[0] = o->eig_fine; out8[1] = o->n_eta; out8[2] = o->n_temp; out8[3] = o->dt;
    out8[4] = o->delta_T; out8[5] = o->res_ref[1]; out8[6] = o->residual_mag[1]; out8[7] = o->last_cycles;
    return TC_OK;
}
// build_grid's metrics, layout of tc_grid_metrics: xr, xrr, xrrr, xrrrr, DERxr
// over -3..nx+3 (0 outside their ranges), the same for z
int tco_metrics(void* h, double* x5, double* z5) {
    Oracle* o = (Oracle*)h;
    const int nx = o->nx, nz = o->nz, si = o->span_interp;
    const size_t lx = (size_t)nx + 7, lz = (size_t)nz + 7;
    std::fill(x5, x5 + 5 * lx, 0.0);
    std::fill(z5, z5 + 5 * lz, 0.0);
    for (int i = -si; i <= nx + si; i++) { x5[i + 3] = o->xr(i); x5[lx + i + 3] = o->xrr(i); }
    for (int i = 0; i <= nx; i++) {
        x5[2 * lx + i + 3] = o->xrrr(i); x5[3 * lx + i + 3] = o->xrrrr(i); x5[4 * lx + i + 3] = o->DERxr[1](i);
    }
    for (int k = -si; k <= nz + si; k++) { z5[k + 3] = o->zs(k); z5[lz + k + 3] = o->zss(k); }
    for (int k = 0; k <= nz; k++) {
        z5[2 * lz + k + 3] = o->zsss(k); z5[3 * lz + k + 3] = o->zssss(k); z5[4 * lz + k + 3] = o->DERzs[1](k);
    }
    return TC_OK;
}

// build_grid's node coordinates: xg(-3:nx+3), zg(-3:nz+3)
int tco_coordinates(void* h, double* xg, double* zg) {
    Oracle* o = (Oracle*)h;
    for (int i = -3; i <= o->nx + 3; i++) xg[i + 3] = o->xg(i);
    for (int k = -3; k <= o->nz + 3; k++) zg[k + 3] = o->zg(k);
    return TC_OK;
}

int tco_eig_bases(void* h, double* out12) {
    Oracle* o = (Oracle*)h;
    double v[12] = {o->Tr_base, o->Trr_base, o->Trrr_base, o->Trrrr_base, o->Ts_base, o->Tss_base,
                    o->Tsss_base, o->Tssss_base, o->Trs_base, o->Trrss_base, o->Trss_base, o->Trrs_base};
    std::memcpy(out12, v, sizeof(v));
    return TC_OK;
}
int tco_fd_coefficients(void* h, double* out) {  // D1,D2,D3,D4 each (-span:span), then D(1..Dnumber,-si:si)
    Oracle* o = (Oracle*)h;
    int n = 2 * o->span + 1, c = 0;
    for (int j = -o->span; j <= o->span; j++) out[c++] = o->D1(j);
    for (int j = -o->span; j <= o->span; j++) out[c++] = o->D2(j);
    for (int j = -o->span; j <= o->span; j++) out[c++] = o->D3(j);
    for (int j = -o->span; j <= o->span; j++) out[c++] = o->D4(j);
    (void)n;
    for (int m = 1; m <= o->Dnumber; m++)
        for (int j = -o->span_interp; j <= o->span_interp; j++) out[c++] = o->D[m](j);
    return c;
}
// coarse band after Compute_Matrix_coarse (before factorisation) for tests
int tco_coarse_matrix(void* h, double* band, double* rowb) {
    Oracle* o = (Oracle*)h;
    o->Compute_Matrix_coarse();
    std::memcpy(band, o->Mc.data(), o->Mc.size() * sizeof(double));
    for (int i = 1; i <= o->ngrid_coarse; i++) rowb[i - 1] = o->RowB[i];
    return TC_OK;
}
// stage positions for tests: which = 0 rtr,1 str,2 rtr0,3 str0,4 rtr1,5 str1,6 rtr2,7 str2
int tco_get_tracers(void* h, int which, double* out) {
    Oracle* o = (Oracle*)h;
    std::vector<double>* v[8] = {&o->rtr, &o->str, &o->rtr0, &o->str0, &o->rtr1, &o->str1, &o->rtr2, &o->str2};
    if (which < 0 || which > 7 || v[which]->size() != (size_t)o->ntr) return TC_ERR_ARG;
    std::memcpy(out, v[which]->data(), o->ntr * sizeof(double));
    return TC_OK;
}
int tco_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
    return n;
#else
    (void)n; return 1;
#endif
}
int tco_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
}  // extern "C"
