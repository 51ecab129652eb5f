// tc_setup.cpp -- host-side setup of a case (computed once per handle).
//
// Reference: multigrid_cycle.f90:1-99 (multigrid_setup + cycle tables) and
// :131-173 (compute_smoothing_parameters), iterative_solver.f90:1-61
// (optimize_grid), basics.f90:112-214 (compute_basics), main.f90:350-469
// (FD_coefficients, Fornberg's recurrence), energy.f90:501-598
// (derivative_eigenvalues), smoother.f90 stability_RK4_smoother /
// stability_vis_smoother, grid.f90:1-147 (uniform grid, zg ghosts).
#include "tc_setup.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>

namespace tcs {

const double kPi = 3.1415926535897932;

void optimize_grid(int& nx, int& nz, int& grids, int n_points_min) {
    int n_points_max = std::min(nx, nz);
    int n_coarse_min = 1, n_coarse_max = grids - 1;
    int n_max = n_points_max * (1 << n_coarse_max);
    int nxbig, n_in;
    if (nz <= nx) { nxbig = 1; n_in = nz; } else { nxbig = 0; n_in = nx; }
    int n_temp = n_max, n_coarse_temp = 0;
    for (int np = n_points_min; np <= n_points_max; np++)
        for (int nc = n_coarse_min; nc <= n_coarse_max; nc++) {
            int n = np * (1 << nc);
            if (n >= n_in && n < n_temp) { n_temp = n; n_coarse_temp = nc; }
        }
    grids = n_coarse_temp + 1;
    if (nxbig == 0) nx = n_temp; else nz = n_temp;
    n_in = (nz <= nx) ? nx : nz;
    int npt = (int)std::lround((double)n_in / (double)(1 << n_coarse_temp));
    n_temp = npt * (1 << n_coarse_temp);
    if (nxbig == 0) nz = n_temp; else nx = n_temp;
}

std::vector<int> cycle_table(int grids) {
    switch (grids) {
        case 2: return {1, 2};
        case 3: return {1, 2, 3, 2, 3, 2};
        case 4: return {1, 2, 3, 4, 3, 4, 3, 2, 3, 4, 3, 4, 3, 2};
        case 5: return {1, 2, 3, 4, 5, 4, 5, 4, 3, 4, 5, 4, 3, 2, 3, 4, 5, 4, 3, 4, 5, 4, 5, 4, 3, 2};
        case 6:
            return {1, 2, 3, 4, 5, 6, 5, 6, 5, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 3,
                    2, 3, 4, 5, 6, 5, 4, 3, 4, 5, 6, 5, 4, 5, 6, 5, 6, 5, 4, 3, 2};
        default: return {};
    }
}

// Fornberg weights on the nodes 0, 1, -1, 2, -2, ... (main.f90:350-446)
void fd_coefficients(int order, FD& fd) {
    const int Dnumber = order;
    const int bigM = std::max(4, Dnumber), bigN = order + bigM - 2;
    const int span = order / 2 + 1;
    std::vector<double> a(bigN + 1, 0.0);
    auto idx = [&](int m, int n, int i) { return (size_t)(m + 1) + (size_t)(bigM + 2) * ((size_t)n + (size_t)(bigN + 1) * i); };
    std::vector<double> delta((size_t)(bigM + 2) * (bigN + 1) * (bigN + 1), 0.0);
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
                delta[idx(m, n, i)] = (a[n] * delta[idx(m, n - 1, i)] - (double)m * delta[idx(m - 1, n - 1, i)]) / c3;
        }
        for (int m = 0; m <= std::min(n, bigM); m++)
            delta[idx(m, n, n)] = (c1 / c2) * ((double)m * delta[idx(m - 1, n - 1, n - 1)] - a[n - 1] * delta[idx(m, n - 1, n - 1)]);
        c1 = c2;
    }
    fd.span = span;
    for (int j = 0; j < 7; j++) { fd.D1[j] = fd.D2[j] = fd.D3[j] = fd.D4[j] = 0.0; }
    auto at = [&](double* D, int j) -> double& { return D[j + 3]; };
    at(fd.D1, 0) = delta[idx(1, order, 0)];
    at(fd.D2, 0) = delta[idx(2, order, 0)];
    k = 1;
    for (int i = 1; i <= order; i += 2) {
        at(fd.D1, k) = delta[idx(1, order, i)]; at(fd.D1, -k) = delta[idx(1, order, i + 1)];
        at(fd.D2, k) = delta[idx(2, order, i)]; at(fd.D2, -k) = delta[idx(2, order, i + 1)];
        k++;
    }
    at(fd.D3, 0) = delta[idx(3, order + 2, 0)];
    at(fd.D4, 0) = delta[idx(4, order + 2, 0)];
    k = 1;
    for (int i = 1; i <= order + 2; i += 2) {
        at(fd.D3, k) = delta[idx(3, order + 2, i)]; at(fd.D3, -k) = delta[idx(3, order + 2, i + 1)];
        at(fd.D4, k) = delta[idx(4, order + 2, i)]; at(fd.D4, -k) = delta[idx(4, order + 2, i + 1)];
        k++;
    }
    at(fd.D1, 0) = 0.0;
    at(fd.D3, 0) = 0.0;
    for (int i = 1; i <= span; i++) {
        at(fd.D1, i) = -at(fd.D1, -i); at(fd.D2, i) = at(fd.D2, -i);
        at(fd.D3, i) = -at(fd.D3, -i); at(fd.D4, i) = at(fd.D4, -i);
    }
}

// derivative_eigenvalues (energy.f90:501-598).  The reference's T_test builds
// each factor with CMPLX() of default kind, i.e. single precision, and
// multiplies them in single precision (energy.f90:597); that rounding is kept.
void derivative_eigenvalues(const FD& fd, int span1, EigBase& e) {
    const int n_angle = (1 << 11) + 1;
    const double d_angle = 2.0 * kPi / (double)(n_angle - 1);
    const int sp = fd.span, w = 2 * sp + 1;
    std::vector<std::complex<float>> fac((size_t)n_angle * w);
    for (int a = 1; a <= n_angle; a++) {
        double kr = (double)(a - 1) * d_angle;
        for (int j = -sp; j <= sp; j++)
            fac[(size_t)(a - 1) * w + (j + sp)] =
                std::complex<float>((float)std::cos(kr * (double)j), (float)std::sin(kr * (double)j));
    }
    auto D = [&](const double* Dv, int j) { return Dv[j + 3]; };
    auto Ttest = [&](int j, int jj, int a, int a2) -> std::complex<double> {
        std::complex<float> x = fac[(size_t)(a - 1) * w + (j + sp)];
        std::complex<float> y = fac[(size_t)(a2 - 1) * w + (jj + sp)];
        volatile float ac = x.real() * y.real(), bd = x.imag() * y.imag();
        volatile float ad = x.real() * y.imag(), bc = x.imag() * y.real();
        float re = ac - bd, im = ad + bc;
        return std::complex<double>((double)re, (double)im);
    };
    double Tr_max = 0, Trr_max = 0, Trrr_max = 0, Trrrr_max = 0, Trs_max = 0, Trrs_max = 0, Trrss_max = 0;
#pragma omp parallel for reduction(max : Tr_max, Trr_max, Trrr_max, Trrrr_max, Trs_max, Trrs_max, Trrss_max) schedule(static)
    for (int angle = 1; angle <= n_angle; angle++) {
        std::complex<double> Tr(0, 0), Trr(0, 0), Trrr(0, 0), Trrrr(0, 0), temp;
        for (int j = -span1; j <= span1; j++) {
            temp = Ttest(j, 0, angle, 1);
            Tr = Tr + D(fd.D1, j) * temp;
            Trr = Trr + D(fd.D2, j) * temp;
        }
        for (int j = -sp; j <= sp; j++) {
            temp = Ttest(j, 0, angle, 1);
            Trrr = Trrr + D(fd.D3, j) * temp;
            Trrrr = Trrrr + D(fd.D4, j) * temp;
        }
        std::complex<double> c0 = Ttest(0, 0, angle, 1);
        Tr = Tr / c0; Trr = Trr / c0; Trrr = Trrr / c0; Trrrr = Trrrr / c0;
        Tr_max = std::max(Tr_max, std::fabs(Tr.imag()));
        Trr_max = std::max(Trr_max, std::fabs(Trr.real()));
        Trrr_max = std::max(Trrr_max, std::fabs(Trrr.imag()));
        Trrrr_max = std::max(Trrrr_max, std::fabs(Trrrr.real()));
        for (int angle2 = 1; angle2 <= n_angle; angle2++) {
            std::complex<double> Trs(0, 0), Trrs(0, 0), Trrss(0, 0);
            for (int j = -span1; j <= span1; j++)
                for (int jj = -span1; jj <= span1; jj++) {
                    std::complex<double> t = Ttest(j, jj, angle, angle2);
                    Trs = Trs + (D(fd.D1, jj) * D(fd.D1, j)) * t;
                    Trrs = Trrs + (D(fd.D1, jj) * D(fd.D2, j)) * t;
                    Trrss = Trrss + (D(fd.D2, jj) * D(fd.D2, j)) * t;
                }
            Trs_max = std::max(Trs_max, std::fabs(Trs.real()));
            Trrs_max = std::max(Trrs_max, std::fabs(Trrs.imag()));
            Trrss_max = std::max(Trrss_max, std::fabs(Trrss.real()));
        }
    }
    e.Tr = Tr_max; e.Trr = Trr_max; e.Trrr = Trrr_max; e.Trrrr = Trrrr_max;
    e.Trs = Trs_max; e.Trrs = Trrs_max; e.Trrss = Trrss_max;
}

double pw(double x, int n) {  // x**n.d0 as gfortran evaluates it: x*x for n=2, libm pow otherwise
    if (n == 2) return x * x;
    if (n == 1) return x;
    return std::pow(x, (double)n);
}

void level_spacing(double aspect, int nxl, int nzl, LevSpacing& s) {
    s.dr = aspect / (double)nxl;
    s.ds = 1.0 / (double)nzl;
    s.dr2 = pw(s.dr, 2); s.ds2 = pw(s.ds, 2);
    s.dr3 = pw(s.dr, 3); s.ds3 = pw(s.ds, 3);
    s.dr4 = pw(s.dr, 4); s.ds4 = pw(s.ds, 4);
    s.drds = s.dr * s.ds; s.drds2 = s.dr * s.ds2; s.dr2ds = s.dr2 * s.ds; s.dr2ds2 = s.dr2 * s.ds2;
}

// Compute_Matrix_coarse with analysis=1 (iterative_solver.f90:1048-1070)
void coarse_bandwidth(int nxc, int nzc, int span, int span1, int& kl, int& ku) {
    int N = nzc + 1, n = (nxc + 1) * (nzc + 1);
    auto limit = [&](int j) { if (j == -span || j == span) return 0; if (j == 0) return span; return span1; };
    kl = 0; ku = 0;
    for (int p = 1; p <= n; p++) {
        int kp = p - N * ((p - 1) / N) - 1, ip = (p - 1) / N;
        for (int j = -span; j <= span; j++) {
            int iq = j + ip;
            if (iq > 0 && iq < nxc)
                for (int kq = -limit(j) + kp; kq <= kp + limit(j); kq++)
                    if (kq > 0 && kq < nzc) {
                        int q = N * iq + kq + 1, t = q - p;
                        ku = std::max(ku, t);
                        kl = std::max(kl, -t);
                    }
        }
    }
}

// xgrid / zgrid (grid.f90:1-35)
static double xgrid(double r, double aspect, int gridX, double spaceX, double Ax) {
    if (gridX == 1) return aspect * (Ax * std::atan(spaceX * (r / aspect - 0.5)) + 0.5);
    return r;
}
static double zgrid(double s, int nz, double ds, int gridZ, double spaceZ, double thickness, int nbound,
                    double Az) {
    if (gridZ == 1) return Az * std::atan(spaceZ * (s - 0.5)) + 0.5;
    if (gridZ == 2) {
        const double dzin = (1.0 - 2.0 * thickness) / (double)(nz - 2 * nbound + 2);
        const double s1 = (double)(nbound - 1) * ds, s2 = 1.0 - s1;
        const double scale = thickness / (std::exp(spaceZ * s1) - 1.0);
        if (s < s1) return scale * (std::exp(spaceZ * s) - 1.0);
        if (s > s2) return 1.0 - scale * (std::exp(-spaceZ * (s - 1.0)) - 1.0);
        return thickness + (s - s1) * dzin / ds;
    }
    return s;
}

void grid_metrics(double aspect, int nx, int nz, int gridX, int gridZ, double spaceX, double spaceZ,
                  double thickness, int nbound, const FD& fd, GridMetrics& g) {
    const int P = g.pad, span = 2, span1 = 1, si = 1;
    LevSpacing sp;
    level_spacing(aspect, nx, nz, sp);
    const double dr = sp.dr, ds = sp.ds;
    // basics.f90:140-141
    const double Ax = std::pow(std::atan(spaceX * 0.5) - std::atan(spaceX * (-0.5)), -1.0);
    const double Az = std::pow(std::atan(spaceZ * 0.5) - std::atan(spaceZ * (-0.5)), -1.0);
    auto alloc = [&](std::vector<double>& v, int n) { v.assign((size_t)n + 1 + 2 * P, 0.0); };
    for (auto* v : {&g.xg, &g.xr, &g.xrr, &g.xrrr, &g.xrrrr, &g.xr3, &g.xr4, &g.dxr}) alloc(*v, nx);
    for (auto* v : {&g.zg, &g.zs, &g.zss, &g.zsss, &g.zssss, &g.zs3, &g.zs4, &g.dzs}) alloc(*v, nz);
    auto X = [&](std::vector<double>& v, int i) -> double& { return v[(size_t)(i + P)]; };
    for (int i = 0; i <= nx; i++) X(g.xg, i) = xgrid(dr * (double)i, aspect, gridX, spaceX, Ax);
    for (int k = 0; k <= nz; k++) X(g.zg, k) = zgrid(ds * (double)k, nz, ds, gridZ, spaceZ, thickness, nbound, Az);
    for (int i = 1; i <= span + si; i++) {
        X(g.xg, -i) = -X(g.xg, i);
        X(g.xg, nx + i) = aspect - X(g.xg, nx - i) + aspect;
    }
    for (int k = 1; k <= span + si; k++) {
        X(g.zg, -k) = -X(g.zg, k);
        X(g.zg, nz + k) = 1.0 - X(g.zg, nz - k) + 1.0;
    }
    X(g.xg, 0) = 0.0; X(g.zg, 0) = 0.0; X(g.xg, nx) = aspect; X(g.zg, nz) = 1.0;
    // dot_product(D(-sp:sp), f(c-sp:c+sp)) in index order
    auto dot = [&](const double* D, int sp_, std::vector<double>& f, int c) {
        double s = 0.0;
        for (int j = -sp_; j <= sp_; j++) s = s + D[j + 3] * X(f, c + j);
        return s;
    };
    for (int i = 0; i <= nx; i++) {
        X(g.xrrr, i) = gridX != 0 ? dot(fd.D3, span, g.xg, i) / sp.dr3 : 0.0;
        X(g.xrrrr, i) = gridX != 0 ? dot(fd.D4, span, g.xg, i) / sp.dr4 : 0.0;
    }
    for (int i = -si; i <= nx + si; i++) {
        X(g.xr, i) = gridX != 0 ? dot(fd.D1, span1, g.xg, i) / dr : 1.0;
        X(g.xrr, i) = gridX != 0 ? dot(fd.D2, span1, g.xg, i) / sp.dr2 : 0.0;
        X(g.xr3, i) = std::pow(X(g.xr, i), 3.0);
        X(g.xr4, i) = std::pow(X(g.xr, i), 4.0);
    }
    for (int k = 0; k <= nz; k++) {
        X(g.zsss, k) = gridZ != 0 ? dot(fd.D3, span, g.zg, k) / sp.ds3 : 0.0;
        X(g.zssss, k) = gridZ != 0 ? dot(fd.D4, span, g.zg, k) / sp.ds4 : 0.0;
    }
    for (int k = -si; k <= nz + si; k++) {
        X(g.zs, k) = gridZ != 0 ? dot(fd.D1, span1, g.zg, k) / ds : 1.0;
        X(g.zss, k) = gridZ != 0 ? dot(fd.D2, span1, g.zg, k) / sp.ds2 : 0.0;
        X(g.zs3, k) = std::pow(X(g.zs, k), 3.0);
        X(g.zs4, k) = std::pow(X(g.zs, k), 4.0);
    }
    // compute_metric_interpolator_derivatives: D(1,-1:1) . xr(i-1:i+1) / dr**1
    for (int i = 0; i <= nx; i++) X(g.dxr, i) = dot(fd.D1, si, g.xr, i) / std::pow(dr, 1.0);
    for (int k = 0; k <= nz; k++) X(g.dzs, k) = dot(fd.D1, si, g.zs, k) / std::pow(ds, 1.0);
}

}  // namespace tcs
