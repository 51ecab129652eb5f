// tc_setup.h -- host-side setup math of a case (see tc_setup.cpp).
#pragma once
#include <vector>

namespace tcs {

struct FD {
    int span;
    double D1[7], D2[7], D3[7], D4[7];  // index j+3, j in -3..3
};
struct EigBase {
    double Tr, Trr, Trrr, Trrrr, Trs, Trrs, Trrss;
};
struct LevSpacing {
    double dr, ds, dr2, ds2, dr3, ds3, dr4, ds4, drds, drds2, dr2ds, dr2ds2;
};

void optimize_grid(int& nx, int& nz, int& grids, int n_points_min);
std::vector<int> cycle_table(int grids);
void fd_coefficients(int order, FD& fd);
void derivative_eigenvalues(const FD& fd, int span1, EigBase& e);
double pw(double x, int n);
void level_spacing(double aspect, int nxl, int nzl, LevSpacing& s);
void coarse_bandwidth(int nxc, int nzc, int span, int span1, int& kl, int& ku);

// build_grid (grid.f90): node coordinates xg(i) = xgrid(i dr), zg(k) =
// zgrid(k ds) with the mirrored ghosts, and the metrics xr, xrr (D1, D2 over
// span1), xrrr, xrrrr (D3, D4 over span) and likewise for z, plus xr**3,
// xr**4, zs**3, zs**4 as libm pow evaluates them.  Every vector holds index
// -pad..n+pad at [i + pad].  gridX: 0 uniform, 1 arctan, 2 uniform through
// the metric path; gridZ: 0 uniform, 1 arctan, 2 boundary layers.
struct GridMetrics {
    int pad = 3;
    std::vector<double> xg, zg, xr, xrr, xrrr, xrrrr, xr3, xr4, zs, zss, zsss, zssss, zs3, zs4;
    std::vector<double> dxr, dzs;  // DERxr(1,i), DERzs(1,k) over 0..n (composition.f90:921-936)
};
void grid_metrics(double aspect, int nx, int nz, int gridX, int gridZ, double spaceX, double spaceZ,
                  double thickness, int nbound, const FD& fd, GridMetrics& g);

}  // namespace tcs
