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

}  // namespace tcs
