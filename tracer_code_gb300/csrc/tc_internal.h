// tc_internal.h -- device state layout and kernel launchers of the GB300 path.
//
// Layout in HBM.  Every field of multigrid level l (1 = finest) is a 2-D FP64
// array over the ghost-padded index box (-SP:nx_l+SP, -SP:nz_l+SP), SP=2
// (span of the order-2 stencils), stored column-major with i fastest and the
// row length padded to a multiple of 32 doubles (256 B) so every k-row starts
// on an L2-sector boundary:  addr(i,k) = (i+SP) + (k+SP)*ld.  Arrays that the
// reference declares with a smaller box (interior-only coefficients, u/w with
// span_interp=1, DERr with i in 0:nx) use the same mapping, so one index
// function serves every kernel.  Tracer arrays are flat FP64/int32 vectors in
// reference id order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "tracer_gpu.h"

#define SP 2
#define TC_MAXLEV 6
#define TC_NCOEF 13
#define TC_MAX_RED_BLOCKS 8192
#define TC_WIN 4  // W-cycle changes kept by the windowed correction

// 13-point stencil offsets used by the folded operator, in this order.
#define TC_OFFSETS_DI {0, -1, 1, -2, 2, 0, 0, 0, 0, -1, 1, -1, 1}
#define TC_OFFSETS_DK {0, 0, 0, 0, 0, -1, 1, -2, 2, -1, -1, 1, 1}

struct Lay {
    int a, b;     // nx_l, nz_l
    int ld, nk;   // padded row length, number of rows (b+1+2SP)
    size_t plane; // ld*nk
};

#ifdef __CUDACC__
__host__ __device__ __forceinline__
#else
inline
#endif
size_t IX(const Lay& L, int i, int k) { return (size_t)(i + SP) + (size_t)(k + SP) * (size_t)L.ld; }

// Metrics of a stretched grid (grid.f90 build_grid): dx/dr and its
// r-derivatives at fine node i, with xr3 = xr**3 and xr4 = xr**4 as the host
// evaluates them, and dz/ds likewise at fine row k; every array is indexed
// [i + TC_MPAD] for i = -TC_MPAD..n+TC_MPAD.  on = 0: a uniform grid (xr = zs
// = 1, the others 0), where the kernels take their uniform-grid form.
#define TC_MPAD 3
struct Metric {
    const double *xr, *xrr, *xrrr, *xrrrr, *xr3, *xr4;
    const double *zs, *zss, *zsss, *zssss, *zs3, *zs4;
    // d(xr)/dr and d(zs)/ds at the nodes (the tracer metric interpolation,
    // composition.f90:921-936)
    const double *dxr, *dzs;
    int on;
    int gx, gz;  // gridX != 0, gridZ != 0: the tracer velocities are divided by the interpolated metric
};

// scaled eigenvalue bounds of one level (the reference's test_eigenvalues /
// iterate_local_time_steps preamble), for the stretched-grid eigenvalues
struct EigScaled {
    double Tr, Ts, Trr, Tss, Trrr, Tsss, Trrrr, Tssss, Trs, Trrs, Trss, Trrss;
};

// Per-level constants (grid spacings and scaled eigenvalue bounds).
struct LevConst {
    double dr, ds, dr2, ds2, dr3, ds3, dr4, ds4, drds, drds2, dr2ds, dr2ds2;
    // eigR constants: K1 = Trr-Tss, K2 = Trrrr+Tssss, Trrss, Trs ; eigI: K5 = Trrr+Trss, K6 = Tsss+Trrs
    double eK1, eK2, eTrrss, eTrs, eK5, eK6;
    // folded-operator basis: for each offset d, (Srr-Sss, Srrrr+Sssss, Srrss, Srs, Srrr+Srss, Ssss+Srrs)
    double fold[TC_NCOEF][6];
    double dtvis_scale;  // unused placeholder
    // reciprocals of dr, ds, dr2, ds2, drds; recip = 1 when all five spacings
    // are powers of two, so that x * (1/h) equals x / h exactly and the
    // viscosity-filter kernels multiply instead of dividing
    double rdr, rds, rdr2, rds2, rdrds;
    int recip;
    // stretched grids: the metrics, this level's stride into the fine grid
    // (node i of the level is fine node i * mf) and the unreduced bounds
    Metric M;
    int mf;
    EigScaled e;
};

// Stretched-grid operator: the 13 tap coefficients are sum_q w[d][q] a_q(i,k)
// over the computational derivatives q = (Sr, Srr, Srrr, Srrrr, Ss, Sss, Ssss,
// Sssss, Srs, Srrs, Srss, Srrss), w[d][q] = the FD weight of q at tap d over
// its spacing, a_q = the coefficient of q in the operator at (i, k)
struct MetricFold {
    double w[TC_NCOEF][12];
};

// Scalars that kernels produce and the host reads back.
struct DevScalars {
    double ratio_min;
    double diff;
    double res_mag[TC_MAXLEV + 1];
    double res_ref;
    double dt;
    double eA_max, eD_max;
    double integ[32];
    double strain_max;
    int    nempty_min, nempty_max, empty_cells;
    int    flag_outside;     // tracer outside the domain
    int    flag_rk2;         // RK2 precondition failed
    int    lu_info;          // first zero pivot of the coarse LU (0 = none)
    int    visit_timeout;    // a fused visit's bounded neighbour wait gave up
    int    pad;
    double acc_alpha[2];     // coefficients of the last correction of psi (k_accel.cu)
    int    cyc_q;            // W-cycle count of the device-side multigrid loop (k_loop.cu)
    int    cyc_status;       // its stop reason: 0 converged, else the tc_status
    int    never_set;        // stays 0: the word the timeout-path tests wait on
    int    net_fail;         // the network's bounded-wait flag, copied after each forward pass
    // windowed correction (cycle_correction 3/4, k_accel.cu): coefficients of
    // the last correction (newest change first, the network's direction
    // last), stored changes, slot of the newest, directions used, and
    // whether the network's direction was one of them
    double win_beta[TC_WIN + 1];
    int    win_n, win_head, win_nd, win_dnn;
    // filter loops on the device (k_loop.cu): the factor of the next
    // smoothing step, the loop counters, the counts and the fine-level
    // eigenvalue ratio they report, and TC_ERR_LOOP_CAP when a loop hit
    // its cap
    double flt_c;
    double eig_fine;
    int    flt_n, flt_nn, flt_niter, flt_phase, flt_guard, flt_status;
    int    vis_nvis_store, vis_nn_store, n_eta, n_temp;
    int    n_comp[TC_MAX_TYPES];
    unsigned long long flt_launches;  // kernels run by the loops' WHILE bodies (the host adds them to its count)
};

// Arguments of the viscosity filter's device check (smoother_vis's tests)
struct VisFltArgs {
    int option, interpolate, ivis0, niter0;
    double eig_ratio_min, eig_ratio;
    long long cap;
    const double* tabA;  // factors of the first phase, by inner index 1..niter0
    const double* tabB;  // option 1 after the first outer pass (Niter 6, lb -2, la -1)
};

// Reduction scratch: per-block partials plus a completion counter.
struct RedScratch {
    double* part;         // [4][TC_MAX_RED_BLOCKS]
    unsigned int* count;  // [8]
};

// FP32 fold weights: coefficient d = sum_j w[d][j] G_j over the fields
// G = (eta_xx - eta_zz, eta, eta_xz, eta_x, eta_z); the entries outside
// kFoldG32Mask are zero for every uniform-grid stencil (checked on the host)
struct FoldG32 {
    float w[TC_NCOEF][5];
};
// tap d of the folded operator (centre, x offsets -1 1 -2 2, z offsets, the
// four diagonals) uses field j where bit j of the mask is set
#define TC_FOLD_G32_MASK {0x03u, 0x0bu, 0x0bu, 0x0bu, 0x0bu, 0x13u, 0x13u, 0x13u, 0x13u, 0x1eu, 0x1eu, 0x1eu, 0x1eu}

struct Level {
    Lay L;
    double* err[2];
    int ecur;
    double* vis[2];
    int vcur;
    double *vx, *vz, *vxx, *vzz, *vxz;
    double* bak[6];  // saved vis, vx, vz, vxx, vzz, vxz (compute_viscosity)
    double *dt_vis, *dt_stream, *ratio, *rhs, *res;
    double* coef;    // TC_NCOEF planes
    double *cA, *cB; // Chebyshev denominators for the level with finite eigenvalue ratios
    LevConst c;
    // FP32 copies for the mixed-precision solve (null unless solver_precision = 1):
    // coefficients, pseudo-time step and Chebyshev denominators rounded from
    // the FP64 ones; RHS, correction (two buffers) and residual in FP32
    float *coef32, *dts32, *cA32, *cB32, *rhs32, *res32;
    float* e32[2];
    int e32cur;
    // level 1 of the mixed solve: the five viscosity fields the folded
    // coefficients are made of (eta_xx - eta_zz, eta, eta_xz, eta_x, eta_z) in
    // FP32, and the fold weights that turn them into the 13 coefficients
    // inside the sweep (null: the sweep reads coef32)
    float* g32;
    FoldG32 gw;
    int use_g32;  // 1: the level's per-sweep FP32 smoother reads g32
    // launch configuration of this level's smoother, set by tc_autotune
    // (defaults: 32x8 blocks; fused visits wherever they fit)
    int sweep_bx, sweep_by;
    int fuse;       // 1 = one cluster launch per visit when the level fits, 0 = one launch per sweep
    int visit_cfg;  // shape of the fused visit: 0 = default, else 100*points per strip + CTAs
    int blk;        // when not fused: 0 = one k_sweep / k_sweep32 launch per sweep, n = n sweeps per k_sweep_blk launch
    MetricFold mfold;  // stretched grids: the tap weights of the computational derivatives
};

// Host-side scalars of the physics configuration, passed by value to kernels.
struct Phys {
    int nx, nz, ntype, comp, ivis, Tbot, Vbc, torder, tracer;
    double aspect, dr, ds, dr2, ds2, dro2, dso2;
    double rdr, rds;             // 1/dr, 1/ds rounded (tracer cell indices: quot_trunc, quot_nint)
    double RaT, RaC[TC_MAX_TYPES], lnvisT, lnvisP, lnvisC[TC_MAX_TYPES], visT2, H, Htype[TC_MAX_TYPES];
    double lncf[TC_MAX_TYPES];   // log(1/conduct_factor)
    double courantT, courantC;
    double Tr_max, Ts_max, Trr_max, Tss_max;  // stability_RK4 scaled bounds (finest grid)
    double visT, yield, yield_gradient, yield_depth;  // ivis = 3 (plastic)
    Metric M;                                         // stretched-grid metrics (M.on = 0: uniform)
};

// ---------------------------------------------------------------------------
// launchers (k_mg.cu)
// ---------------------------------------------------------------------------
void launch_visf_level1(cudaStream_t s, const Lay& L, const Phys& P, double* vis, const double* Tvis,
                        const double* const* Cvis, const double* zg, const double* T, const double* strain);
void launch_vis_grad(cudaStream_t s, const Level& lv, const double* vis, int do_eig, int ivis, RedScratch rs,
                     DevScalars* ds);
// cdev: when non-null the factor is read from the device (filter loop graph)
void launch_vis_smooth(cudaStream_t s, const Level& lv, const double* vin, double* vout, double c, int kmin,
                       int kmax, int RaT_nonzero, double visT2, const double* cdev = nullptr);
void launch_restrict_vis(cudaStream_t s, const Level& coarse, const Level& fine, const double* vfine, double* vcoarse);
void launch_vis_bcs_init(cudaStream_t s, const Level& coarse, double* v, int RaT_nonzero, double visT2);
void launch_level_coefs(cudaStream_t s, const Level& lv, const double* vis, int ivis, double courant_stream,
                        int cheb_level, bool with_dt = true);
void launch_sweep(cudaStream_t s, const Level& lv, const double* Sin, double* Sout, double c_uniform,
                  int per_point, double temp, int Vbc);
void launch_residual(cudaStream_t s, const Level& lv, const double* S, RedScratch rs, double* res_out);
// zero != null: also clears that plane (the coarse level's correction) in the same launch
void launch_restrict_res(cudaStream_t s, const Level& coarse, const Level& fine, const double* rf, double* rhs_c,
                         double* zero = nullptr);
void launch_prolong(cudaStream_t s, const Level& coarse, const Level& fine, const double* ec, double* ef, int Vbc);
void launch_stream_bcs(cudaStream_t s, const Level& lv, double* S, int Vbc);
void launch_coarse_build(cudaStream_t s, const Level& lv, double* band, double* rowb, int kl, int ku, int Vbc);
void launch_coarse_lu(cudaStream_t s, double* band, int* ipiv, int n, int kl, int ku, DevScalars* ds);
void launch_coarse_inverse(cudaStream_t s, const double* band, const int* ipiv, int n, int kl, int ku, double* Ainv,
                           double* bscratch);
void launch_coarse_solve(cudaStream_t s, const Level& lv, const double* band, const int* ipiv, const double* rowb,
                         int n, int kl, int ku, double* err, int Vbc);
void launch_coarse_solve32(cudaStream_t s, const Level& lv, const double* band, const int* ipiv, const double* rowb,
                           int n, int kl, int ku, float* err, int Vbc);
void launch_coarse_apply(cudaStream_t s, const Level& lv, const double* Ainv, const double* rowb, int n,
                         const int* cq, const int* cx, int m, double* err, int Vbc);
void launch_copy_plane(cudaStream_t s, double* dst, const double* src, size_t n);

// (k_visit.cu) one whole smoother visit of a small level as one cluster launch
int visit_cluster_setup();
int visit_cluster_fits(const Lay& L, int nsweeps, int fp32, int cfg = 0);
void launch_cheb_table(cudaStream_t s, const Level& lv, const double* tvals, int nsweeps, double* tab);
// grid transfers a visit can do in the same launch (nullptr = none): add the
// prolongation of the next coarser level's correction ec before the first
// sweep; after the last, restrict the residual into the coarser RHS rc and
// zero the coarser correction zc (zn values)
template <typename T>
struct VisitXfer {
    const T* ec = nullptr;
    Lay Lc{};
    T* rc = nullptr;
    Lay Lr{};
    T* zc = nullptr;
    size_t zn = 0;
};
// test_flag: the timeout-path test (tc_debug_wait_test); null in solves
int launch_visit_cluster(cudaStream_t s, const Level& lv, double* S, const double* cvals, const double* tvals,
                         const double* ctab, int nsweeps, int per_point, int Vbc, int* timeout_flag,
                         const VisitXfer<double>* x = nullptr, const int* test_flag = nullptr);
int launch_visit_cluster32(cudaStream_t s, const Level& lv, float* S, const double* cvals, const double* tvals,
                           int nsweeps, int per_point, int Vbc, int* timeout_flag,
                           const VisitXfer<float>* x = nullptr, const int* test_flag = nullptr);

// (k_subcycle.cu) the bottom of the W-cycle (smoothing of level S = grids-1
// and the coarsest solves between a restriction into S and the prolongation
// out of it) as precomputed FP64 n_S x n_S matrices M_k, k = coarse solves
// of the pattern; M[k-1] null where no pattern has k coarse solves.  The
// apply reads the level's RHS and writes its correction in the solver's
// precision (fp32: rhs32 / e32).
int subcycle_fits(const Lay& LS, const Lay& LG);
int launch_subcycle_build(cudaStream_t s, const Level& S, const Level& G, int fp32, const void* tab,
                          const void* ctab, int nsweeps, int per_point_down, const double* Ainv, const double* rowb,
                          const int* cq, const int* cx, int n, int m, int Vbc, int kmax, void* const* M,
                          float* Ac = nullptr);  // Ac: FP32 build with a compact FP32 coarse inverse (m x m)
void launch_subcycle_apply(cudaStream_t s, const Level& S, const void* M, int fp32, int m32, void* err, int Vbc);
void launch_cheb_table32(cudaStream_t s, const Level& lv, const double* tvals, int nsweeps, float* tab);

// (k_accel.cu) residual-minimising correction of the level-1 streamfunction along up to
// two directions: TC_ACCEL_DK = psi - prev (the last W-cycle's correction),
// TC_ACCEL_DNN = dnn (the network's predicted change); record_prev: prev =
// the corrected psi afterwards
enum { TC_ACCEL_NONE = 0, TC_ACCEL_DK = 1, TC_ACCEL_DNN = 2 };
void launch_accel(cudaStream_t s, const Level& l1, double* psi, double* prev, const double* dnn, int k1, int k2,
                  int record_prev, RedScratch rs, DevScalars* ds, int Vbc);
void launch_plane_diff(cudaStream_t s, double* dst, const double* a, const double* b, size_t n);
// windowed correction: the change d = psi - prev of the last W-cycle joins
// a window of the last TC_WIN changes (P, their images A d in AP; slots in
// ring order, ds->win_n / win_head), and psi moves to the minimiser of the
// L1-weighted residual over psi + span{window, dnn (when use_dnn)}; prev =
// the corrected psi.  ds->win_n = 0 starts a new window.
// rn: this cycle's residual RHS - A psi (written); rp: RHS - A prev (read,
// then replaced by the corrected psi's, by linearity); adnn = A dnn.
// launch_accel_window_init forms rp for the solve's start and adnn.
void launch_accel_window(cudaStream_t s, const Level& l1, double* psi, double* prev, double* P, double* AP,
                         double* rn, double* rp, const double* dnn, const double* adnn, int use_dnn, RedScratch rs,
                         DevScalars* ds, int Vbc);
void launch_accel_window_init(cudaStream_t s, const Level& l1, const double* prev, const double* dnn, double* rp,
                              double* adnn);

// (k_loop.cu) the multigrid convergence loop on the device: the cycle counter
// and the reference's tests after each level-1 visit, setting the condition
// of the CUDA-graph WHILE node that repeats the cycle
void launch_cycle_init(cudaStream_t s, DevScalars* ds);
// filter loops as WHILE graphs: smoother_time_T, smoother_time (one type),
// smoother_vis; each check follows a smoothness / grad_eig reduction and
// sets the condition (1: smooth once more and test again)
// (body: kernels in the WHILE body, added to ds->flt_launches per pass)
void launch_tflt_init(cudaStream_t s, DevScalars* ds);
void launch_tflt_check(cudaStream_t s, DevScalars* ds, double delta, long long cap, int body,
                       cudaGraphConditionalHandle cond);
void launch_cflt_init(cudaStream_t s, DevScalars* ds, int first_type);
void launch_cflt_check(cudaStream_t s, DevScalars* ds, int type, double delta, long long cap, const double* tab10,
                       const double* tab1, int body, cudaGraphConditionalHandle cond);
void launch_vflt_init(cudaStream_t s, DevScalars* ds, int reset_store, const VisFltArgs& a);
void launch_vflt_check(cudaStream_t s, DevScalars* ds, const VisFltArgs& a, int body,
                       cudaGraphConditionalHandle cond);
void launch_cycle_check(cudaStream_t s, DevScalars* ds, double tolerance, int max_cycles,
                        cudaGraphConditionalHandle cond);

// (k_mixed.cu) FP32 multigrid of the mixed-precision solve and its FP64 bridges
void launch_level_to_f32(cudaStream_t s, const Level& lv, int cheb);
void launch_level_g32(cudaStream_t s, const Level& lv, const double* vis);
bool fold_g32_weights(const LevConst& c, FoldG32* out);
void launch_sweep32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, float c_uniform, int per_point,
                    float temp, int Vbc);
void launch_residual32(cudaStream_t s, const Level& lv, const float* S);
// ns sweeps in one launch (k_sweepblk.cu); false if ns is not available
bool launch_sweep_blk32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, int ns, const float* c,
                        const float* temp, int per_point, int Vbc);
bool launch_sweep_blk64(cudaStream_t s, const Level& lv, const double* Sin, double* Sout, int ns, const double* c,
                        const double* temp, int per_point, int Vbc);
int sweep_blk_tiles(const Lay& L);  // CTAs of one launch of the tiled smoother
// ns = 2 or 3 sweeps of the level-1 field sweep (k_sweep_g32) per launch
// (k_sweep_gblk); false when the level has no fields or ns is not built
bool launch_sweep_gblk32(cudaStream_t s, const Level& lv, const float* Sin, float* Sout, int ns, const float* c,
                         const float* temp, int per_point, int Vbc);
void launch_restrict32(cudaStream_t s, const Level& coarse, const Level& fine, const float* rf, float* rhs_c,
                       float* zero = nullptr);
void launch_restrict64to32(cudaStream_t s, const Level& coarse, const Level& fine, const double* rf, float* rhs_c,
                           float* zero = nullptr);
void launch_prolong32(cudaStream_t s, const Level& coarse, const Level& fine, const float* ec, float* ef, int Vbc);
void launch_prolong_into64(cudaStream_t s, const Level& coarse, const Level& fine, const float* ec, double* S,
                           int Vbc);
void launch_residual_to32(cudaStream_t s, const Level& lv, const double* S, float* rhs32, float* zero = nullptr);
void launch_update64(cudaStream_t s, const Level& lv, double* S, const float* e, int Vbc);
void launch_coarse_apply32(cudaStream_t s, const Level& lv, const double* Ainv, const double* rowb, int n,
                           const int* cq, const int* cx, int m, float* err, int Vbc);
void launch_rhs1(cudaStream_t s, const Lay& L, const Phys& P, const double* Tbuoy, const double* const* Cbuoy,
                 double* rhs, RedScratch rs, DevScalars* ds);

// ---------------------------------------------------------------------------
// launchers (k_field.cu)
// ---------------------------------------------------------------------------
void launch_enforce_T(cudaStream_t s, const Lay& L, double* T, int Tbot);
void launch_enforce_comp(cudaStream_t s, const Lay& L, double* C, const double* Cprev_ghosts);
void launch_smoothness(cudaStream_t s, const Lay& L, const double* f, RedScratch rs, DevScalars* ds);
void launch_smooth_T_step(cudaStream_t s, const Lay& L, const Phys& P, const double* Tin, double* Tout,
                          const double* dts);
void launch_smooth_C_step(cudaStream_t s, const Lay& L, const Phys& P, const double* Cin, double* Cout,
                          const double* dts, double c, const double* cdev = nullptr);
void launch_conductivity(cudaStream_t s, const Lay& L, const Phys& P, const double* const* Cvis, double* conduct,
                         double* conduct_r, double* conduct_s);
void launch_velocities(cudaStream_t s, const Lay& L, const Phys& P, const double* SF, double* u, double* w);
void launch_derivatives(cudaStream_t s, const Lay& L, const Phys& P, const double* f, double* der);
void launch_stability(cudaStream_t s, const Lay& L, const Phys& P, const double* conduct, const double* conduct_r,
                      const double* conduct_s, const double* u, const double* w, double courant, double dt_manual,
                      RedScratch rs, DevScalars* ds);
void launch_energy_stage(cudaStream_t s, const Lay& L, const Phys& P, int stage, const double* Tin,
                         const double* T0, double* T, double* Tout, const double* conduct, const double* conduct_r,
                         const double* conduct_s, const double* u, const double* w, const double* const* Cvis,
                         const DevScalars* ds);
void launch_strain(cudaStream_t s, const Lay& L, const Phys& P, const double* u, const double* w, double* strain);
void launch_stats(cudaStream_t s, const Lay& L, const Phys& P, int kent, const double* T, const double* u,
                  const double* w, const double* conduct, const double* vis, const double* strain,
                  const double* const* Cnew, const int* nempty, double* rows, DevScalars* ds);

// ---------------------------------------------------------------------------
// launchers (k_tracer.cu)
// ---------------------------------------------------------------------------
void launch_tracer_stage(cudaStream_t s, const Lay& L, const Phys& P, int torder, int stage, int64_t ntr,
                         const double* rin, const double* sin, const double* r0, const double* s0, double* racc,
                         double* sacc, double* rout, double* sout, const double* u, const double* w,
                         const double* du, const double* dw, const DevScalars* ds, const double* tsa = nullptr,
                         const double* dT = nullptr, const double* Ttr0 = nullptr, double* Ttr = nullptr,
                         double* Tout = nullptr);
// counts per type and volume; with Tt (temperature tracers) also the exact
// per-volume sums of Tt into tsum (2 x L.plane words: low, high)
void launch_histogram(cudaStream_t s, const Lay& L, const Phys& P, int64_t ntr, const double* r, const double* sv,
                      const int* ttype, int* counts, DevScalars* ds, const double* Tt = nullptr,
                      unsigned long long* tsum = nullptr);
// cell sort of the tracer arrays (k_tracer.cu): rr/ss/tt/perm[/Tt] -> r2/s2/t2/p2[/T2]
void launch_sort_tracers(cudaStream_t s, const Lay& L, const Phys& P, int64_t ntr, const double* rr, const double* ss,
                         const int* tt, const int* perm, int* cnt, int* off, int* bsum, double* r2, double* s2,
                         int* t2, int* p2, const double* Tt = nullptr, double* T2 = nullptr);
// tracer repositioning (equalize_tracers): device buffers and sizes of one call
struct EqHost {
    Lay L;
    Phys P;
    int ntype, NR, comp, tracer, tpc;
    int64_t ntr;
    double dist_r, dist_s;
    long long Nideal[TC_MAX_TYPES + 1];
    int* counts;          // count_type planes (modified by the lottery)
    const int* nempty;
    double* const* Cnew;
    double *rtr, *str;    // slot order
    int* ttype;
    const int* perm;
    int *iperm, *nex, *off, *cur, *ids, *cnt, *bsum, *seeds, *isv, *isv2, *nfr, *nx_loop, *nz_loop;
    long long* sc;        // 64 scalars
    const double* Tratio; // temperature tracers
    double *Td, *dTd, *Ttr;
};
int launch_equalize_count(cudaStream_t s, const EqHost& H, int64_t* nfree, int* nonzero);
int launch_equalize_move(cudaStream_t s, const EqHost& H, int64_t nfree, int* donor, int64_t* row, int* row_len);
// extendT + tracer_space on (-1:nx+1, -1:nz+1) (temperature tracers)
void launch_tracer_space(cudaStream_t s, const Lay& L, const Phys& P, const double* Tratio, const double* conduct,
                         const double* conduct_r, const double* conduct_s, const double* const* Cvis, double* tsa);
void launch_perm_scatter(cudaStream_t s, int64_t n, const int* perm, const double* in, double* out);
void launch_perm_scatter(cudaStream_t s, int64_t n, const int* perm, const int* in, int* out);
void launch_perm_gather(cudaStream_t s, int64_t n, const int* perm, const double* in, double* out);
void launch_iota(cudaStream_t s, int64_t n, int* p);
void launch_counts_to_comp(cudaStream_t s, const Lay& L, const Phys& P, int* counts, int* nempty,
                           double* const* Cnew, const unsigned long long* tsum = nullptr, double* Tratio = nullptr);
