/*
 * tracer_gpu.h -- C ABI of the GB300 (sm_103a) per-timestep hot path of
 * seantrim/tracer_code: variable-viscosity streamfunction multigrid solve,
 * Runge-Kutta tracer advection with grid-to-tracer Taylor interpolation, and
 * the tracer-ratio composition step.
 *
 * The reference is one Fortran program whose state lives in the modules
 * `basics` (basics.f90:1-35) and `arrays` (arrays.f90:1-19).  Its hot path is
 * called from main.f90:174-205 through four argument-less subroutines:
 *
 *     multigrid            iterative_solver.f90:79-173
 *     compute_velocities   momentum.f90:532-551
 *     stats                basics.f90:236-324
 *     energy_time          energy.f90:117-453
 *
 * This header replaces those four calls with handle-based entry points.  The
 * module state becomes an opaque handle (tc_handle) whose fields live in HBM;
 * host arrays cross the boundary only in tc_upload_state/tc_download_state.
 * A Fortran host binds these functions through ISO_C_BINDING (one interface
 * block per function in a small binding module) and maps a non-zero status
 * to `stop`, which is what the reference does at each of its error sites.
 *
 * Array conventions (identical to the reference's allocations, basics.f90:37-110):
 *   - FP64, Fortran column-major (i, the horizontal index, fastest);
 *   - T, SF        : (-span:nx+span, -span:nz+span), span = order/2+1;
 *   - Cnew         : (1:ntype, -span:nx+span, -span:nz+span), type fastest;
 *   - u, w         : (-span_interp:nx+span_interp, -span_interp:nz+span_interp);
 *   - rtr, str     : (1:ntr) FP64; Ttype : (1:ntr) int32 (0 = ambient);
 *   - ntr = (nx+1)*(nz+1)*tpc  (basics.f90:146).
 *
 * Every function returns a tc_status (0 = success).  Handles are independent
 * (an ensemble runs one handle per case); a handle is not re-entrant and is
 * used from one host thread at a time.  All device work of a handle is issued
 * on one CUDA stream (tc_set_stream).
 */
#ifndef TRACER_GPU_H
#define TRACER_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TC_MAX_TYPES 4
#define TC_ABI_VERSION 4

/* Status codes.  Each reference `stop` site has its own code. */
typedef enum tc_status {
    TC_OK = 0,
    TC_ERR_ARG = 1,              /* bad argument / null pointer / size mismatch          */
    TC_ERR_UNSUPPORTED = 2,      /* input combination outside the implemented path        */
    TC_ERR_MG_CYCLES = 3,        /* "Too Many Multigrid Cycles Needed" iterative_solver.f90:164-167 */
    TC_ERR_MG_RESIDUAL = 4,      /* "Abnormally High Residual Detected" iterative_solver.f90:275-278 */
    TC_ERR_TRACER_OUTSIDE = 5,   /* "Tracer advected outside of domain" composition.f90:709-712 */
    TC_ERR_RK2_STABILITY = 6,    /* "Advective Eigenvalues Exceed Diffusive" energy.f90:626-629 */
    TC_ERR_LOOP_CAP = 7,         /* a data-dependent smoothing loop hit its iteration cap   */
    TC_ERR_CUDA = 8,             /* a CUDA runtime error; see tc_last_error()               */
    TC_ERR_ALLOC = 9,            /* device or host allocation failed                        */
    TC_ERR_STATE = 10,           /* call order violated (e.g. step before upload)           */
    TC_ERR_SINGULAR = 11,        /* zero pivot in the coarsest-grid banded LU (DGBTRF INFO>0) */
    TC_ERR_TOO_LARGE = 12,       /* input larger than the fixed buffer of an allocation-free call */
    TC_ERR_DEVICE_TIMEOUT = 13,  /* a bounded wait inside a kernel gave up (the kernel returned; the
                                    handle's results are invalid, the CUDA context stays usable) */
    TC_ERR_EQUALIZE = 14         /* "# of donor tracers found inconsistent with nfree value"
                                    composition.f90:366-369 */
} tc_status;

/*
 * Inputs of main.f90:8-116 that the hot path reads.  Field names follow the
 * reference.  Fixed by this implementation (not parameters): Database=2,
 * iterate=1, local_time=0 (see tc_create).
 */
typedef struct tc_params {
    /* grid options (main.f90:9-21) */
    int32_t nx, nz;             /* cells; multigrid_setup may change them (optimize_grid) */
    double  aspect;
    int32_t order;              /* space order (even); the GPU path implements order=2   */
    int32_t gridX, gridZ;       /* 0 uniform; gridX 1 arctan; gridZ 1 arctan, 2 layers  */
    double  spaceX, spaceZ, thickness;
    int32_t nbound;
    /* velocity solver options (main.f90:23-34) */
    int32_t non_Newtonian;      /* 1: viscosity rebuilt every W-cycle (FP64 solver only)  */
    int32_t iterate_order;      /* 1 = Richardson/Chebyshev smoother                     */
    double  tolerance;          /* relative L1 residual for multigrid convergence       */
    int32_t Nmulti;             /* smoother sweeps per level visit                        */
    int32_t mingrid;
    int32_t grids;              /* max multigrid levels, 2..6                            */
    double  eig_ratio;
    int32_t vis_iter;
    int32_t max_cycles;
    /* time stepping (main.f90:36-50) */
    int32_t torder;             /* 2 or 4 (RK4 for the field T method, main.f90:37)     */
    double  courant, courantT, courantC, courant_stream;
    int32_t RK_update;
    double  dt_manual;
    /* tracers (main.f90:52-59) */
    int32_t comp;               /* 1 = compositional tracers                              */
    int32_t ntype;              /* enriched tracer types (1..TC_MAX_TYPES)                */
    int32_t tpc;                /* tracers per cell corner                                */
    double  dist_factor;
    /* initial and boundary conditions (main.f90:61-74) */
    int32_t Tbot, Vbc;
    double  dlayer, dent;
    /* buoyancy, heating, conductivity (main.f90:76-96) */
    double  RaT;
    double  RaC[TC_MAX_TYPES];
    double  H;
    double  conduct_factor[TC_MAX_TYPES];
    double  Htype[TC_MAX_TYPES];
    /* viscosity (main.f90:98-115) */
    double  eig_ratio_min;
    int32_t ivis;               /* 0 isoviscous, 1 T,z, 2 T,z,C, 3 T + plastic (oracle)  */
    double  visP, visT, delta_visT, yield, yield_gradient, yield_depth;
    double  visC[TC_MAX_TYPES];
    double  delta_visC[TC_MAX_TYPES];
    /* Multigrid coarse-level start (no reference input).  0 = the reference's
     * behaviour (iterative_solver.f90:120-160): a smoothed coarse level keeps
     * its previous correction as the starting guess when a new restricted
     * residual arrives.  1 = that correction restarts from zero (textbook
     * correction scheme).  With more than two levels the reference behaviour
     * stalls or diverges on high-contrast starts (e.g. 1024x256, visT=1e4). */
    int32_t mg_zero_coarse;
    /* No reference counterpart.  0 = every multigrid operation in FP64 with
     * the reference's arithmetic.  1 = mixed precision: the smoother, the
     * residuals of levels 2..grids-1 and the restrictions/prolongations
     * between them run in FP32, inside an FP64 defect-correction loop that
     * keeps the level-1 residual (and with it the convergence test), the
     * streamfunction and its updates in FP64; the coarsest direct solve
     * stays FP64.  The tolerance test is the reference's, so the solution
     * meets the same relative residual; cycle counts may differ. */
    int32_t solver_precision;
    /* No reference counterpart.  1 = start each multigrid solve from the
     * attached network's guess (tracer_nn.h) when its level-1 residual is
     * below that of the previous streamfunction; after 8 rejections in a row
     * the guess is offered on every 32nd solve only, until it is taken again
     * (the plain start is used alone meanwhile); 2 = always from the guess;
     * 3 = from the previous streamfunction plus the multiple of the
     * network's predicted change that minimises the residual's 2-norm:
     * alpha = <A d, r> / <A d, A d> with d = guess - SF and r = RHS - A SF,
     * so the start's residual never exceeds the previous streamfunction's
     * (alpha near 0 when the prediction does not help);
     * 0 = always from the previous streamfunction. */
    int32_t learned_guess;
    /* Passes of a separable (1,2,1)/4 filter applied to the network's
     * correction before it is added (removes grid-scale noise that the
     * BF16 output carries; 0 = none). */
    int32_t learned_smooth;
    /* No reference counterpart.  The tracer arrays are kept in the order of
     * the corner control volume each tracer is counted in: tc_energy_time
     * re-sorts them (a counting sort by cell) before its RK stages when
     * tstep is a multiple of this interval (0 = never).  Results do not
     * depend on it; every host-facing call keeps the reference's tracer
     * order.  Default 10. */
    int32_t tracer_sort_interval;
    /* Temperature tracers (main.f90:56): 0 = T is a grid field advanced by
     * energy_space; 1 = T is carried by the tracers (Ttr, Lagrangian
     * conduction + heating by tracer_space, energy.f90:82-115) and the grid
     * T is their per-volume mean (Tratio).  Works with comp = 0 or 1. */
    int32_t tracer;
    /* Tracer repositioning, TRA (equalize_tracers, composition.f90:83-580;
     * main.f90:55): 1 = before every energy_time, move the excess tracers of
     * over-full control volumes to the poorest volumes by the reference's
     * lottery.  Its random streams (mzran, one per OpenMP thread, seeded as
     * basics.f90:198-212) and its work split follow the reference run with
     * equalize_threads OpenMP threads (static schedule); 0 means 1. */
    int32_t equalize;
    int32_t equalize_threads;
    /* No reference counterpart.  1 = evaluate the bottom of each W-cycle --
     * the smoothing of level grids-1 and the coarsest direct solves between
     * a restriction into level grids-1 and the prolongation out of it -- as
     * one matrix-vector product with that sub-cycle's exact linear map,
     * built once per multigrid call (one column per interior unknown of
     * level grids-1).  Same iterates in exact arithmetic; only rounding
     * differs.  Needs mg_zero_coarse = 1 (otherwise the sub-cycle also
     * depends on the previous corrections), non_Newtonian = 0, grids >= 3,
     * at most 1024 interior unknowns on level grids-1 and a coarsest grid
     * solved by its explicit inverse; where these do not hold the cycle runs
     * as with 0.  0 = sweep by sweep (default). */
    int32_t mg_coarse_matrix;
    /* No reference counterpart: a correction after every level-1 visit.
     * 0 = none (the reference's cycle).  1 = the minimal-residual correction
     * of the level-1 streamfunction along its change over the last W-cycle
     * (psi now minus psi after the previous correction).  2 = the learned
     * coarse-level correction: the minimal-residual correction on the
     * two-dimensional space spanned by that change and the attached
     * network's predicted change of the solve (formed once per multigrid
     * call); it needs an attached network (without one it acts as 1).
     * 3 = the windowed correction: the minimiser over psi + the span of the
     * changes of the last four W-cycles (each stored with its image under
     * the operator; a change nearly in the span of the newer ones is
     * dropped), a Krylov acceleration of the W-cycle restarted at every
     * multigrid call.  4 = 3 with the network's direction added to the span
     * (without a network it acts as 3).  The coefficients minimise the
     * residual weighted by 1/|r| (one reweighted least-squares step towards
     * its L1 norm, the norm of the convergence test); the convergence test
     * is the reference's and is taken after the correction, so the solution
     * meets the same tolerance; cycle counts differ.  Not with
     * non_Newtonian = 1. */
    int32_t cycle_correction;
} tc_params;

/* One row of stats.dat (basics.f90:283-314) plus viscosity_smoother.dat
 * (basics.f90:316-322).  Arrays are indexed by type-1. */
typedef struct tc_stats_row {
    double  time, Tavg, vrms, Nu, Nu_bot, RaT_avg, mobility, strain_max, q1, q2, q3, q4;
    int32_t empty_cells, tracer_min, tracer_max, tstep;
    double  Cavg[TC_MAX_TYPES];
    double  ent[TC_MAX_TYPES];
    int32_t n_eta, n_temp;
    int32_t n_comp[TC_MAX_TYPES];
    double  eig_fine;
} tc_stats_row;

/* Derived sizes a caller needs to size its arrays. */
typedef struct tc_info {
    int32_t nx, nz;             /* after optimize_grid                                    */
    int32_t span, span_interp, grids, nsteps;
    int64_t ntr;
    int32_t ngrid_coarse, kl, ku;
    int32_t nx_grid[8], nz_grid[8];
    double  dr, ds;
} tc_info;

typedef struct tc_handle tc_handle;

/* Fills *p with the shipped main.f90 defaults, switched to the path this
 * library implements (comp=1, ntype=1, tracer=0, equalize=0, non_Newtonian=0,
 * ivis=2, torder=4).  Replaces the hard-coded input block main.f90:8-116. */
void tc_default_params(tc_params* p);

/* Setup: main.f90:118-136 (compute_smoothing_parameters, multigrid_setup,
 * compute_basics, storage, FD_coefficients, build_grid with restart=0 grid
 * coordinates, derivative_eigenvalues, stability_RK4_smoother,
 * stability_vis_smoother).  Allocates all device state for one case. */
tc_status tc_create(const tc_params* p, tc_handle** out);
tc_status tc_destroy(tc_handle* h);
tc_status tc_get_info(const tc_handle* h, tc_info* info);

/* All later device work of the handle is issued on `stream` (a cudaStream_t;
 * NULL = the legacy default stream). */
tc_status tc_set_stream(tc_handle* h, void* stream);

/* Restart-style state injection: the restart branch of build_grid
 * (grid.f90:55-96: enforceBCs(T), enforceBCs_stream(1,SF), enforceBCs_comp,
 * tracers_to_corners with smoothing off) followed by main.f90:137-143
 * (smoother_time_T(T), smoother_time, load_conductivity_array) and the
 * zeroed coarse-level corrections of main.f90:162.  Cnew may be NULL
 * (zero start).  Ttype may be NULL when comp=0. */
tc_status tc_upload_state(tc_handle* h, const double* T, const double* Cnew,
                          const double* SF, const double* rtr, const double* str,
                          const int32_t* Ttype, int64_t ntr);

/* Copies the state back in the same layouts (any pointer may be NULL). */
tc_status tc_download_state(tc_handle* h, double* T, double* Cnew, double* SF,
                            double* rtr, double* str, int32_t* Ttype);

/* tc_upload_state with the tracers' temperatures Ttr(1:ntr), required when
 * tracer = 1 (tc_upload_state then returns TC_ERR_ARG): build_grid's
 * restart branch reads rtr, str[, Ttype], Ttr (grid.f90:74-84) and
 * tracers_to_corners(rtr, str, Ttr, T) with smoothing off sets Tratio (the
 * per-volume tracer mean; empty volumes keep T).  Ttype may be NULL when
 * comp = 0 (all tracers ambient).  The per-volume sums of Ttr are exact
 * (128-bit fixed point, rounded once), so Tratio does not depend on the
 * order the tracers are summed in; the reference's FP64 sums depend on its
 * OpenMP thread count and differ from it by a few ulps. */
tc_status tc_upload_state_ex(tc_handle* h, const double* T, const double* Cnew, const double* SF,
                             const double* rtr, const double* str, const int32_t* Ttype,
                             const double* Ttr, int64_t ntr);
/* The equalize.dat values of the last tracer repositioning (equalize = 1,
 * composition.f90:559-574): out[0] = n = ntype+1, then tpc_type(0:ntype)
 * (tpc when comp = 0), minexcess(0:ntype), the sum of the deficits
 * (nexcess <= 0), the tracers moved, nfree and count_display(0:ntype);
 * *len = 0 when the last call found every volume on its target (the
 * reference then writes no row).  TC_ERR_ARG if cap is too small. */
tc_status tc_equalize_row(const tc_handle* h, int64_t* out, int32_t cap, int32_t* len);
/* Ttr(1:ntr) in the reference's tracer order (tracer = 1; TC_ERR_ARG otherwise). */
tc_status tc_download_tracer_temperature(tc_handle* h, double* Ttr);

/* The parameters the handle was created with (nx, nz as passed; tc_info has
 * the optimized grid). */
tc_status tc_get_params(const tc_handle* h, tc_params* p);

/* Restart files in the reference's format: one gfortran unformatted
 * sequential record each (4-byte little-endian length, payload, length;
 * records of 2^31 bytes or more return TC_ERR_TOO_LARGE, files that do not
 * hold exactly the expected record return TC_ERR_ARG).
 *
 * Trestart (print_restart main.f90:305-320, read by build_grid
 * grid.f90:56-65): xg(-3:nx+3), zg(-3:nz+3), then T if `thermal` (RaT /= 0),
 * then Cnew(1:ntype, field box) if ntype > 0 (comp = 1), then SF; T, SF on
 * (-2:nx+2, -2:nz+2), i fastest.  T and Cnew may be NULL when not written. */
tc_status tc_restart_write(const char* path, int32_t nx, int32_t nz, int32_t ntype, int32_t thermal,
                           const double* xg, const double* zg, const double* T, const double* Cnew,
                           const double* SF);
tc_status tc_restart_read(const char* path, int32_t nx, int32_t nz, int32_t ntype, int32_t thermal,
                          double* xg, double* zg, double* T, double* Cnew, double* SF);

/* restart_tracers (main.f90:321-330, grid.f90:74-84): rtr(ntr), str(ntr),
 * then Ttype(ntr) when Ttype is not NULL (comp = 1) and Ttr(ntr) when Ttr
 * is not NULL (tracer = 1); at least one of the two. */
tc_status tc_restart_tracers_write(const char* path, int64_t ntr, const double* rtr, const double* str,
                                   const int32_t* Ttype, const double* Ttr);
tc_status tc_restart_tracers_read(const char* path, int64_t ntr, double* rtr, double* str, int32_t* Ttype,
                                  double* Ttr);

/* The reference's text outputs as gfortran writes them (host only).
 *
 * tc_format_g: one real under the edit descriptor Gw.d (e = 0) or Gw.dEe
 * into out[0..w] (w characters and a NUL); returns w, or -1 for arguments
 * out of range (w 1..200, d 1..60, e 0..9).
 *
 * tc_format_stats_line: the stats.dat row of basics.f90:283-314 for
 * local_time = 0 (the branches on comp, tracer and RaT = 0 included):
 * '(12(g20.8))', '(12(g20.8),3(i6))', '(12(g20.8),3(i6),10(g20.8))', ... with
 * Cavg and ent of types 1..ntype.  tc_format_vis_line: the
 * viscosity_smoother.dat row of basics.f90:316-322 (empty when RaT = 0 and
 * comp = 0, where the reference writes none).  Both write a NUL-terminated
 * line without its newline; TC_ERR_TOO_LARGE if it does not fit in cap. */
int32_t tc_format_g(double x, int32_t w, int32_t d, int32_t e, char* out);
/* The equalize.dat row '(g20.8,15(i10))' (composition.f90:568-574) of a
 * tc_equalize_row result at `time`. */
tc_status tc_format_equalize_line(double time, const int64_t* row, int32_t len, char* buf, int32_t cap);
tc_status tc_format_stats_line(const tc_stats_row* row, int32_t comp, int32_t tracer, int32_t ntype, double RaT,
                               char* buf, int32_t cap);
tc_status tc_format_vis_line(const tc_stats_row* row, int32_t comp, int32_t ntype, double RaT, char* buf,
                             int32_t cap);

/* snapshots (main.f90:237-270): the T1xxxx file for the handle's current
 * state, one '(9(g14.5E3),i6,20(g14.5E3))' line per node (xg, zg, T, SF, u,
 * w, strain, vis, Tvis, nempty, Cnew(1:ntype), Cvis(1:ntype); the comp = 0
 * and RaT = 0 forms as the reference has them), i outer, k inner, and a
 * list-directed blank record after each i.  Call it where the reference
 * calls snapshots: after tc_stats (strain and the level-1 viscosity are
 * the ones stats used). */
tc_status tc_write_snapshot(tc_handle* h, const char* path);

/* build_grid's uniform coordinates with the ghost mirrors and exact end
 * nodes (grid.f90:46-54, 97-108): xg(-3:nx+3), zg(-3:nz+3). */
void tc_restart_grid(int32_t nx, int32_t nz, double aspect, double* xg, double* zg);

/* build_grid's metrics for the grid of `p` (p->nx, p->nz as given; host
 * only, no device needed): x5 receives five arrays of nx+7 doubles, xr, xrr,
 * xrrr, xrrrr and DERxr (composition.f90:921-936), each at [i + 3]; z5 the
 * same five for z over nz+7.  Entries outside the reference's ranges (xr,
 * xrr: -1..nx+1; the others 0..nx) are 0. */
tc_status tc_grid_metrics(const tc_params* p, double* x5, double* z5);

/* build_grid's node coordinates of a handle (grid.f90:37-109, restart = 0:
 * xgrid(i dr), zgrid(k ds) with the mirrored ghosts), xg[i + 3] for i =
 * -3..nx+3 and zg[k + 3] for k = -3..nz+3; on a uniform grid they equal
 * tc_restart_grid's. */
tc_status tc_grid_coordinates(const tc_handle* h, double* xg, double* zg);

/* print_restart for a handle: downloads the state and writes Trestart (and
 * restart_tracers when comp = 1 or tracer = 1 and `tracers` is not NULL),
 * the coordinates from tc_grid_coordinates. */
tc_status tc_write_restart(tc_handle* h, const char* trestart, const char* tracers);

/* build_grid's restart branch for a handle: reads Trestart (and
 * restart_tracers when comp = 1 or tracer = 1; then `tracers` must not be
 * NULL) and uploads them with tc_upload_state_ex.  The file's xg, zg are read and
 * dropped: the handle keeps the grid its parameters build (tc_grid_coordinates). */
tc_status tc_read_restart(tc_handle* h, const char* trestart, const char* tracers);

/* Module clock: basics::tstep and basics::time, owned by the host loop. */
tc_status tc_set_clock(tc_handle* h, int32_t tstep, double time);

/* multigrid (iterative_solver.f90:79-173): solves for SF; *cycles_out
 * (may be NULL) receives the number of multigrid cycles q. */
tc_status tc_multigrid(tc_handle* h, int32_t* cycles_out);

/* compute_velocities (momentum.f90:532-551) with velocityBCs. */
tc_status tc_compute_velocities(tc_handle* h);

/* stats (basics.f90:236-324): one stats.dat row. */
tc_status tc_stats(tc_handle* h, tc_stats_row* row);

/* energy_time (energy.f90:117-453): one RK step of T, tracers and C,
 * including the multigrid re-solves between stages (RK_update=1).
 * *dt_out (may be NULL) receives dt. */
tc_status tc_energy_time(tc_handle* h, double* dt_out);

/* One pass of the main.f90:174-205 loop body: multigrid, compute_velocities,
 * stats, energy_time, time += dt, tstep += 1.  *cycles receives the W-cycles
 * of all multigrid solves of the step (the main solve and the RK re-solves).
 * row, cycles and dt_out may be NULL. */
tc_status tc_step(tc_handle* h, tc_stats_row* row, int32_t* cycles, double* dt_out);

/* One main-loop step with the state in HOST arrays (the drop-in for a host
 * that keeps the reference's module arrays): copies T, Cnew, SF, rtr, str,
 * Ttype in, runs tc_step, copies T, Cnew, SF, rtr, str back.  The arrays
 * must hold the state the previous call (or tc_download_state) returned;
 * after changing them, call tc_upload_state instead.  Any of row, cycles,
 * dt_out may be NULL.  No counterpart in the reference beyond tc_step.
 * Temperature tracers (tracer = 1) are refused (TC_ERR_UNSUPPORTED): Ttr is
 * not among the arrays; step with tc_step and download Ttr instead. */
tc_status tc_step_host(tc_handle* h, double* T, double* Cnew, double* SF, double* rtr, double* str,
                       const int32_t* Ttype, int64_t ntr, tc_stats_row* row, int32_t* cycles, double* dt_out);

/* Autotuner (no reference counterpart).  For each smoothed level it times,
 * on this handle's GPU and in its solver precision, the per-sweep smoother
 * kernel under eight block shapes of at most 256 threads, then visits of 1
 * to 6 sweeps per launch of the tiled smoother (FP64: 1 or 2) and fused
 * cluster visits of every shape that fits (1 or 2 points per thread strip,
 * 1 to 16 CTAs), with CUDA-graph replays, and keeps the fastest of each.
 * Results are unchanged by the choice (the arithmetic per point does not
 * depend on the launch shape).  If `choices` is not NULL it receives (block
 * x, block y, visit) for levels 1..grids-1, visit = 0 for one launch per
 * sweep, 1000 + n for n sweeps per launch, 1 for the default fused shape,
 * else 100 x points per strip + CTAs.  Needs uploaded state; the levels'
 * corrections are restored afterwards. */
tc_status tc_autotune(tc_handle* h, int32_t* choices);
/* Applies launch shapes in tc_autotune's `choices` format (3 ints per level
 * 1..grids-1: sweep block x, block y, visit = 0 one launch per sweep / 1
 * default fused visit / 100*P + C / 1000 + n for n sweeps per launch of the
 * tiled smoother, n = 1..2, or 1..6 in the mixed solver), e.g. shapes tuned once on
 * another handle of the same grid and precision.  TC_ERR_ARG (nothing
 * changed) if a block has more than 256 threads or a visit shape does not fit
 * its level.  Shapes do not change the arithmetic. */
tc_status tc_set_launch_shapes(tc_handle* h, const int32_t* choices);

/* Ensemble of independent cases (no reference counterpart: the reference
 * runs one case per process).  One tc_step on each of the n handles, the
 * handles' work issued concurrently by up to nthreads host threads, each
 * handle on its own stream, so the GPU runs the cases' kernels side by side.
 * rows[i], cycles[i], dts[i], status[i] receive case i's results (any may be
 * NULL); returns the first non-OK status or TC_OK.  The handles must be
 * distinct, and no other thread may use them during the call. */
tc_status tc_ensemble_step(tc_handle* const* hs, int32_t n, int32_t nthreads, tc_stats_row* rows, int32_t* cycles,
                           double* dts, tc_status* status);

/* The timestep as one CUDA graph launch (no reference counterpart; the
 * reference's main.f90 time loop calls the same subroutines one by one).
 * tc_set_step_graph(h, 1): from the handle's second step on, tc_step
 * captures the whole step (multigrid with its convergence loop and the
 * filter loops as conditional WHILE nodes, velocities, stats, energy_time)
 * once per tracer-sort flag and then launches it once per step with one
 * synchronisation; the reads of the device scalars the step makes (cycle
 * counts, stop tests, the stats row, dt) are recorded into pinned memory by
 * the graph and processed after it, in the eager step's order, so results,
 * status codes and the stats row are those of the eager step (state after a
 * failing step may differ: a graph step runs to its end).  Steps that need a
 * host decision run eagerly: the first step, non_Newtonian = 1, equalize =
 * 1, learned_guess 1 or 2, a solve recorder, the host loops.  A capture the
 * CUDA runtime refuses switches the handle back to eager steps (state 2).
 * tc_step_graph_info: steps run as one graph, state 0 off / 1 on / 2
 * refused. */
tc_status tc_set_step_graph(tc_handle* h, int32_t on);
tc_status tc_step_graph_info(const tc_handle* h, int64_t* graph_steps, int32_t* state);

/* An ensemble stepped by one graph launch per timestep: every case's
 * captured step is a branch of one graph forked from the ensemble's own
 * stream onto the cases' streams and joined back; graphs are cached by the
 * case list (at most four).  tc_ensemble_run takes the cases of this step
 * (the same contract as tc_ensemble_step, whose thread pool of nthreads
 * threads runs a step whenever a case is not ready for a captured step);
 * the handles must outlive the ensemble object.  tc_ensemble_info: steps
 * run as one launch and steps run by the thread pool. */
typedef struct tc_ensemble tc_ensemble;
tc_status tc_ensemble_create(int32_t nthreads, tc_ensemble** out);
tc_status tc_ensemble_run(tc_ensemble* e, tc_handle* const* hs, int32_t n, tc_stats_row* rows, int32_t* cycles,
                          double* dts, tc_status* status);
tc_status tc_ensemble_info(const tc_ensemble* e, int64_t* graph_steps, int64_t* eager_steps);
tc_status tc_ensemble_destroy(tc_ensemble* e);

/* Diagnostics (no counterpart in the reference).  tc_time_sweep times
 * `nsweeps` back-to-back launches of the multigrid smoother kernel of `level`
 * (the FP32 one under solver_precision = 1), replayed as one CUDA graph as
 * the solver runs them, with CUDA events on the handle's stream (state left
 * unchanged) and writes
 * the mean milliseconds per launch.  tc_kernel_launches returns how many
 * kernels this library has launched in the process so far (graph replays
 * count every kernel node). */
tc_status tc_time_sweep(tc_handle* h, int32_t level, int32_t nsweeps, double* ms_per_sweep);
/* Times `reps` back-to-back smoother visits (Nmulti sweeps and the residual,
 * in the handle's solver precision; level 1 of the mixed solve includes its
 * FP64 residual, FP32 RHS and FP64 update) of `level` on the handle's stream
 * and writes the mean milliseconds per visit.  The level's correction arrays
 * are left changed; the next tc_multigrid starts from SF as always. */
tc_status tc_time_visit(tc_handle* h, int32_t level, int32_t reps, double* ms_per_visit);
/* With mg_coarse_matrix in effect: times `reps` back-to-back products with
 * the bottom-of-cycle matrix of the pattern with k coarsest solves (one
 * kernel each) and writes the mean milliseconds per product.
 * TC_ERR_UNSUPPORTED if the handle has no such matrix. */
tc_status tc_time_subcycle(tc_handle* h, int32_t k, int32_t reps, double* ms_per_apply);
/* Timeout-path test (no counterpart in the reference).  With on != 0 every
 * fused cluster visit of the handle first waits, with a bounded poll, for a
 * device word that nothing sets, before it issues any sweep or write to
 * another CTA; the poll runs out, the visit takes its timeout exit and the
 * next tc_multigrid returns TC_ERR_DEVICE_TIMEOUT.  on = 0 restores normal
 * visits; the handle then solves as before. */
tc_status tc_debug_wait_test(tc_handle* h, int32_t on);
/* Level-1 FP32 smoother of the mixed solve (no counterpart in the reference).
 * By default it forms the 13 folded coefficients from five FP32 viscosity
 * fields inside each sweep; with fields = 0 it reads the 13 coefficient
 * planes rounded from FP64 instead (the same taps and factors; only the
 * coefficients' rounding differs).  For tests that compare the two;
 * TC_ERR_UNSUPPORTED when the handle has no field sweep (FP64 solve). */
tc_status tc_debug_sweep_fields(tc_handle* h, int32_t fields);
int64_t tc_kernel_launches(void);

/* Copies u, w ((-span_interp:nx+span_interp, ...) each) to the host. */
tc_status tc_download_velocities(tc_handle* h, double* u, double* w);

/* tracers_to_corners (composition.f90:669-790) on the given positions,
 * smoothing on: Cnew, count_type, nempty, Cvis, Cbuoy, conduct are updated.
 * rtr/str are HOST arrays of ntr doubles. */
tc_status tc_tracers_to_corners(tc_handle* h, const double* rtr, const double* str);

/* compute_strain_rate_invariant (momentum.f90:32-62): the strain-rate
 * invariant of the current velocities (tc_compute_velocities first); the
 * plastic viscosity (ivis = 3) uses it.  tc_stats computes it as well. */
tc_status tc_compute_strain_rate_invariant(tc_handle* h);
/* compute_viscosity (iterative_solver.f90:331-377) for one level: visf and
 * the viscosity filter at level 1, restriction and filter below (levels in
 * order, as multigrid calls them); updates the viscosity_smoother scalars
 * that tc_stats reports (n_eta, eig_fine).  tc_multigrid calls it itself. */
tc_status tc_compute_viscosity(tc_handle* h, int32_t level);

/* Diagnostic (no reference counterpart): perm[j] (ntr int32) = the
 * reference's index of the tracer in storage slot j on the device (the
 * identity after an upload; the cell order after a re-sort, see
 * tracer_sort_interval). */
tc_status tc_tracer_order(tc_handle* h, int32_t* perm);

/* Copies count_type (0:ntype, -span:nx+span, -span:nz+span) as int32. */
tc_status tc_download_counts(tc_handle* h, int32_t* count_type);

/* Diagnostic copy of an internal field (no counterpart in the reference; used
 * by the parity tests).  `name` is a reference array name: T, SF, Tvis, Tbuoy,
 * u, w, conduct, conduct_r, conduct_s, Cnew, Cvis, Cbuoy (type >= 1),
 * vis_grid, vis_x, vis_z, vis_xx, vis_zz, vis_xz, dt_stream, ratio, RHS,
 * error, residual, dt_vis (level >= 1), DERr_u, DERr_w, dts_array, strain,
 * Tratio, tracer_space_array (tracer = 1).  out
 * receives the level's ghost-padded box (-span:nx_l+span, -span:nz_l+span)
 * in Fortran order; entries outside the reference array's own bounds are
 * unspecified. */
tc_status tc_debug_field(tc_handle* h, const char* name, int32_t level, int32_t type, double* out);

/* sizeof(tc_params), sizeof(tc_stats_row), sizeof(tc_info) as compiled, so a
 * binding can check its struct layouts. */
void tc_abi_sizes(int32_t sizes[3]);

/* Allocation-free stats.dat row (no counterpart in the reference: it exists
 * for hosts that cannot let a library allocate device memory, e.g. an
 * OpenACC / CUDA Fortran port of the reference that owns every device array
 * in its own pool, or an application under a fixed device-memory budget;
 * such a host cannot create a tc_handle, which allocates).  Computes the
 * same row as tc_stats (basics.f90:236-324) from device arrays the caller
 * owns, in the reference's layouts: T, conduct, vis (vis_grid of level 1)
 * and nempty on (-2:nx+2, -2:nz+2); u, w on (-1:nx+1, -1:nz+1); Cnew on
 * (1:ntype, -2:nx+2, -2:nz+2).  Uniform grid, order 2.  Pass nempty when the
 * run has compositional or temperature tracers (comp = 1 or tracer = 1, the
 * rule of basics.f90:263-267: empty_cells, tracer_min and tracer_max are then
 * filled) and NULL otherwise; it is required when ntype > 0.  kent and mass
 * (host array, may be NULL: ent = 0) are the entrainment inputs of stats;
 * time, tstep and the smoother counters of the row are left 0.  Work is
 * issued on `stream` (a cudaStream_t, NULL = legacy default) and the call
 * returns after it finished.
 * It calls no cudaMalloc/cudaFree: its scratch is one fixed device array of
 * 229,712 bytes that every GPU loading this library holds until exit, which
 * limits nz to TC_NOALLOC_MAX_NZ (larger nz returns TC_ERR_TOO_LARGE).  The
 * first call on a device looks up that array's device address (with the
 * device current) and should come before any stream capture on it; the
 * address is looked up again when the device's context changed (after
 * cudaDeviceReset).  All calls share the array: calls whose work overlaps on
 * the GPU race.  Launch failures are read from the launches' return codes;
 * the runtime's last-error state is left as the caller left it. */
#define TC_NOALLOC_MAX_NZ 4096
tc_status tc_stats_noalloc(const double* T, const double* u, const double* w, const double* conduct,
                           const double* vis, const double* Cnew, const int32_t* nempty, int32_t nx, int32_t nz,
                           int32_t ntype, double aspect, double RaT, int32_t kent, const double* mass,
                           tc_stats_row* row, void* stream);

/* Text of the last CUDA error seen by the handle ("" if none). */
const char* tc_last_error(const tc_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* TRACER_GPU_H */
