// k_loop.cu -- the convergence loop of multigrid (iterative_solver.f90:
// 105-168) and the filter loops (smoother.f90:166-263, 287-341, 343-377) on
// the device.
//
// The solve is one CUDA graph: [init, level-1 visit, check] followed by a
// WHILE node whose body is [rest of the W-cycle, level-1 visit, check].  The
// check kernel applies the reference's tests in the host loop's order --
// a fused visit's bounded wait that gave up, the residual blow-up test
// (res > 1e10 res_ref), the tolerance test (res / res_ref <= tolerance),
// then the cycle count (q > max_cycles) -- and sets the WHILE node's
// condition: 1 to run another cycle, 0 to stop.  The host reads the count
// and the stop reason once, after the whole solve.  When the cycle cap is
// reached the loop stops before that cycle's coarse-grid work (the host
// loop ran it and then stopped); the solve returns TC_ERR_MG_CYCLES either
// way.
#include "tc_device.cuh"

namespace {

__global__ void k_cycle_init(DevScalars* ds) {
    ds->cyc_q = 1;
    ds->cyc_status = 0;
}

__global__ void k_cycle_check(DevScalars* ds, double tolerance, int max_cycles, cudaGraphConditionalHandle cond) {
    pdl_entry();
    const double ref = __ldcg(&ds->res_ref), rm = __ldcg(&ds->res_mag[1]);
    int q = __ldcg(&ds->cyc_q);
    unsigned int more = 0;
    if (__ldcg(&ds->visit_timeout) != 0) {
        ds->cyc_status = TC_ERR_DEVICE_TIMEOUT;
    } else if (rm > 1.0e10 * ref) {
        ds->cyc_status = TC_ERR_MG_RESIDUAL;
    } else if (rm / ref <= tolerance) {
        ds->cyc_status = 0;
    } else {
        q = q + 1;
        if (q > max_cycles) ds->cyc_status = TC_ERR_MG_CYCLES;
        else more = 1;
        ds->cyc_q = q;
    }
    cudaGraphSetConditional(cond, more);
    pdl_done();
}

// ---- filter loops ------------------------------------------------------------
// smoother_time_T (smoother.f90:343-377): after smoothness(Tvis) -- stop when
// diff < delta_T (n_temp = steps done), fail at the cap, else one more step.
__global__ void k_tflt_init(DevScalars* ds) {
    ds->flt_n = 0;
}
__global__ void k_tflt_check(DevScalars* ds, double delta, long long cap, int body, cudaGraphConditionalHandle cond) {
    const int n = ds->flt_n;
    unsigned int more = 0;
    if (__ldcg(&ds->diff) < delta) {
        ds->n_temp = n;
    } else if (n >= cap) {
        ds->flt_status = TC_ERR_LOOP_CAP;
    } else {
        ds->flt_n = n + 1;
        more = 1;
    }
    if (more) ds->flt_launches += (unsigned long long)body;
    cudaGraphSetConditional(cond, more);
}

// smoother_time (smoother.f90:287-341), one type: inner passes n = 1..Niter
// (Niter = 10 at the call's start, 1 after any type's first outer pass), a
// Chebyshev factor in the first outer pass (nn = 0) and 1 after it; the
// test precedes every step.
__global__ void k_cflt_init(DevScalars* ds, int first_type) {
    if (first_type) ds->flt_niter = 10;
    ds->flt_n = 1;
    ds->flt_nn = 0;
    ds->flt_guard = 0;
}
__global__ void k_cflt_check(DevScalars* ds, int type, double delta, long long cap, const double* tab10,
                             const double* tab1, int body, cudaGraphConditionalHandle cond) {
    unsigned int more = 0;
    if (__ldcg(&ds->diff) < delta) {
        ds->n_comp[type] = ds->flt_nn;
    } else {
        int n = ds->flt_n, niter = ds->flt_niter, nn = ds->flt_nn;
        ds->flt_c = (nn == 0) ? ((niter == 10) ? tab10[n - 1] : tab1[n - 1]) : 1.0;
        more = 1;
        if (++n > niter) {
            niter = 1;
            nn++;
            n = 1;
            if (++ds->flt_guard > cap) {
                ds->flt_status = TC_ERR_LOOP_CAP;
                more = 0;
            }
        }
        ds->flt_n = n;
        ds->flt_niter = niter;
        ds->flt_nn = nn;
    }
    if (more) ds->flt_launches += (unsigned long long)body;
    cudaGraphSetConditional(cond, more);
}

// smoother_vis (smoother.f90:166-263): the module scalars Nvis_store and
// nn_store live on the device between calls.  flt_n is the outer counter n,
// flt_nn the inner index nn, flt_phase 1 once option 1 switched to its
// second factor set.
__device__ __forceinline__ void vflt_next_outer(DevScalars* ds, const VisFltArgs& a, int& n, int& nn, int& niter,
                                                unsigned int& more) {
    ds->vis_nvis_store += 1;
    ds->vis_nn_store = 1;
    if (a.option == 1) {
        niter = 6;
        ds->flt_phase = 1;
    }
    n += 1;
    nn = 1;
    if (++ds->flt_guard > a.cap) {
        ds->flt_status = TC_ERR_LOOP_CAP;
        more = 0;
    }
}
__global__ void k_vflt_init(DevScalars* ds, int reset_store, VisFltArgs a) {
    if (reset_store) {
        ds->vis_nvis_store = 0;
        ds->vis_nn_store = 1;
    }
    ds->flt_phase = 0;
    ds->flt_guard = 0;
    int n = 0, nn = ds->vis_nn_store, niter = a.niter0;
    unsigned int more = 1;
    // an inner loop with no passes (nn_store > Niter) goes straight to the
    // next outer pass, as the host loop does
    if (nn > niter) vflt_next_outer(ds, a, n, nn, niter, more);
    ds->flt_n = n;
    ds->flt_nn = nn;
    ds->flt_niter = niter;
}
__global__ void k_vflt_check(DevScalars* ds, VisFltArgs a, int body, cudaGraphConditionalHandle cond) {
    const double rmin = __ldcg(&ds->ratio_min);
    int n = ds->flt_n, nn = ds->flt_nn, niter = ds->flt_niter;
    const int nvis = ds->vis_nvis_store;
    bool stop;
    if (a.option == 1) {
        stop = (nvis >= 1 && rmin > a.eig_ratio_min) || a.ivis0 || n > 20;
        if (stop) {
            ds->eig_fine = a.ivis0 ? 1.0e99 : rmin;
            ds->n_eta = n;
        }
    } else if (a.interpolate == 0) {
        const double r = a.ivis0 ? 0.0 : rmin;
        stop = (r > a.eig_ratio) || a.ivis0;
        if (stop) ds->vis_nn_store = nn;
    } else {
        stop = (nvis >= 1) || a.ivis0;
    }
    unsigned int more = 0;
    if (!stop) {
        ds->flt_c = (ds->flt_phase == 0) ? a.tabA[nn - 1] : a.tabB[nn - 1];
        more = 1;
        if (++ds->flt_guard > a.cap) {
            ds->flt_status = TC_ERR_LOOP_CAP;
            more = 0;
        }
        if (++nn > niter) vflt_next_outer(ds, a, n, nn, niter, more);
        ds->flt_n = n;
        ds->flt_nn = nn;
        ds->flt_niter = niter;
    }
    if (more) ds->flt_launches += (unsigned long long)body;
    cudaGraphSetConditional(cond, more);
}

}  // namespace

void launch_tflt_init(cudaStream_t s, DevScalars* ds) {
    k_tflt_init<<<1, 1, 0, s>>>(ds);
    tc_note_launch();
}
void launch_tflt_check(cudaStream_t s, DevScalars* ds, double delta, long long cap, int body,
                       cudaGraphConditionalHandle cond) {
    k_tflt_check<<<1, 1, 0, s>>>(ds, delta, cap, body, cond);
    tc_note_launch();
}
void launch_cflt_init(cudaStream_t s, DevScalars* ds, int first_type) {
    k_cflt_init<<<1, 1, 0, s>>>(ds, first_type);
    tc_note_launch();
}
void launch_cflt_check(cudaStream_t s, DevScalars* ds, int type, double delta, long long cap, const double* tab10,
                       const double* tab1, int body, cudaGraphConditionalHandle cond) {
    k_cflt_check<<<1, 1, 0, s>>>(ds, type, delta, cap, tab10, tab1, body, cond);
    tc_note_launch();
}
void launch_vflt_init(cudaStream_t s, DevScalars* ds, int reset_store, const VisFltArgs& a) {
    k_vflt_init<<<1, 1, 0, s>>>(ds, reset_store, a);
    tc_note_launch();
}
void launch_vflt_check(cudaStream_t s, DevScalars* ds, const VisFltArgs& a, int body,
                       cudaGraphConditionalHandle cond) {
    k_vflt_check<<<1, 1, 0, s>>>(ds, a, body, cond);
    tc_note_launch();
}

void launch_cycle_init(cudaStream_t s, DevScalars* ds) {
    k_cycle_init<<<1, 1, 0, s>>>(ds);
    tc_note_launch();
}

void launch_cycle_check(cudaStream_t s, DevScalars* ds, double tolerance, int max_cycles,
                        cudaGraphConditionalHandle cond) {
    launch_pdl(k_cycle_check, dim3(1), dim3(1), 0, s, ds, tolerance, max_cycles, cond);
    tc_note_launch();
}
