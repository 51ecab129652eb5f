// k_loop.cu -- the convergence loop of multigrid (iterative_solver.f90:
// 105-168) on the device.
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

}  // namespace

void launch_cycle_init(cudaStream_t s, DevScalars* ds) {
    k_cycle_init<<<1, 1, 0, s>>>(ds);
    tc_note_launch();
}

void launch_cycle_check(cudaStream_t s, DevScalars* ds, double tolerance, int max_cycles,
                        cudaGraphConditionalHandle cond) {
    launch_pdl(k_cycle_check, dim3(1), dim3(1), 0, s, ds, tolerance, max_cycles, cond);
    tc_note_launch();
}
