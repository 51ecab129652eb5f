// tc_api.cu -- the C ABI of include/tracer_gpu.h and the host-side sequencing
// that sequence the kernels exactly as the reference sequences its loops.
//
// Control flow replaces these reference subroutines (one C++ function each,
// same names): multigrid, iterate_stream, compute_viscosity, smoother_vis,
// smoother_time, smoother_time_T, tracers_to_corners, energy_time, stats
// (iterative_solver.f90, smoother.f90, composition.f90, energy.f90,
// basics.f90).  All arithmetic runs in the kernels; the host only keeps the
// reference's module scalars (Nvis_store, nn_store, n_eta, eig_fine, n_temp,
// n_comp, kent, mass, time, tstep) and reads back the device scalars that the
// reference's data-dependent loops branch on.
#include "tc_device.cuh"
#include "tc_setup.h"
#include "tracer_nn.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include <atomic>
#include <functional>
#include <map>
#include <thread>

static std::atomic<long long> g_launches{0};
static std::atomic<long long> g_handle_uid{0};
// per host thread, so that graph capture counts only its own thread's
// launches while other handles run on other threads (tc_ensemble_step)
static thread_local long long t_launches = 0;
void tc_note_launch(long long n) {
    g_launches.fetch_add(n);
    t_launches += n;
}

// learned initial guess (k_nn.cu, tc_nn_api.cu)
struct tc_net_impl;
tc_net_impl* tcnn_impl(tc_net* n);
int* net_fail(tc_net_impl* n);
void net_dims(const tc_net_impl* n, int* H, int* W);
void nn_fields_to_raw(cudaStream_t s, const Lay& L, const double* vis, const double* rhs, const double* SF,
                      float* raw);
void nn_field_to_img(cudaStream_t s, const Lay& L, const double* S, float* img);
int nn_guess(tc_net_impl* n, cudaStream_t s, const Lay& L, const double* vis, const double* rhs, const double* SF,
             float* raw, double* G, int Vbc, int smooth);

namespace {

const double kPi = 3.1415926535897932;

struct CycleGraphs;
// largest coarse grid (unknowns) solved through an explicit inverse (a
// matrix-vector product per visit, n^2 doubles); larger ones use banded
// substitution with the LU factors each visit
constexpr int kCoarseInverseMax = 2048;

struct Handle {
    tc_params p{};
    int nx = 0, nz = 0, grids = 0, nsteps = 0, ntype = 0;
    int64_t ntr = 0;
    int ngrid_coarse = 0, kl = 0, ku = 0;
    std::vector<int> multi;  // multi(0:nsteps+1)
    double grid_dr = 0, grid_ds = 0;
    double delta_T = 2.0, delta_C[TC_MAX_TYPES];
    tcs::EigBase eb{};
    Phys P{};
    Level lev[TC_MAXLEV + 1];
    Lay L1{};
    // fine fields (level-1 layout)
    double *T = nullptr, *T0 = nullptr, *T1 = nullptr, *T2 = nullptr, *SF = nullptr;
    double *Tvis = nullptr, *Tvis2 = nullptr, *Tbuoy = nullptr;
    double *u = nullptr, *w = nullptr, *du = nullptr, *dw = nullptr;
    double *conduct = nullptr, *conduct_r = nullptr, *conduct_s = nullptr, *dts = nullptr, *strain = nullptr;
    double* Cnew[TC_MAX_TYPES] = {};
    double* C0[TC_MAX_TYPES] = {};
    double* Cvis[TC_MAX_TYPES] = {};
    double* Cvis2[TC_MAX_TYPES] = {};
    double* Cbuoy[TC_MAX_TYPES] = {};
    int *counts = nullptr, *nempty = nullptr;
    double* zg = nullptr;  // device, index k+SP+1
    double *rtr = nullptr, *str = nullptr, *rtr0 = nullptr, *str0 = nullptr, *rtr1 = nullptr, *str1 = nullptr,
           *rtr2 = nullptr, *str2 = nullptr;
    int* ttype = nullptr;
    // temperature tracers (tracer = 1): Ttr and its RK copies, the per-volume
    // mean Tratio, tracer_space_array and its r-derivatives, the exact sums
    double *Ttr = nullptr, *Ttr0 = nullptr, *Ttr1 = nullptr, *Ttr2 = nullptr;
    double *Tratio = nullptr, *tsa = nullptr, *dT = nullptr;
    unsigned long long* tsum = nullptr;
    // tracer repositioning (equalize = 1): index and list buffers, the mzran
    // state of each reproduced OpenMP thread, the growable donor table,
    // Cinit (stats at time 0) and the last equalize.dat row
    int eq_NR = 1;
    int *eq_iperm = nullptr, *eq_nex = nullptr, *eq_off = nullptr, *eq_cur = nullptr, *eq_ids = nullptr,
        *eq_cnt = nullptr, *eq_seeds = nullptr, *eq_isv = nullptr, *eq_isv2 = nullptr, *eq_nfr = nullptr,
        *eq_nxl = nullptr, *eq_nzl = nullptr, *eq_donor = nullptr;
    size_t eq_donor_cap = 0;
    long long* eq_sc = nullptr;
    double *eq_Td = nullptr, *eq_dTd = nullptr;
    double Cinit[TC_MAX_TYPES] = {};
    long long nequalize = 0;
    std::vector<int64_t> eq_row;
    double *band = nullptr, *rowb = nullptr, *bvec = nullptr, *ainv = nullptr;
    // coarse grids above kCoarseInverseMax unknowns are solved by banded
    // substitution each visit instead of an explicit inverse
    bool coarse_banded = false;
    // interior unknowns of the coarsest grid: index p and level offset
    int *coarse_q = nullptr, *coarse_x = nullptr;
    int coarse_m = 0;
    int* ipiv = nullptr;
    double* rows = nullptr;
    RedScratch rs{};
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;  // pinned mirror
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<void*> allocs;
    // module state
    int tstep = 0;
    double time = 0.0, dt = 0.0;
    int kent = 0;
    double mass[TC_MAX_TYPES] = {};
    int n_eta = 0, n_temp = 0, n_comp[TC_MAX_TYPES] = {};
    double eig_fine = 0.0;
    int Nvis_store = 0, nn_store = 1;
    int ratio_level = 0;
    bool uploaded = false, lu_valid = false;
    int last_cycles = 0;
    long loop_cap = 100000;
    std::string err;
    CycleGraphs* graphs = nullptr;
    bool no_graphs = false;
    bool no_device_loop = false;  // convergence and filter loops on the host (one read per pass)
    // filter loops as cached WHILE graphs (k_loop.cu), keyed by loop kind,
    // level / type and the interpolate flag; their factor tables on the
    // device: [option-1 first phase 6][option-1 second phase 6][option 0
    // vis_iter][C Niter 10][C Niter 1]
    std::map<int, cudaGraphExec_t> flt_graphs;
    bool flt_failed = false;
    bool flt_dev_state = false;  // the filter counters and Nvis_store/nn_store live on the device
    double* flt_tab = nullptr;
    bool wait_test = false;       // tc_debug_wait_test: fused visits wait on a word nothing sets
    int cycles_acc = 0;  // W-cycles of all solves since tc_step began
    bool fuse_visits = false;  // small levels smoothed by one cluster launch per visit
    // cell order of the tracer arrays: perm[j] = reference index of slot j
    int* perm = nullptr;
    int* itmp[2] = {nullptr, nullptr};  // scatter targets of ttype and perm
    int *sort_cnt = nullptr, *sort_off = nullptr, *sort_bsum = nullptr;
    double* ctab = nullptr;    // per-point Chebyshev factors of the fused ratio level [Nmulti][(a-1)(b-1)]
    int ctab_level = 0;        // level the table was built for (0 = none)
    cudaError_t enq_err = cudaSuccess;  // first error of an enqueue-only helper (checked by its caller)
    int device = 0;                     // CUDA device the handle's memory lives on
    // learned initial guess
    tc_net_impl* net = nullptr;
    double* guess = nullptr;  // candidate start (level-1 layout)
    float* nn_raw = nullptr;  // network input scratch [3][nz][nx]
    long long guess_used = 0, guess_offered = 0;
    // learned_guess = 1 stops offering the guess after kGuessPatience
    // rejections in a row and then offers it on every kGuessProbe-th solve
    // only (the plain start is then used alone, as it was chosen anyway)
    int guess_reject_streak = 0;
    long long guess_solves = 0;
    // training-sample recorder (caller-owned device buffers)
    float *rec_raw = nullptr, *rec_sf = nullptr;
    int rec_cap = 0, rec_count = 0;
    // bottom of the W-cycle as precomputed matrices (mg_coarse_matrix = 1):
    // sub_k[pp] = coarse solves of the pattern that starts at cycle step pp
    // (a step entering level grids-1 from above; 0 elsewhere), sub_end[pp]
    // its last step; subM[k-1] = M_k (FP32 in the mixed solve); sub_tab =
    // the c and temp tables of a downward and an upward visit
    bool sub_on = false, sub_valid = false;
    bool sub_m32 = false;  // the matrices are built and held in FP32 (mixed solve)
    float* sub_ac = nullptr;  // the FP32 build's compact coarse inverse (coarse_m^2)
    int sub_kmax = 0;
    std::vector<int> sub_k, sub_end;
    double* subM[4] = {nullptr, nullptr, nullptr, nullptr};
    double* sub_tab = nullptr;
    double* sub_ctab = nullptr;  // per-point Chebyshev factors of level grids-1 [Nmulti][n_S]
    // corrections of psi (k_accel.cu): psi after the previous correction,
    // the network's predicted change of the current solve
    double *acc_prev = nullptr, *acc_dnn = nullptr;
    double *win_p = nullptr, *win_ap = nullptr;  // windowed correction: TC_WIN changes and their images
    double *win_rn = nullptr, *win_rp = nullptr, *win_adnn = nullptr;  // r of psi, of prev; A dnn
    bool acc_dnn_on = false;  // the current solve has a network direction
    // whole-step graphs (tc_set_step_graph, tc_ensemble_*): while a step is
    // captured, each point where the host would read the device scalars
    // instead records them into hsnap[k] (a copy node of the graph) and
    // queues its host work in `deferred`, which runs after every launch of
    // the graph in the order the eager step would have run it; the WHILE
    // bodies of the step's loops are captured on body_st
    bool capturing = false;
    cudaStream_t body_st = nullptr;
    DevScalars* hsnap = nullptr;  // pinned, kMaxSnap entries
    int nsnap = 0;
    std::vector<std::function<tc_status()>> deferred;
    bool step_graph = false, step_graph_failed = false;
    std::map<int, struct StepGraph*> step_graphs;  // by whether the step sorts the tracers
    tc_stats_row stats_row{};                      // the row the last stats read formed
    long long sub_tab_key = -1;                    // the sweep tables now in sub_tab
    long long graph_steps = 0;                     // steps run as one graph launch
    long long epoch = 0;  // bumped whenever a captured step would be stale (launch shapes, network, stream)
    long long uid = 0;    // unique per handle in the process (an ensemble's graph cache key)
    std::vector<double> xg_h, zg_h;  // node coordinates of build_grid, index i + 3 for i = -3..n+3
};

constexpr int kMaxSnap = 64;

struct StepGraph {
    cudaGraphExec_t ge = nullptr;
    std::vector<std::function<tc_status()>> post;  // host work after the launch, in order
    long long n_static = 0;                        // kernel nodes outside the WHILE bodies
};

#define CK(call)                                                      \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) {                                      \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return TC_ERR_CUDA;                                       \
        }                                                             \
    } while (0)
#define CKV(call)                                                    \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess && h->enq_err == cudaSuccess) h->enq_err = e_; \
    } while (0)
#define TRY(x)                    \
    do {                          \
        tc_status s_ = (x);       \
        if (s_ != TC_OK) return s_; \
    } while (0)

tc_status dalloc(Handle* h, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        h->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return TC_ERR_ALLOC;
    }
    h->allocs.push_back(*p);
    e = cudaMemset(*p, 0, bytes);
    if (e != cudaSuccess) {
        h->err = std::string("cudaMemset: ") + cudaGetErrorString(e);
        return TC_ERR_CUDA;
    }
    return TC_OK;
}
template <class T>
tc_status dalloc_t(Handle* h, T** p, size_t n) {
    void* q = nullptr;
    tc_status s = dalloc(h, &q, n * sizeof(T));
    *p = (T*)q;
    return s;
}

Lay make_lay(int a, int b) {
    Lay L;
    L.a = a; L.b = b;
    int ni = a + 1 + 2 * SP;
    L.ld = (ni + 31) / 32 * 32;
    L.nk = b + 1 + 2 * SP;
    L.plane = (size_t)L.ld * L.nk;
    return L;
}

// The host's side of a read of the device scalars (already in *h->hs): the
// kernels the filter loops' WHILE bodies ran since the last read, their
// status and the module scalars they keep on the device.  `reset` clears
// the device's counters (a captured step clears them inside its graph).
tc_status scalars_to_host(Handle* h, bool reset) {
    if (h->hs->flt_launches != 0) {
        tc_note_launch((long long)h->hs->flt_launches);
        if (reset) CK(cudaMemsetAsync(&h->ds->flt_launches, 0, sizeof(unsigned long long), h->st));
    }
    if (h->hs->flt_status != 0) {
        const int st = h->hs->flt_status;
        if (reset) CK(cudaMemsetAsync(&h->ds->flt_status, 0, sizeof(int), h->st));
        h->hs->flt_status = 0;
        return (tc_status)st;
    }
    if (h->flt_dev_state) {
        h->n_temp = h->hs->n_temp;
        h->n_eta = h->hs->n_eta;
        h->eig_fine = h->hs->eig_fine;
        for (int t = 0; t < TC_MAX_TYPES; t++) h->n_comp[t] = h->hs->n_comp[t];
        h->Nvis_store = h->hs->vis_nvis_store;
        h->nn_store = h->hs->vis_nn_store;
    }
    return TC_OK;
}

// Synchronise and fetch the device scalars; reports sticky kernel faults.
tc_status sync_scalars(Handle* h) {
    CK(cudaMemcpyAsync(h->hs, h->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    return scalars_to_host(h, true);
}

// A point where the step reads the device scalars and then runs `post` on
// them.  Eager: synchronise, read, run post now.  While a step is captured:
// the graph copies the scalars into the next pinned snapshot and clears the
// filter counters, and post runs after each launch of the graph.
tc_status sync_point(Handle* h, std::function<tc_status()> post) {
    if (!h->capturing) {
        TRY(sync_scalars(h));
        return post ? post() : TC_OK;
    }
    if (h->nsnap >= kMaxSnap) {
        if (h->enq_err == cudaSuccess) h->enq_err = cudaErrorInvalidValue;
        return TC_OK;
    }
    const int k = h->nsnap++;
    CKV(cudaMemcpyAsync(h->hsnap + k, h->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, h->st));
    CKV(cudaMemsetAsync(&h->ds->flt_launches, 0, sizeof(unsigned long long), h->st));
    CKV(cudaMemsetAsync(&h->ds->flt_status, 0, sizeof(int), h->st));
    h->deferred.push_back([h, k, post]() -> tc_status {
        *h->hs = h->hsnap[k];
        TRY(scalars_to_host(h, false));
        return post ? post() : TC_OK;
    });
    return TC_OK;
}

// Inside a step being captured on h->st: pre(cond), then a WHILE node on
// cond whose body(cond) is captured on body_st into the node's body graph.
// The body's kernels are taken out of the launch count (*n_body holds them).
// False (with h->enq_err set) when the CUDA runtime refuses.
bool emit_while(Handle* h, const std::function<void(cudaGraphConditionalHandle)>& pre,
                const std::function<void(cudaGraphConditionalHandle)>& body, long long* n_body) {
    *n_body = 0;
    cudaStreamCaptureStatus cs;
    cudaGraph_t capg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphConditionalHandle cond;
    bool ok = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &capg, &deps, nullptr, &nd) == cudaSuccess &&
              cs == cudaStreamCaptureStatusActive && cudaGraphConditionalHandleCreate(&cond, capg, 0, 0) == cudaSuccess;
    if (ok) {
        pre(cond);
        ok = h->enq_err == cudaSuccess;
    }
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t wn = nullptr;
    ok = ok && cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &capg, &deps, nullptr, &nd) == cudaSuccess &&
         cs == cudaStreamCaptureStatusActive && cudaGraphAddNode(&wn, capg, deps, nullptr, nd, &np) == cudaSuccess &&
         cudaStreamUpdateCaptureDependencies(h->st, &wn, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    if (ok) {
        cudaStream_t keep = h->st;
        const long long before = t_launches;
        h->st = h->body_st;
        ok = cudaStreamBeginCaptureToGraph(h->st, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            body(cond);
            cudaGraph_t b2 = nullptr;
            ok = cudaStreamEndCapture(h->st, &b2) == cudaSuccess && h->enq_err == cudaSuccess;
        }
        h->st = keep;
        *n_body = t_launches - before;
        g_launches.fetch_sub(*n_body);
        t_launches = before;
    }
    if (!ok && h->enq_err == cudaSuccess) h->enq_err = cudaErrorStreamCaptureUnsupported;
    return ok;
}

// A graph of pre(cond) followed by a WHILE node on cond whose body is
// body(cond), captured from the handle's stream; the kernels of body are
// counted by the check kernels, not here.  False when the CUDA runtime refuses.
bool build_while_graph(Handle* h, const std::function<void(cudaGraphConditionalHandle)>& pre,
                       const std::function<void(cudaGraphConditionalHandle)>& body, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle cond;
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    const long long before = t_launches;
    bool ok = cudaGraphConditionalHandleCreate(&cond, g, 0, 0) == cudaSuccess &&
              cudaStreamBeginCaptureToGraph(h->st, g, nullptr, nullptr, 0, mode) == cudaSuccess;
    if (!ok) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        return false;
    }
    h->enq_err = cudaSuccess;
    pre(cond);
    cudaStreamCaptureStatus cs;
    cudaGraph_t capg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t wn = nullptr;
    ok = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &capg, &deps, nullptr, &nd) == cudaSuccess &&
         cs == cudaStreamCaptureStatusActive && cudaGraphAddNode(&wn, capg, deps, nullptr, nd, &np) == cudaSuccess &&
         cudaStreamUpdateCaptureDependencies(h->st, &wn, nullptr, 1, cudaStreamSetCaptureDependencies) ==
             cudaSuccess;
    cudaGraph_t g2 = nullptr;
    const bool ended = cudaStreamEndCapture(h->st, &g2) == cudaSuccess;
    if (ok && ended && h->enq_err == cudaSuccess) {
        cudaGraph_t bg = np.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(h->st, bg, nullptr, nullptr, 0, mode) == cudaSuccess;
        if (ok) {
            body(cond);
            cudaGraph_t b2 = nullptr;
            ok = cudaStreamEndCapture(h->st, &b2) == cudaSuccess && h->enq_err == cudaSuccess;
        }
    } else {
        ok = false;
    }
    // the kernels were counted at capture; the graph's launches count them
    g_launches.fetch_sub(t_launches - before);
    t_launches = before;
    cudaGraphExec_t ge = nullptr;
    if (ok) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
    cudaGraphDestroy(g);
    h->enq_err = cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return false;
    }
    *out = ge;
    return true;
}

// The cached filter graph `key`, built by make() on first use; null when
// graphs are off or the CUDA runtime refused one (from then on the host loops
// run, after the device's filter state was read back).
cudaGraphExec_t filter_graph(Handle* h, int key, const std::function<bool(cudaGraphExec_t*)>& make) {
    if (h->flt_failed || h->no_graphs || h->no_device_loop) return nullptr;
    auto it = h->flt_graphs.find(key);
    if (it != h->flt_graphs.end()) return it->second;
    cudaGraphExec_t ge = nullptr;
    if (!make(&ge)) {
        h->flt_failed = true;
        return nullptr;
    }
    h->flt_graphs[key] = ge;
    return ge;
}

// Reads the device's filter state back into the handle (before a host
// loop runs after the device ones did).
tc_status filter_state_to_host(Handle* h) {
    if (!h->flt_dev_state) return TC_OK;
    TRY(sync_scalars(h));
    h->flt_dev_state = false;
    return TC_OK;
}

// Launches a filter graph (n_pre kernels before its WHILE node), first
// handing the module scalars over to the device.
tc_status launch_filter_graph(Handle* h, cudaGraphExec_t ge, int n_pre) {
    if (!h->flt_dev_state) {
        DevScalars init{};
        init.vis_nvis_store = h->Nvis_store;
        init.vis_nn_store = h->nn_store;
        init.n_eta = h->n_eta;
        init.n_temp = h->n_temp;
        init.eig_fine = h->eig_fine;
        for (int t = 0; t < TC_MAX_TYPES; t++) init.n_comp[t] = h->n_comp[t];
        // eig_fine to the end of DevScalars: the filter state (counters,
        // status and launch count zero)
        const size_t o0 = offsetof(DevScalars, eig_fine), o1 = sizeof(DevScalars);
        CK(cudaMemcpyAsync((char*)h->ds + o0, (const char*)&init + o0, o1 - o0, cudaMemcpyHostToDevice, h->st));
        CK(cudaStreamSynchronize(h->st));
        h->flt_dev_state = true;
    }
    CK(cudaGraphLaunch(ge, h->st));
    tc_note_launch(n_pre);
    return TC_OK;
}

// filter graph keys: kind * 1000 + level or type * 10 + interpolate
enum { kFltT = 1, kFltC = 2, kFltVis = 3 };
// factor-table offsets in h->flt_tab
constexpr int kTabVisA1 = 0, kTabVisB = 6, kTabVis0 = 12;
inline int tab_c10(const Handle* h) { return kTabVis0 + h->p.vis_iter; }
inline int tab_c1(const Handle* h) { return kTabVis0 + h->p.vis_iter + 10; }

// ---------------------------------------------------------------------------
// boundary-condition and copy helpers
// ---------------------------------------------------------------------------
void copy_plane(Handle* h, double* dst, const double* src) {
    cudaMemcpyAsync(dst, src, sizeof(double) * h->L1.plane, cudaMemcpyDeviceToDevice, h->st);
}

// load_conductivity_array (energy.f90:31-58)
void load_conductivity_array(Handle* h) {
    launch_conductivity(h->st, h->L1, h->P, h->Cvis, h->conduct, h->conduct_r, h->conduct_s);
}

// smoother_time_T (smoother.f90:343-377)
tc_status smoother_time_T(Handle* h, const double* Tin) {
    copy_plane(h, h->Tvis, Tin);
    copy_plane(h, h->Tbuoy, Tin);
    if (h->p.RaT == 0.0) return TC_OK;
    // on the device: [smoothness, test] then WHILE {step, BCs, copy back,
    // smoothness, test}; Tvis keeps its buffer (Tvis2 is the step's target)
    auto pre = [&](cudaGraphConditionalHandle c) {
        launch_tflt_init(h->st, h->ds);
        launch_smoothness(h->st, h->L1, h->Tvis, h->rs, h->ds);
        launch_tflt_check(h->st, h->ds, h->delta_T, h->loop_cap, 4, c);
    };
    auto body = [&](cudaGraphConditionalHandle c) {
        launch_smooth_T_step(h->st, h->L1, h->P, h->Tvis, h->Tvis2, h->dts);
        launch_enforce_T(h->st, h->L1, h->Tvis2, h->p.Tbot);
        copy_plane(h, h->Tvis, h->Tvis2);
        launch_smoothness(h->st, h->L1, h->Tvis, h->rs, h->ds);
        launch_tflt_check(h->st, h->ds, h->delta_T, h->loop_cap, 4, c);
    };
    if (h->capturing) {
        long long nb;
        emit_while(h, pre, body, &nb);  // the body's kernels are counted on the device
        return TC_OK;
    }
    cudaGraphExec_t ge =
        filter_graph(h, kFltT * 1000, [&](cudaGraphExec_t* out) { return build_while_graph(h, pre, body, out); });
    if (ge) return launch_filter_graph(h, ge, 3);
    TRY(filter_state_to_host(h));
    int n = 0;
    for (;;) {
        launch_smoothness(h->st, h->L1, h->Tvis, h->rs, h->ds);
        TRY(sync_scalars(h));
        if (h->hs->diff < h->delta_T) { h->n_temp = n; break; }
        if (n >= h->loop_cap) return TC_ERR_LOOP_CAP;
        launch_smooth_T_step(h->st, h->L1, h->P, h->Tvis, h->Tvis2, h->dts);
        launch_enforce_T(h->st, h->L1, h->Tvis2, h->p.Tbot);
        std::swap(h->Tvis, h->Tvis2);
        n++;
    }
    return TC_OK;
}

// smoother_time (smoother.f90:287-341)
tc_status smoother_time(Handle* h) {
    int Niter = 10;
    const double lb = -5.0, la = -1.0;
    for (int t = 0; t < h->ntype; t++) {
        copy_plane(h, h->Cvis[t], h->Cnew[t]);
        copy_plane(h, h->Cbuoy[t], h->Cnew[t]);
    }
    // on the device, per type: [init, smoothness, test] then WHILE {step
    // with the factor the test chose, BCs, copy back, smoothness, test};
    // every type's graph is built before any runs
    std::vector<cudaGraphExec_t> ges(h->ntype, nullptr);
    bool dev = true;
    for (int t = 0; t < h->ntype && dev; t++) {
        const double* tab = h->flt_tab;
        auto pre = [&](cudaGraphConditionalHandle c) {
            launch_cflt_init(h->st, h->ds, t == 0 ? 1 : 0);
            launch_smoothness(h->st, h->L1, h->Cvis[t], h->rs, h->ds);
            launch_cflt_check(h->st, h->ds, t, h->delta_C[t], h->loop_cap, tab + tab_c10(h), tab + tab_c1(h), 4, c);
        };
        auto body = [&](cudaGraphConditionalHandle c) {
            launch_smooth_C_step(h->st, h->L1, h->P, h->Cvis[t], h->Cvis2[t], h->dts, 0.0, &h->ds->flt_c);
            launch_enforce_comp(h->st, h->L1, h->Cvis2[t], h->Cvis[t]);
            copy_plane(h, h->Cvis[t], h->Cvis2[t]);
            launch_smoothness(h->st, h->L1, h->Cvis[t], h->rs, h->ds);
            launch_cflt_check(h->st, h->ds, t, h->delta_C[t], h->loop_cap, tab + tab_c10(h), tab + tab_c1(h), 4, c);
        };
        if (h->capturing) {
            long long nb;
            emit_while(h, pre, body, &nb);
            continue;
        }
        ges[t] = filter_graph(h, kFltC * 1000 + t * 10,
                              [&](cudaGraphExec_t* out) { return build_while_graph(h, pre, body, out); });
        dev = ges[t] != nullptr;
    }
    if (h->capturing) return TC_OK;
    if (dev) {
        for (int t = 0; t < h->ntype; t++) TRY(launch_filter_graph(h, ges[t], 3));
        return TC_OK;
    }
    TRY(filter_state_to_host(h));
    for (int t = 0; t < h->ntype; t++) {
        int nn = 0;
        bool trigger = false;
        long guard = 0;
        for (;;) {
            for (int n = 1; n <= Niter; n++) {
                launch_smoothness(h->st, h->L1, h->Cvis[t], h->rs, h->ds);
                TRY(sync_scalars(h));
                if (h->hs->diff < h->delta_C[t]) { trigger = true; break; }
                double c;
                if (nn == 0) {
                    int ntemp = Niter - n + 1;
                    c = 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * kPi / (double)(2 * Niter)));
                } else c = 1.0;
                launch_smooth_C_step(h->st, h->L1, h->P, h->Cvis[t], h->Cvis2[t], h->dts, c);
                launch_enforce_comp(h->st, h->L1, h->Cvis2[t], h->Cvis[t]);
                std::swap(h->Cvis[t], h->Cvis2[t]);
            }
            if (trigger) break;
            Niter = 1;
            nn++;
            if (++guard > h->loop_cap) return TC_ERR_LOOP_CAP;
        }
        h->n_comp[t] = nn;
    }
    return TC_OK;
}

// the tracer arrays in cell order (k_tracer.cu): positions, types and the
// reference index move together.  The sort writes into the RK temporaries
// and is copied back, so every tracer buffer keeps its role from step to
// step (a captured step graph bakes the buffers in).
tc_status sort_tracers(Handle* h) {
    launch_sort_tracers(h->st, h->L1, h->P, h->ntr, h->rtr, h->str, h->ttype, h->perm, h->sort_cnt, h->sort_off,
                        h->sort_bsum, h->rtr1, h->str1, h->itmp[0], h->itmp[1], h->Ttr, h->Ttr1);
    const size_t n = (size_t)h->ntr;
    CK(cudaMemcpyAsync(h->rtr, h->rtr1, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->str, h->str1, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->ttype, h->itmp[0], sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->perm, h->itmp[1], sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, h->st));
    if (h->Ttr) CK(cudaMemcpyAsync(h->Ttr, h->Ttr1, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->st));
    return TC_OK;
}

// energy_time sorts the tracers at the start of this step
bool sorts_this_step(const Handle* h) {
    const bool trc = (h->p.comp == 1) || (h->p.tracer == 1);
    return trc && h->ntr > 0 && h->p.tracer_sort_interval > 0 && h->tstep % h->p.tracer_sort_interval == 0;
}

// tracer arrays to host arrays in the reference's order (any may be null);
// the copies are queued on the handle's stream
tc_status download_tracers(Handle* h, double* rtr, double* str, int32_t* Ttype, double* Ttr = nullptr) {
    const size_t n = (size_t)h->ntr;
    if (Ttr && h->Ttr) {
        launch_perm_scatter(h->st, h->ntr, h->perm, h->Ttr, h->Ttr2);
        CK(cudaMemcpyAsync(Ttr, h->Ttr2, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    }
    if (rtr) {
        launch_perm_scatter(h->st, h->ntr, h->perm, h->rtr, h->rtr2);
        CK(cudaMemcpyAsync(rtr, h->rtr2, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    }
    if (str) {
        launch_perm_scatter(h->st, h->ntr, h->perm, h->str, h->str2);
        CK(cudaMemcpyAsync(str, h->str2, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
    }
    if (Ttype) {
        launch_perm_scatter(h->st, h->ntr, h->perm, h->ttype, h->itmp[0]);
        CK(cudaMemcpyAsync(Ttype, h->itmp[0], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->st));
    }
    return TC_OK;
}

// tracers_to_corners (composition.f90:669-790).  With temperature tracers
// (Tt != nullptr) Tratio starts as T0 (kept in empty volumes) and takes the
// exact per-volume mean of Tt elsewhere, then enforceBCs and, when
// smoothing, smoother_time_T(Tratio).
tc_status tracers_to_corners(Handle* h, const double* rr, const double* ss, bool smooth, const double* Tt = nullptr,
                             const double* T0 = nullptr) {
    if (Tt) copy_plane(h, h->Tratio, T0);
    launch_histogram(h->st, h->L1, h->P, h->ntr, rr, ss, h->ttype, h->counts, h->ds, Tt, h->tsum);
    launch_counts_to_comp(h->st, h->L1, h->P, h->counts, h->nempty, h->Cnew, Tt ? h->tsum : nullptr,
                          Tt ? h->Tratio : nullptr);
    if (h->p.comp == 1) {
        for (int t = 0; t < h->ntype; t++) launch_enforce_comp(h->st, h->L1, h->Cnew[t], h->Cnew[t]);
        if (smooth) TRY(smoother_time(h));
    }
    if (Tt) {
        launch_enforce_T(h->st, h->L1, h->Tratio, h->p.Tbot);
        if (smooth) TRY(smoother_time_T(h, h->Tratio));
    }
    load_conductivity_array(h);
    return TC_OK;
}

// ---------------------------------------------------------------------------
// multigrid pieces
// ---------------------------------------------------------------------------
double* cur_vis(Handle* h, int l) { return h->lev[l].vis[h->lev[l].vcur]; }
double* cur_err(Handle* h, int l) { return h->lev[l].err[h->lev[l].ecur]; }

// viscosity_gradients + test_eigenvalues
void grad_eig(Handle* h, int level, bool eig) {
    Level& lv = h->lev[level];
    launch_vis_grad(h->st, lv, cur_vis(h, level), eig ? 1 : 0, h->p.ivis, h->rs, h->ds);
    if (eig) h->ratio_level = (h->p.ivis != 0) ? level : 0;
}

// smoother_vis (smoother.f90:166-263)
tc_status smoother_vis(Handle* h, int level, int interpolate) {
    Level& lv = h->lev[level];
    int option, Niter;
    double lb, la;
    if (level == 1 && interpolate == 0) { option = 1; Niter = 6; lb = -5.0; la = -2.0; }
    else { option = 0; Niter = h->p.vis_iter; lb = -2.0; la = -1.0; }
    if (interpolate == 0 || level == 1) { h->Nvis_store = 0; h->nn_store = 1; }
    const int a = lv.L.a, b = lv.L.b;
    int kmin, kmax;
    if (h->p.RaT == 0.0) { kmin = 0; kmax = b; } else { kmin = 1; kmax = b - 1; }
    const int RaTnz = (h->p.RaT != 0.0) ? 1 : 0;
    const double visT2 = h->p.visT * h->p.visT;
    (void)a;
    // on the device: [copy, init, grad_eig, test] then WHILE {step with the
    // factor the test chose, copy back, grad_eig, test}; vis[vcur] keeps its
    // buffer
    {
        VisFltArgs fa{};
        fa.option = option;
        fa.interpolate = interpolate;
        fa.ivis0 = (h->p.ivis == 0) ? 1 : 0;
        fa.niter0 = Niter;
        fa.eig_ratio_min = h->p.eig_ratio_min;
        fa.eig_ratio = h->p.eig_ratio;
        fa.cap = h->loop_cap;
        fa.tabA = h->flt_tab + (option == 1 ? kTabVisA1 : kTabVis0);
        fa.tabB = h->flt_tab + kTabVisB;
        const int reset = (interpolate == 0 || level == 1) ? 1 : 0;
        double* cur = lv.vis[lv.vcur];
        double* oth = lv.vis[1 - lv.vcur];
        const size_t by = sizeof(double) * lv.L.plane;
        auto pre = [&](cudaGraphConditionalHandle c) {
            if (cudaMemcpyAsync(oth, cur, by, cudaMemcpyDeviceToDevice, h->st) != cudaSuccess)
                h->enq_err = cudaErrorUnknown;
            launch_vflt_init(h->st, h->ds, reset, fa);
            launch_vis_grad(h->st, lv, cur, 1, h->p.ivis, h->rs, h->ds);
            launch_vflt_check(h->st, h->ds, fa, 3, c);
        };
        auto body = [&](cudaGraphConditionalHandle c) {
            launch_vis_smooth(h->st, lv, cur, oth, 0.0, kmin, kmax, RaTnz, visT2, &h->ds->flt_c);
            if (cudaMemcpyAsync(cur, oth, by, cudaMemcpyDeviceToDevice, h->st) != cudaSuccess)
                h->enq_err = cudaErrorUnknown;
            launch_vis_grad(h->st, lv, cur, 1, h->p.ivis, h->rs, h->ds);
            launch_vflt_check(h->st, h->ds, fa, 3, c);
        };
        if (h->capturing) {
            long long nb;
            emit_while(h, pre, body, &nb);
            h->ratio_level = (h->p.ivis != 0) ? level : 0;
            return TC_OK;
        }
        cudaGraphExec_t ge = filter_graph(h, kFltVis * 1000 + level * 10 + interpolate,
                                          [&](cudaGraphExec_t* out) { return build_while_graph(h, pre, body, out); });
        if (ge) {
            h->ratio_level = (h->p.ivis != 0) ? level : 0;  // grad_eig's, run at least once
            return launch_filter_graph(h, ge, 3);
        }
        TRY(filter_state_to_host(h));
    }
    // the buffer that smoothing writes must already hold the rows it leaves unchanged
    CK(cudaMemcpyAsync(lv.vis[1 - lv.vcur], lv.vis[lv.vcur], sizeof(double) * lv.L.plane, cudaMemcpyDeviceToDevice,
                       h->st));
    int n = 0;
    bool trigger = false;
    long guard = 0;
    for (;;) {
        const int nn_begin = h->nn_store;
        for (int nn = nn_begin; nn <= Niter; nn++) {
            grad_eig(h, level, true);
            const bool ivis0 = (h->p.ivis == 0);
            if (option == 1) {
                bool need = (h->Nvis_store >= 1) && !ivis0 && !(n > 20);
                double rmin = 0.0;
                if (need || (h->Nvis_store >= 1 || ivis0 || n > 20)) {
                    TRY(sync_scalars(h));
                    rmin = h->hs->ratio_min;
                }
                if ((h->Nvis_store >= 1 && rmin > h->p.eig_ratio_min) || ivis0 || n > 20) {
                    h->eig_fine = ivis0 ? 1.0e99 : rmin;
                    h->n_eta = n;
                    trigger = true;
                    break;
                }
            } else if (interpolate == 0) {
                double rmin = 0.0;
                if (!ivis0) {
                    TRY(sync_scalars(h));
                    rmin = h->hs->ratio_min;
                }
                if (rmin > h->p.eig_ratio || ivis0) { trigger = true; h->nn_store = nn; break; }
            } else {
                if (h->Nvis_store >= 1 || ivis0) { trigger = true; break; }
            }
            const int ntemp = Niter - nn + 1;
            const double c = 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * kPi / (double)(2 * Niter)));
            launch_vis_smooth(h->st, lv, lv.vis[lv.vcur], lv.vis[1 - lv.vcur], c, kmin, kmax, RaTnz, visT2);
            lv.vcur = 1 - lv.vcur;
            if (++guard > h->loop_cap) return TC_ERR_LOOP_CAP;
        }
        if (trigger) break;
        h->Nvis_store = h->Nvis_store + 1;
        h->nn_store = 1;
        if (option == 1) { h->nn_store = 1; Niter = 6; lb = -2.0; la = -1.0; }
        n = n + 1;
        if (++guard > h->loop_cap) return TC_ERR_LOOP_CAP;
    }
    return TC_OK;
}

// compute_viscosity (iterative_solver.f90:331-377)
tc_status compute_viscosity(Handle* h, int level) {
    if (level == 1) {
        launch_visf_level1(h->st, h->L1, h->P, cur_vis(h, 1), h->Tvis, h->Cvis, h->zg, h->T, h->strain);
        TRY(smoother_vis(h, 1, 0));
        return TC_OK;
    }
    const int l1 = level - 1;
    Level& f = h->lev[l1];
    Level& c = h->lev[level];
    const size_t by = sizeof(double) * f.L.plane;
    double* src[6] = {cur_vis(h, l1), f.vx, f.vz, f.vxx, f.vzz, f.vxz};
    for (int q = 0; q < 6; q++) CK(cudaMemcpyAsync(f.bak[q], src[q], by, cudaMemcpyDeviceToDevice, h->st));
    TRY(smoother_vis(h, l1, 1));
    launch_restrict_vis(h->st, c, f, cur_vis(h, l1), cur_vis(h, level));
    launch_vis_bcs_init(h->st, c, cur_vis(h, level), h->p.RaT != 0.0 ? 1 : 0, h->p.visT * h->p.visT);
    if (level < h->grids) TRY(smoother_vis(h, level, 0));
    else grad_eig(h, level, false);
    double* dst[6] = {cur_vis(h, l1), f.vx, f.vz, f.vxx, f.vzz, f.vxz};
    for (int q = 0; q < 6; q++) CK(cudaMemcpyAsync(dst[q], f.bak[q], by, cudaMemcpyDeviceToDevice, h->st));
    return TC_OK;
}

// Chebyshev node temp(n) and uniform factor c(n) of sweep n=1..Niter
// (iterative_solver.f90:873-885), stored at index n-1.
void cheb_temps(int Niter, int dir, double* tv, double* cv) {
    for (int n = 1; n <= Niter; n++) {
        const double ntemp = (double)(Niter - n + 1);
        const double la = -1.0, lb = -2.0;
        tv[n - 1] = std::cos((2.0 * ntemp - 1.0) * kPi / (double)(2 * Niter));
        cv[n - 1] = (dir == 1) ? 1.0 : 2.0 / (-lb - la + (lb - la) * tv[n - 1]);
    }
}

// factor c and Chebyshev node temp of sweep n (1-based) of a visit of Niter
// sweeps: iterate_stream's expressions (c = 1 for a Richardson visit, dir=1;
// c unused on the per-point Chebyshev level)
static void sweep_factors(int Niter, int n, int dir, bool cheb_pp, double* c, double* temp) {
    const double ntemp = (double)(Niter - n + 1);
    const double la = -1.0, lb = -2.0;
    *temp = std::cos((2.0 * ntemp - 1.0) * kPi / (double)(2 * Niter));
    *c = (dir != 1 && !cheb_pp) ? 2.0 / (-lb - la + (lb - la) * *temp) : 1.0;
}

// Would iterate_stream / iterate_stream32 smooth `level` in direction dir as
// one cluster visit?  (the conditions under which launch_visit_cluster runs)
static bool visit_fuses(Handle* h, int level, int dir) {
    const Level& lv = h->lev[level];
    const bool mixed = (h->p.solver_precision == 1);
    if (!(h->fuse_visits && lv.fuse && level > 1 && level < h->grids && h->p.Nmulti <= 128)) return false;
    if (!visit_cluster_fits(lv.L, h->p.Nmulti, mixed ? 1 : 0, lv.visit_cfg)) return false;
    const bool pp = (dir != 1 && level == h->ratio_level);
    return mixed || !pp || h->ctab_level == level;
}

// iterate_stream (iterative_solver.f90:860-963), iterate_order=1.
// pro: first add the prolongation of level+1's correction (prolong);
// rst: afterwards restrict the residual into level+1's RHS (restrict),
// zeroing level+1's correction if rst_zero.  A cluster visit does both in
// its own launch; otherwise they are separate kernels.
void iterate_stream(Handle* h, int level, int dir, int pro = 0, int rst = 0, int rst_zero = 0) {
    Level& lv = h->lev[level];
    const int Niter = h->p.Nmulti;
    const bool cheb_pp = (level == h->ratio_level);
    if (h->fuse_visits && lv.fuse && level > 1 && Niter <= 128) {
        // the whole visit in one cluster launch (same arithmetic, same result)
        double cv[128], tv[128];
        cheb_temps(Niter, dir, tv, cv);
        const int pp = (dir != 1 && cheb_pp) ? 1 : 0;
        VisitXfer<double> x;
        if (pro) {
            x.ec = cur_err(h, level + 1);
            x.Lc = h->lev[level + 1].L;
        }
        if (rst) {
            x.rc = h->lev[level + 1].rhs;
            x.Lr = h->lev[level + 1].L;
            if (rst_zero) {
                x.zc = cur_err(h, level + 1);
                x.zn = h->lev[level + 1].L.plane;
            }
        }
        if (launch_visit_cluster(h->st, lv, lv.err[lv.ecur], cv, tv, (h->ctab_level == level) ? h->ctab : nullptr,
                                 Niter, pp, h->p.Vbc, &h->ds->visit_timeout, &x,
                                 h->wait_test ? &h->ds->never_set : nullptr) == 0)
            return;
    }
    if (pro) launch_prolong(h->st, h->lev[level + 1], lv, cur_err(h, level + 1), cur_err(h, level), h->p.Vbc);
    const int per_point = (dir != 1 && cheb_pp) ? 1 : 0;
    int flips = 0;
    for (int n = 1; n <= Niter;) {
        double cs[2], ts[2];
        for (int j = 0; j < 2 && n + j <= Niter; j++) sweep_factors(Niter, n + j, dir, cheb_pp, &cs[j], &ts[j]);
        const int ns = (lv.blk == 2 && n + 1 <= Niter) ? 2 : (lv.blk >= 1 ? 1 : 0);
        if (ns > 0 &&
            launch_sweep_blk64(h->st, lv, lv.err[lv.ecur], lv.err[1 - lv.ecur], ns, cs, ts, per_point, h->p.Vbc)) {
            n += ns;
        } else {
            launch_sweep(h->st, lv, lv.err[lv.ecur], lv.err[1 - lv.ecur], cs[0], per_point, ts[0], h->p.Vbc);
            n += 1;
        }
        lv.ecur = 1 - lv.ecur;
        flips++;
    }
    if (flips % 2 == 1) {
        // keep the level's current buffer fixed across visits (graph replay relies on it)
        launch_copy_plane(h->st, lv.err[1 - lv.ecur], lv.err[lv.ecur], lv.L.plane);
        lv.ecur = 1 - lv.ecur;
    }
    launch_residual(h->st, lv, lv.err[lv.ecur], h->rs, &h->ds->res_mag[level]);
    if (rst)
        launch_restrict_res(h->st, h->lev[level + 1], lv, lv.res, h->lev[level + 1].rhs,
                            rst_zero ? cur_err(h, level + 1) : nullptr);
}

// Transfers of cycle step pp that the adjacent visits take over: the
// restriction into the next step's level when this step's visit fuses and
// the cycle goes down; the prolongation out of this step's level when the
// next step's visit fuses and the cycle goes up.
struct StepFusion {
    int rst = 0, rst_zero = 0, pro_next = 0;
};
static StepFusion step_fusion(Handle* h, int pp) {
    StepFusion f;
    const int G = h->grids, level = h->multi[pp];
    const int dir = (h->multi[pp + 1] > level) ? 0 : 1;
    if (level < G && h->multi[pp + 1] == level + 1 && visit_fuses(h, level, dir)) {
        f.rst = 1;
        f.rst_zero = (level + 1 < G && h->p.mg_zero_coarse) ? 1 : 0;
    }
    if (pp + 1 <= h->nsteps && h->multi[pp + 1] == level - 1) {
        const int nl = level - 1;
        f.pro_next = visit_fuses(h, nl, (h->multi[pp + 2] > nl) ? 0 : 1) ? 1 : 0;
    }
    return f;
}

// cycle_correction: the minimal-residual correction of the level-1
// streamfunction after each level-1 visit, along the change of psi since the
// previous one (one whole W-cycle: coarse-grid correction and smoothing)
// and, with cycle_correction = 2, the network's direction.  It runs at the
// smoothed point of the cycle: right after the coarse-grid correction (level
// 1 has no second visit in the reference's tables) psi carries the
// prolongation's high-frequency error, which dominates the residual, and a
// step there tends to cancel the cycle.  The residual the convergence test
// reads is taken after the correction.
// returns true when the correction wrote the level-1 residual and its mean
// (the windowed correction), false when the residual kernel must follow
bool enqueue_cycle_correction(Handle* h) {
    if (h->p.cycle_correction == 0 || h->acc_prev == nullptr) return false;
    if (h->p.cycle_correction >= 3) {
        launch_accel_window(h->st, h->lev[1], cur_err(h, 1), h->acc_prev, h->win_p, h->win_ap, h->win_rn,
                            h->win_rp, h->acc_dnn, h->win_adnn, (h->p.cycle_correction == 4 && h->acc_dnn_on) ? 1 : 0,
                            h->rs, h->ds, h->p.Vbc);
        return true;
    }
    const int k2 = (h->p.cycle_correction == 2 && h->acc_dnn_on) ? TC_ACCEL_DNN : TC_ACCEL_NONE;
    launch_accel(h->st, h->lev[1], cur_err(h, 1), h->acc_prev, h->acc_dnn, TC_ACCEL_DK, k2, 1, h->rs, h->ds,
                 h->p.Vbc);
    return false;
}

// Work of one multigrid cycle after the level-1 visit (p = 2..nsteps);
// no host synchronisation inside, so it can be captured in a CUDA graph.
void enqueue_cycle_rest(Handle* h) {
    const int G = h->grids;
    bool restricted = false, pending_pro = false;
    for (int pp = 2; pp <= h->nsteps; pp++) {
        const int level = h->multi[pp];
        const int dir = (h->multi[pp + 1] > h->multi[pp]) ? 0 : 1;
        const bool zero = h->multi[pp - 1] < h->multi[pp] && level > 1 && level < G && h->p.mg_zero_coarse;
        if (h->multi[pp - 1] < h->multi[pp] && level > 1 && !restricted)
            launch_restrict_res(h->st, h->lev[level], h->lev[level - 1], h->lev[level - 1].res, h->lev[level].rhs,
                                zero ? cur_err(h, level) : nullptr);
        // the sub-cycle below level grids-1 entered here: one product with its
        // matrix, then continue with the step that leaves level grids-1
        const int sub = h->sub_on ? h->sub_k[pp] : 0;
        if (sub) {
            launch_subcycle_apply(h->st, h->lev[level], h->subM[sub - 1], 0, 0, cur_err(h, level), h->p.Vbc);
            pp = h->sub_end[pp];
        }
        const StepFusion f = step_fusion(h, pp);
        if (sub) {
        } else if (level < G) {
            iterate_stream(h, level, dir, pending_pro ? 1 : 0, f.rst, f.rst_zero);
        } else {
            if (h->coarse_banded)
                launch_coarse_solve(h->st, h->lev[G], h->band, h->ipiv, h->rowb, h->ngrid_coarse, h->kl, h->ku,
                                    cur_err(h, G), h->p.Vbc);
            else
                launch_coarse_apply(h->st, h->lev[G], h->ainv, h->rowb, h->ngrid_coarse, h->coarse_q, h->coarse_x,
                                    h->coarse_m, cur_err(h, G), h->p.Vbc);
        }
        restricted = f.rst != 0;
        pending_pro = false;
        if (h->multi[pp + 1] < h->multi[pp]) {
            if (f.pro_next) pending_pro = true;
            else
                launch_prolong(h->st, h->lev[level], h->lev[level - 1], cur_err(h, level), cur_err(h, level - 1),
                               h->p.Vbc);
        }
    }
}

// ---- mixed precision (solver_precision = 1) --------------------------------
float* cur_e32(Handle* h, int l) { return h->lev[l].e32[h->lev[l].e32cur]; }

// iterate_stream on the FP32 correction of `level` (same sweeps and factors
// as iterate_stream); level 1 skips the FP32 residual (its residual is FP64).
void iterate_stream32(Handle* h, int level, int dir, int pro = 0, int rst = 0, int rst_zero = 0) {
    Level& lv = h->lev[level];
    const int Niter = h->p.Nmulti;
    const bool cheb_pp = (level == h->ratio_level);
    const int pp = (dir != 1 && cheb_pp) ? 1 : 0;
    if (h->fuse_visits && lv.fuse && level > 1 && Niter <= 128) {
        double cv[128], tv[128];
        cheb_temps(Niter, dir, tv, cv);
        VisitXfer<float> x;
        if (pro) {
            x.ec = cur_e32(h, level + 1);
            x.Lc = h->lev[level + 1].L;
        }
        if (rst) {
            x.rc = h->lev[level + 1].rhs32;
            x.Lr = h->lev[level + 1].L;
            if (rst_zero) {
                x.zc = cur_e32(h, level + 1);
                x.zn = h->lev[level + 1].L.plane;
            }
        }
        if (launch_visit_cluster32(h->st, lv, cur_e32(h, level), cv, tv, Niter, pp, h->p.Vbc,
                                   &h->ds->visit_timeout, &x, h->wait_test ? &h->ds->never_set : nullptr) == 0)
            return;
    }
    if (pro) launch_prolong32(h->st, h->lev[level + 1], lv, cur_e32(h, level + 1), cur_e32(h, level), h->p.Vbc);
    int flips = 0;
    for (int n = 1; n <= Niter;) {
        // lv.blk sweeps per launch of the tiled smoother, the remainder of the
        // visit in one last launch (lv.blk = 0: k_sweep32; a level swept from
        // its viscosity fields, g32: lv.blk = 2 or 3 sweeps per k_sweep_gblk
        // launch, a remainder of one as a k_sweep_g32 sweep)
        const bool gf = lv.g32 && lv.use_g32;
        const int blk = gf ? ((lv.blk == 2 || lv.blk == 3) ? lv.blk : 0) : lv.blk;
        const int ns = (blk >= 1) ? std::min(blk, Niter - n + 1) : 0;
        float cs[6], ts[6];
        for (int j = 0; j < (ns > 0 ? ns : 1); j++) {
            double c, temp;
            sweep_factors(Niter, n + j, dir, cheb_pp, &c, &temp);
            cs[j] = (float)c;
            ts[j] = (float)temp;
        }
        if (ns > 0 && (gf ? launch_sweep_gblk32(h->st, lv, lv.e32[lv.e32cur], lv.e32[1 - lv.e32cur], ns, cs, ts, pp,
                                                 h->p.Vbc)
                          : launch_sweep_blk32(h->st, lv, lv.e32[lv.e32cur], lv.e32[1 - lv.e32cur], ns, cs, ts, pp,
                                               h->p.Vbc))) {
            n += ns;
        } else {
            launch_sweep32(h->st, lv, lv.e32[lv.e32cur], lv.e32[1 - lv.e32cur], cs[0], pp, ts[0], h->p.Vbc);
            n += 1;
        }
        lv.e32cur = 1 - lv.e32cur;
        flips++;
    }
    if (flips % 2 == 1) {
        CKV(cudaMemcpyAsync(lv.e32[1 - lv.e32cur], lv.e32[lv.e32cur], sizeof(float) * lv.L.plane,
                            cudaMemcpyDeviceToDevice, h->st));
        lv.e32cur = 1 - lv.e32cur;
    }
    if (level > 1) launch_residual32(h->st, lv, cur_e32(h, level));
    if (rst)
        launch_restrict32(h->st, h->lev[level + 1], lv, lv.res32, h->lev[level + 1].rhs32,
                          rst_zero ? cur_e32(h, level + 1) : nullptr);
}

// level-1 visit of the mixed solve: r = RHS - L psi (FP64) -> FP32 RHS,
// correction from zero, psi += e (FP64), FP64 residual and its L1 mean
void enqueue_l1_mixed(Handle* h, int dir) {
    Level& l1 = h->lev[1];
    launch_residual_to32(h->st, l1, cur_err(h, 1), l1.rhs32, cur_e32(h, 1));
    iterate_stream32(h, 1, dir);
    launch_update64(h->st, l1, cur_err(h, 1), cur_e32(h, 1), h->p.Vbc);
    if (!enqueue_cycle_correction(h)) launch_residual(h->st, l1, cur_err(h, 1), h->rs, &h->ds->res_mag[1]);
}

// p = 2..nsteps of the mixed solve (enqueue_cycle_rest on FP32 corrections)
void enqueue_rest_mixed(Handle* h, int) {
    const int G = h->grids;
    bool restricted = false, pending_pro = false;
    for (int pp = 2; pp <= h->nsteps; pp++) {
        const int level = h->multi[pp];
        const int dir = (h->multi[pp + 1] > h->multi[pp]) ? 0 : 1;
        const bool down = h->multi[pp - 1] < h->multi[pp];
        float* zero = (down && level > 1 && level < G && h->p.mg_zero_coarse) ? cur_e32(h, level) : nullptr;
        if (down && level == 2)
            launch_restrict64to32(h->st, h->lev[2], h->lev[1], h->lev[1].res, h->lev[2].rhs32, zero);
        else if (down && level > 2 && !restricted)
            launch_restrict32(h->st, h->lev[level], h->lev[level - 1], h->lev[level - 1].res32, h->lev[level].rhs32,
                              zero);
        const int sub = h->sub_on ? h->sub_k[pp] : 0;
        if (sub) {
            launch_subcycle_apply(h->st, h->lev[level], h->subM[sub - 1], 1, h->sub_m32 ? 1 : 0, cur_e32(h, level),
                                  h->p.Vbc);
            pp = h->sub_end[pp];
        }
        const StepFusion f = step_fusion(h, pp);
        if (sub) {
        } else if (level < G) iterate_stream32(h, level, dir, pending_pro ? 1 : 0, f.rst, f.rst_zero);
        else if (h->coarse_banded)
            launch_coarse_solve32(h->st, h->lev[G], h->band, h->ipiv, h->rowb, h->ngrid_coarse, h->kl, h->ku,
                                  cur_e32(h, G), h->p.Vbc);
        else launch_coarse_apply32(h->st, h->lev[G], h->ainv, h->rowb, h->ngrid_coarse, h->coarse_q, h->coarse_x,
                                   h->coarse_m, cur_e32(h, G), h->p.Vbc);
        restricted = f.rst != 0;
        pending_pro = false;
        if (h->multi[pp + 1] < h->multi[pp]) {
            if (level == 2)
                launch_prolong_into64(h->st, h->lev[2], h->lev[1], cur_e32(h, 2), cur_err(h, 1), h->p.Vbc);
            else if (f.pro_next)
                pending_pro = true;
            else
                launch_prolong32(h->st, h->lev[level], h->lev[level - 1], cur_e32(h, level), cur_e32(h, level - 1),
                                 h->p.Vbc);
        }
    }
}

// Graph of a replayable sequence; rebuilt when the inputs it bakes in change.
struct CycleGraphs {
    cudaGraphExec_t l1 = nullptr, rest = nullptr;
    long long n_l1 = 0, n_rest = 0;  // kernel nodes per graph
    // the whole solve with its convergence loop on the device (k_loop.cu):
    // kernels before the WHILE node and in its body
    cudaGraphExec_t loop = nullptr;
    long long n_pre = 0, n_body = 0;
    bool loop_failed = false;  // the CUDA runtime refused the conditional node: host loop
    int ratio_level = -1, zero = -1, dir1 = -1, dnn = -1;
    cudaStream_t st = nullptr;
};

tc_status capture(Handle* h, cudaGraphExec_t* out, void (*fn)(Handle*, int), int arg, long long* nkernels) {
    cudaGraph_t g = nullptr;
    const long long before = t_launches;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    fn(h, arg);
    CK(cudaStreamEndCapture(h->st, &g));
    if (h->enq_err != cudaSuccess) {
        cudaGraphDestroy(g);
        CK(h->enq_err);
    }
    *nkernels = t_launches - before;
    g_launches.fetch_sub(*nkernels);  // capturing enqueues nothing
    t_launches -= *nkernels;
    cudaError_t e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { h->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e); return TC_ERR_CUDA; }
    return TC_OK;
}
// The solve as one graph: [init, level-1 visit, check] then a WHILE node
// whose body is [rest of the cycle, level-1 visit, check]; both parts are
// filled by stream capture (cudaStreamBeginCaptureToGraph).  Returns false
// (with the stream out of capture and no error left pending) when the
// CUDA runtime does not take the conditional node.
bool build_loop_graph(Handle* h, void (*f_l1)(Handle*, int), void (*f_rest)(Handle*, int), int dir1,
                      cudaGraphExec_t* out, long long* n_pre, long long* n_body) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
    cudaGraphConditionalHandle cond;
    if (cudaGraphConditionalHandleCreate(&cond, g, 0, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        return false;
    }
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    long long before = t_launches;
    h->enq_err = cudaSuccess;
    if (cudaStreamBeginCaptureToGraph(h->st, g, nullptr, nullptr, 0, mode) != cudaSuccess) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        return false;
    }
    launch_cycle_init(h->st, h->ds);
    f_l1(h, dir1);
    launch_cycle_check(h->st, h->ds, h->p.tolerance, h->p.max_cycles, cond);
    cudaStreamCaptureStatus cs;
    cudaGraph_t capg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t wn = nullptr;
    bool ok = cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &capg, &deps, nullptr, &nd) == cudaSuccess &&
              cs == cudaStreamCaptureStatusActive &&
              cudaGraphAddNode(&wn, capg, deps, nullptr, nd, &np) == cudaSuccess &&
              cudaStreamUpdateCaptureDependencies(h->st, &wn, nullptr, 1, cudaStreamSetCaptureDependencies) ==
                  cudaSuccess;
    cudaGraph_t g2 = nullptr;
    const bool ended = cudaStreamEndCapture(h->st, &g2) == cudaSuccess;
    *n_pre = t_launches - before;
    g_launches.fetch_sub(*n_pre);
    t_launches = before;
    if (!ok || !ended || h->enq_err != cudaSuccess) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        h->enq_err = cudaSuccess;
        return false;
    }
    cudaGraph_t body = np.conditional.phGraph_out[0];
    before = t_launches;
    ok = cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0, mode) == cudaSuccess;
    if (ok) {
        f_rest(h, 0);
        f_l1(h, dir1);
        launch_cycle_check(h->st, h->ds, h->p.tolerance, h->p.max_cycles, cond);
        cudaGraph_t b2 = nullptr;
        ok = cudaStreamEndCapture(h->st, &b2) == cudaSuccess;
    }
    *n_body = t_launches - before;
    g_launches.fetch_sub(*n_body);
    t_launches = before;
    cudaGraphExec_t ge = nullptr;
    if (ok && h->enq_err == cudaSuccess) ok = cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
    else ok = false;
    cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        h->enq_err = cudaSuccess;
        return false;
    }
    *out = ge;
    return true;
}

void enqueue_l1(Handle* h, int dir) {
    iterate_stream(h, 1, dir);
    if (h->p.cycle_correction != 0 && h->acc_prev != nullptr) {
        if (!enqueue_cycle_correction(h)) launch_residual(h->st, h->lev[1], cur_err(h, 1), h->rs, &h->ds->res_mag[1]);
    }
}
void enqueue_rest(Handle* h, int) { enqueue_cycle_rest(h); }

void compute_velocities(Handle* h);

// multigrid (iterative_solver.f90:79-173).  Newtonian rheology
// (non_Newtonian = 0): viscosities, level operators and the coarse LU once
// per solve.  non_Newtonian = 1: every cycle starts from the current
// correction (SF = error(1), velocities, strain rate) and rebuilds every
// level's viscosity, local time steps and the coarse LU; after the level-1
// visit the level-1 viscosity is brought up to date and the residual the
// convergence test reads is taken with it (iterative_solver.f90:106-116,
// 141-148).  The non-Newtonian iteration runs in FP64 without the learned
// start and issues its launches directly (its level setup has host-side
// loops between kernels).
// The device-side convergence loop's outcome after a read of the scalars:
// its W-cycle count and stop reason (iterative_solver.f90:147-156); the
// kernels it ran are n_pre before the WHILE node and n_body per pass.
tc_status loop_result(Handle* h, long long n_pre, long long n_body) {
    const int q = h->hs->cyc_q;
    const int st = h->hs->cyc_status;
    const long long bodies = (st == TC_ERR_MG_CYCLES) ? q - 2 : q - 1;
    tc_note_launch(n_pre + (bodies > 0 ? bodies : 0) * n_body);
    if (h->hs->visit_timeout || st == TC_ERR_DEVICE_TIMEOUT) {
        h->err = "fused smoother visit: neighbour wait exceeded its bound";
        return TC_ERR_DEVICE_TIMEOUT;
    }
    if (st == TC_ERR_MG_RESIDUAL) return TC_ERR_MG_RESIDUAL;
    h->last_cycles = q;
    if (st == TC_ERR_MG_CYCLES) return TC_ERR_MG_CYCLES;
    if (st != 0) return (tc_status)st;
    h->cycles_acc += q;
    return TC_OK;
}

tc_status multigrid(Handle* h) {
    if (!h->uploaded) return TC_ERR_STATE;
    const bool nonN = (h->p.non_Newtonian == 1);
    const int G = h->grids;
    const bool mixed = (h->p.solver_precision == 1);
    copy_plane(h, cur_err(h, 1), h->SF);
    launch_rhs1(h->st, h->L1, h->P, h->Tbuoy, h->Cbuoy, h->lev[1].rhs, h->rs, h->ds);
    // compute_viscosity + iterate_local_time_steps of every level, in the
    // folded form the sweeps read
    auto level_setup = [&]() -> tc_status {
        for (int l = 1; l <= G; l++) TRY(compute_viscosity(h, l));
        for (int l = 1; l <= G; l++)
            launch_level_coefs(h->st, h->lev[l], cur_vis(h, l), h->p.ivis, h->p.courant_stream,
                               l == h->ratio_level ? 1 : 0);
        if (mixed) {
            for (int l = 1; l < G; l++) launch_level_to_f32(h->st, h->lev[l], l == h->ratio_level ? 1 : 0);
            if (h->lev[1].g32) launch_level_g32(h->st, h->lev[1], cur_vis(h, 1));
        }
        h->ctab_level = 0;
        if (!mixed && h->ctab && h->ratio_level > 1 && h->p.Nmulti <= 128 &&
            visit_cluster_fits(h->lev[h->ratio_level].L, h->p.Nmulti, 0)) {
            double cv[128], tv[128];
            cheb_temps(h->p.Nmulti, 0, tv, cv);
            launch_cheb_table(h->st, h->lev[h->ratio_level], tv, h->p.Nmulti, h->ctab);
            h->ctab_level = h->ratio_level;
        }
        return TC_OK;
    };
    // Compute_Matrix_coarse + DGBTRF (and the explicit inverse the coarse visits apply)
    auto coarse_setup = [&]() {
        launch_coarse_build(h->st, h->lev[G], h->band, h->rowb, h->kl, h->ku, h->p.Vbc);
        launch_coarse_lu(h->st, h->band, h->ipiv, h->ngrid_coarse, h->kl, h->ku, h->ds);
        if (!h->coarse_banded)
            launch_coarse_inverse(h->st, h->band, h->ipiv, h->ngrid_coarse, h->kl, h->ku, h->ainv, h->bvec);
        h->lu_valid = true;
    };
    // SF = error(1); compute_velocities; compute_strain_rate_invariant
    auto strain_from_correction = [&]() {
        copy_plane(h, h->SF, cur_err(h, 1));
        compute_velocities(h);
        launch_strain(h->st, h->L1, h->P, h->u, h->w, h->strain);
    };
    // the bottom of the W-cycle as matrices M_k (k_subcycle.cu): the level
    // grids-1 sweep tables of a downward and an upward visit, then one CTA
    // per column runs the sub-cycle on a unit vector
    auto subcycle_setup = [&]() -> tc_status {
        const int S = G - 1, Nm = h->p.Nmulti;
        const bool cheb_pp = (S == h->ratio_level);
        std::vector<double> tv((size_t)4 * Nm);
        for (int dir = 0; dir < 2; dir++)
            for (int n = 1; n <= Nm; n++)
                sweep_factors(Nm, n, dir, cheb_pp, &tv[(size_t)(2 * dir) * Nm + n - 1],
                              &tv[(size_t)(2 * dir + 1) * Nm + n - 1]);
        // the sweep tables depend on Nmulti and the Chebyshev flag only: uploaded
        // once (a captured step cannot copy from pageable host memory)
        const long long key = (long long)Nm * 4 + (cheb_pp ? 2 : 0) + (h->sub_m32 ? 1 : 0);
        if (h->sub_tab_key != key) {
            if (h->capturing) {
                if (h->enq_err == cudaSuccess) h->enq_err = cudaErrorStreamCaptureUnsupported;
                return TC_OK;
            }
            if (h->sub_m32) {
                std::vector<float> tf(tv.begin(), tv.end());
                CK(cudaMemcpyAsync(h->sub_tab, tf.data(), sizeof(float) * tf.size(), cudaMemcpyHostToDevice, h->st));
            } else {
                CK(cudaMemcpyAsync(h->sub_tab, tv.data(), sizeof(double) * tv.size(), cudaMemcpyHostToDevice, h->st));
            }
            CK(cudaStreamSynchronize(h->st));
            h->sub_tab_key = key;
        }
        if (cheb_pp) {
            if (h->sub_m32) launch_cheb_table32(h->st, h->lev[S], tv.data() + Nm, Nm, (float*)h->sub_ctab);
            else launch_cheb_table(h->st, h->lev[S], tv.data() + Nm, Nm, h->sub_ctab);
        }
        if (launch_subcycle_build(h->st, h->lev[S], h->lev[G], h->sub_m32 ? 1 : 0, h->sub_tab, h->sub_ctab, Nm,
                                  cheb_pp ? 1 : 0,
                                  h->ainv, h->rowb, h->coarse_q, h->coarse_x, h->ngrid_coarse, h->coarse_m,
                                  h->p.Vbc, h->sub_kmax, (void* const*)h->subM, h->sub_ac) != 0) {
            h->err = "k_subcycle_build: launch failed";
            return TC_ERR_CUDA;
        }
        h->sub_valid = true;
        return TC_OK;
    };
    // the network's predicted change of this solve, d = guess - SF
    // (learned_guess = 3: the start SF + alpha d, alpha residual-minimising;
    // cycle_correction = 2 / 4: d spans the correction with the cycles' own)
    h->acc_dnn_on = h->net != nullptr && !nonN && h->acc_dnn != nullptr &&
                    (h->p.learned_guess == 3 || h->p.cycle_correction == 2 || h->p.cycle_correction == 4);
    if (!nonN) {
        TRY(level_setup());
        const bool rebuild = (h->time == 0.0 || h->p.ivis > 0 || !h->lu_valid);
        if (rebuild) coarse_setup();
        if (h->sub_on && (rebuild || !h->sub_valid)) TRY(subcycle_setup());
    }
    CK(cudaMemsetAsync(&h->ds->visit_timeout, 0, sizeof(int), h->st));
    const size_t img = (size_t)h->nx * h->nz;
    const bool rec = h->rec_raw && h->rec_count < h->rec_cap;
    if (rec)
        nn_fields_to_raw(h->st, h->lev[1].L, cur_vis(h, 1), h->lev[1].rhs, cur_err(h, 1),
                         h->rec_raw + (size_t)h->rec_count * 3 * img);
    const int kGuessPatience = 8, kGuessProbe = 32;
    bool try_guess = (h->p.learned_guess == 1 || h->p.learned_guess == 2) && h->net != nullptr && !nonN;
    if (try_guess && h->p.learned_guess == 1 && h->guess_reject_streak >= kGuessPatience &&
        (h->guess_solves % kGuessProbe) != 0)
        try_guess = false;
    if (h->p.learned_guess != 0 && h->net != nullptr) h->guess_solves++;
    if (try_guess) {
        // candidate start from the network; with learned_guess = 1 it is kept
        // only if its level-1 residual is smaller
        if (nn_guess(h->net, h->st, h->lev[1].L, cur_vis(h, 1), h->lev[1].rhs, cur_err(h, 1), h->nn_raw, h->guess,
                     h->p.Vbc, h->p.learned_smooth) != 0) {
            h->err = "learned guess: network forward failed";
            return TC_ERR_CUDA;
        }
        CK(cudaMemcpyAsync(&h->ds->net_fail, net_fail(h->net), sizeof(int), cudaMemcpyDeviceToDevice, h->st));
        launch_residual(h->st, h->lev[1], cur_err(h, 1), h->rs, &h->ds->res_mag[1]);
        launch_residual(h->st, h->lev[1], h->guess, h->rs, &h->ds->res_mag[0]);
    }
    if (h->acc_dnn_on) {
        if (nn_guess(h->net, h->st, h->lev[1].L, cur_vis(h, 1), h->lev[1].rhs, cur_err(h, 1), h->nn_raw, h->guess,
                     h->p.Vbc, h->p.learned_smooth) != 0) {
            h->err = "learned guess: network forward failed";
            return TC_ERR_CUDA;
        }
        CK(cudaMemcpyAsync(&h->ds->net_fail, net_fail(h->net), sizeof(int), cudaMemcpyDeviceToDevice, h->st));
        launch_plane_diff(h->st, h->acc_dnn, h->guess, cur_err(h, 1), h->L1.plane);
        if (h->p.learned_guess == 3)
            launch_accel(h->st, h->lev[1], cur_err(h, 1), nullptr, h->acc_dnn, TC_ACCEL_DNN, TC_ACCEL_NONE, 0, h->rs,
                         h->ds, h->p.Vbc);
    }
    // the start's read: the network's wait flag, the learned start's
    // bookkeeping and the coarse LU's pivot test
    const bool dnn_on = h->acc_dnn_on, lg3 = (h->p.learned_guess == 3);
    TRY(sync_point(h, [h, dnn_on, lg3]() -> tc_status {
        if (dnn_on) {
            if (h->hs->net_fail) {
                h->err = "learned guess: a convolution's bounded wait gave up";
                return TC_ERR_DEVICE_TIMEOUT;
            }
            if (lg3) {
                h->guess_offered++;
                if (h->hs->acc_alpha[0] != 0.0) h->guess_used++;
            }
        }
        if (h->hs->lu_info != 0) return TC_ERR_SINGULAR;
        return TC_OK;
    }));
    if (h->p.cycle_correction != 0 && h->acc_prev != nullptr && !nonN) {
        copy_plane(h, h->acc_prev, cur_err(h, 1));
        if (h->p.cycle_correction >= 3) {
            // a new window per solve: the start's residual and the network direction's image
            CK(cudaMemsetAsync(&h->ds->win_n, 0, sizeof(int), h->st));
            const bool dnn = (h->p.cycle_correction == 4 && h->acc_dnn_on);
            launch_accel_window_init(h->st, h->lev[1], h->acc_prev, dnn ? h->acc_dnn : nullptr, h->win_rp,
                                     dnn ? h->win_adnn : nullptr);
        }
    }
    if (try_guess) {
        if (h->hs->net_fail) {
            h->err = "learned guess: a convolution's bounded wait gave up";
            return TC_ERR_DEVICE_TIMEOUT;
        }
        h->guess_offered++;
        if (h->p.learned_guess == 2 || h->hs->res_mag[0] < h->hs->res_mag[1]) {
            copy_plane(h, cur_err(h, 1), h->guess);
            h->guess_used++;
            h->guess_reject_streak = 0;
        } else {
            h->guess_reject_streak++;
        }
    }
    const double res_ref1 = h->hs->res_ref;
    // p=1 is the only level-1 visit of every cycle table; the convergence test
    // follows it, then p=2..nsteps run unconditionally.
    const int dir1 = (h->multi[2] > h->multi[1]) ? 0 : 1;
    CycleGraphs& cg = *h->graphs;
    const bool use_graphs = (h->st != nullptr) && !h->no_graphs && !nonN;
    void (*f_l1)(Handle*, int) = mixed ? enqueue_l1_mixed : enqueue_l1;
    void (*f_rest)(Handle*, int) = mixed ? enqueue_rest_mixed : enqueue_rest;
    if (h->capturing) {
        // inside a captured step: the convergence loop as this step's own
        // WHILE node, its result read after the step
        long long n_body = 0;
        emit_while(
            h,
            [&](cudaGraphConditionalHandle c) {
                launch_cycle_init(h->st, h->ds);
                f_l1(h, dir1);
                launch_cycle_check(h->st, h->ds, h->p.tolerance, h->p.max_cycles, c);
            },
            [&](cudaGraphConditionalHandle c) {
                f_rest(h, 0);
                f_l1(h, dir1);
                launch_cycle_check(h->st, h->ds, h->p.tolerance, h->p.max_cycles, c);
            },
            &n_body);
        TRY(sync_point(h, [h, n_body]() { return loop_result(h, 0, n_body); }));
        copy_plane(h, h->SF, cur_err(h, 1));
        return TC_OK;
    }
    h->enq_err = cudaSuccess;
    if (use_graphs && (cg.l1 == nullptr || cg.ratio_level != h->ratio_level || cg.zero != h->p.mg_zero_coarse ||
                       cg.dir1 != dir1 || cg.st != h->st || cg.dnn != (h->acc_dnn_on ? 1 : 0))) {
        if (cg.l1) cudaGraphExecDestroy(cg.l1);
        if (cg.rest) cudaGraphExecDestroy(cg.rest);
        if (cg.loop) cudaGraphExecDestroy(cg.loop);
        cg.l1 = cg.rest = cg.loop = nullptr;
        TRY(capture(h, &cg.l1, f_l1, dir1, &cg.n_l1));
        TRY(capture(h, &cg.rest, f_rest, 0, &cg.n_rest));
        if (!cg.loop_failed && !h->no_device_loop &&
            !build_loop_graph(h, f_l1, f_rest, dir1, &cg.loop, &cg.n_pre, &cg.n_body))
            cg.loop_failed = true;
        cg.ratio_level = h->ratio_level;
        cg.zero = h->p.mg_zero_coarse;
        cg.dir1 = dir1;
        cg.st = h->st;
        cg.dnn = h->acc_dnn_on ? 1 : 0;
    }
    int q = 1;
    if (use_graphs && cg.loop != nullptr) {
        // the whole convergence loop on the device; one host read per solve
        CK(cudaGraphLaunch(cg.loop, h->st));
        TRY(sync_point(h, [h, &cg]() { return loop_result(h, cg.n_pre, cg.n_body); }));
        copy_plane(h, h->SF, cur_err(h, 1));
        if (rec) {
            nn_field_to_img(h->st, h->lev[1].L, h->SF, h->rec_sf + (size_t)h->rec_count * img);
            h->rec_count++;
        }
        return TC_OK;
    }
    for (;;) {
        if (nonN) {
            strain_from_correction();
            TRY(level_setup());
            coarse_setup();
        }
        if (use_graphs) { CK(cudaGraphLaunch(cg.l1, h->st)); tc_note_launch(cg.n_l1); }
        else f_l1(h, dir1);
        CK(h->enq_err);
        if (nonN) {
            // the level-1 viscosity of the new correction, its operator (the
            // local time steps stay those of the cycle start) and the residual
            strain_from_correction();
            TRY(compute_viscosity(h, 1));
            launch_level_coefs(h->st, h->lev[1], cur_vis(h, 1), h->p.ivis, h->p.courant_stream,
                               h->ratio_level == 1 ? 1 : 0, false);
            launch_residual(h->st, h->lev[1], cur_err(h, 1), h->rs, &h->ds->res_mag[1]);
        }
        TRY(sync_scalars(h));
        if (nonN && h->hs->lu_info != 0) return TC_ERR_SINGULAR;
        if (h->hs->visit_timeout) {
            h->err = "fused smoother visit: neighbour wait exceeded its bound";
            return TC_ERR_DEVICE_TIMEOUT;
        }
        const double rm = h->hs->res_mag[1];
        if (rm > 1.0e10 * res_ref1) return TC_ERR_MG_RESIDUAL;
        if (rm / res_ref1 <= h->p.tolerance) break;
        if (use_graphs) { CK(cudaGraphLaunch(cg.rest, h->st)); tc_note_launch(cg.n_rest); }
        else f_rest(h, 0);
        CK(h->enq_err);
        q = q + 1;
        if (q > h->p.max_cycles) { h->last_cycles = q; return TC_ERR_MG_CYCLES; }
    }
    copy_plane(h, h->SF, cur_err(h, 1));
    h->last_cycles = q;
    h->cycles_acc += q;
    if (rec) {
        nn_field_to_img(h->st, h->lev[1].L, h->SF, h->rec_sf + (size_t)h->rec_count * img);
        h->rec_count++;
    }
    return TC_OK;
}

void compute_velocities(Handle* h) { launch_velocities(h->st, h->L1, h->P, h->SF, h->u, h->w); }

// the tracer and RK2 stop tests of the reference (energy.f90) on the last read
tc_status flags_result(Handle* h) {
    if (h->hs->flag_outside) return TC_ERR_TRACER_OUTSIDE;
    if (h->hs->flag_rk2) return TC_ERR_RK2_STABILITY;
    return TC_OK;
}

tc_status check_flags(Handle* h) {
    return sync_point(h, [h]() { return flags_result(h); });
}

tc_status update_velocities(Handle* h) {
    TRY(multigrid(h));
    compute_velocities(h);
    return TC_OK;
}

// equalize_tracers (composition.f90:83-580), then tracers_to_corners with
// smoothing off (:576-578)
tc_status equalize_tracers(Handle* h) {
    EqHost H{};
    H.L = h->L1; H.P = h->P; H.ntype = h->ntype; H.NR = h->eq_NR; H.comp = h->p.comp; H.tracer = h->p.tracer;
    H.tpc = h->p.tpc; H.ntr = h->ntr; H.dist_r = h->p.dist_factor * h->P.dr; H.dist_s = h->p.dist_factor * h->P.ds;
    if (h->p.comp == 1) {
        long long sum = 0;
        for (int t = 1; t <= h->ntype; t++) {
            H.Nideal[t] = std::llround(h->Cinit[t - 1] * (double)h->ntr);
            sum += H.Nideal[t];
        }
        H.Nideal[0] = h->ntr - sum;
    } else {
        H.Nideal[0] = h->ntr;
    }
    H.counts = h->counts; H.nempty = h->nempty; H.Cnew = h->Cnew; H.rtr = h->rtr; H.str = h->str;
    H.ttype = h->ttype; H.perm = h->perm; H.iperm = h->eq_iperm; H.nex = h->eq_nex; H.off = h->eq_off;
    H.cur = h->eq_cur; H.ids = h->eq_ids; H.cnt = h->eq_cnt; H.bsum = h->sort_bsum; H.seeds = h->eq_seeds;
    H.isv = h->eq_isv; H.isv2 = h->eq_isv2; H.nfr = h->eq_nfr; H.nx_loop = h->eq_nxl; H.nz_loop = h->eq_nzl;
    H.sc = h->eq_sc; H.Tratio = h->Tratio; H.Td = h->eq_Td; H.dTd = h->eq_dTd; H.Ttr = h->Ttr;
    int64_t nfree = 0;
    int nonzero = 0;
    if (launch_equalize_count(h->st, H, &nfree, &nonzero) != 0) { CK(cudaGetLastError()); return TC_ERR_CUDA; }
    h->eq_row.clear();
    if (!nonzero) return TC_OK;
    h->nequalize++;
    const size_t need = (size_t)h->eq_NR * (size_t)(h->ntype + 1) * (size_t)(nfree + 1);
    if (need > h->eq_donor_cap) {
        if (h->eq_donor) cudaFree(h->eq_donor);
        h->eq_donor = nullptr;
        h->eq_donor_cap = 0;
        CK(cudaMalloc((void**)&h->eq_donor, sizeof(int) * need));
        h->eq_donor_cap = need;
    }
    int64_t row[64];
    int len = 0;
    const int st = launch_equalize_move(h->st, H, nfree, h->eq_donor, row, &len);
    if (st == TC_ERR_EQUALIZE) return TC_ERR_EQUALIZE;
    if (st != 0) { CK(cudaGetLastError()); return TC_ERR_CUDA; }
    h->eq_row.assign(row, row + len);
    return tracers_to_corners(h, h->rtr, h->str, false, h->p.tracer == 1 ? h->Ttr : nullptr, h->T);
}

// energy_time (energy.f90:117-453): field T or temperature tracers,
// compositional tracers, local_time=0
tc_status energy_time(Handle* h) {
    if (!h->uploaded) return TC_ERR_STATE;
    const bool tt = (h->p.tracer == 1);
    const bool cmp = (h->p.comp == 1);
    const bool trc = cmp || tt;
    const int torder = h->p.torder;
    const bool rat = (h->p.RaT != 0.0);
    launch_stability(h->st, h->L1, h->P, h->conduct, h->conduct_r, h->conduct_s, h->u, h->w, h->p.courant,
                     h->p.dt_manual, h->rs, h->ds);
    TRY(check_flags(h));
    if (h->p.equalize == 1) TRY(equalize_tracers(h));
    for (int t = 0; t < h->ntype; t++) copy_plane(h, h->C0[t], h->Cnew[t]);
    copy_plane(h, h->T0, tt ? h->Tratio : h->T);
    if (sorts_this_step(h)) TRY(sort_tracers(h));
    // the step's start positions (and temperatures); rtr, str and Ttr are
    // the RK accumulators, which stage 1 writes first
    const size_t nb = sizeof(double) * (size_t)h->ntr;
    if (trc && h->ntr > 0) {
        CK(cudaMemcpyAsync(h->rtr0, h->rtr, nb, cudaMemcpyDeviceToDevice, h->st));
        CK(cudaMemcpyAsync(h->str0, h->str, nb, cudaMemcpyDeviceToDevice, h->st));
    }
    if (tt && h->ntr > 0) CK(cudaMemcpyAsync(h->Ttr0, h->Ttr, nb, cudaMemcpyDeviceToDevice, h->st));
    auto derivs = [&]() {
        launch_derivatives(h->st, h->L1, h->P, h->u, h->du);
        launch_derivatives(h->st, h->L1, h->P, h->w, h->dw);
    };
    auto restore_C = [&]() { for (int t = 0; t < h->ntype; t++) copy_plane(h, h->Cnew[t], h->C0[t]); };
    auto stage_T = [&](int stage, const double* Tin, double* Tout) {
        launch_energy_stage(h->st, h->L1, h->P, stage, Tin, h->T0, h->T, Tout, h->conduct, h->conduct_r, h->conduct_s,
                            h->u, h->w, h->Cvis, h->ds);
        launch_enforce_T(h->st, h->L1, stage == 4 ? h->T : Tout, h->p.Tbot);
    };
    // load_tracer_space_array + compute_derivatives(tracer_space_array)
    auto tracer_space = [&]() {
        launch_tracer_space(h->st, h->L1, h->P, h->Tratio, h->conduct, h->conduct_r, h->conduct_s, h->Cvis, h->tsa);
        launch_derivatives(h->st, h->L1, h->P, h->tsa, h->dT);
    };
    // a stage's tracer update; Tout is the stage's Ttr1/Ttr2 (temperature tracers)
    auto stage_tracers = [&](int stage, const double* rin, const double* sin, double* rout, double* sout,
                             double* Tout) {
        launch_tracer_stage(h->st, h->L1, h->P, torder, stage, h->ntr, rin, sin, h->rtr0, h->str0, h->rtr, h->str,
                            rout, sout, h->u, h->w, h->du, h->dw, h->ds, tt ? h->tsa : nullptr, h->dT, h->Ttr0,
                            h->Ttr, Tout);
    };
    // ---- stage 1 ----
    if (rat) {
        if (tt) tracer_space();
        else stage_T(1, h->T0, h->T1);
    }
    if (trc) {
        derivs();
        stage_tracers(1, h->rtr0, h->str0, h->rtr1, h->str1, h->Ttr1);
    }
    // ---- stage 2 ----
    if (tt) {
        TRY(tracers_to_corners(h, h->rtr1, h->str1, true, h->Ttr1, h->T0));
        tracer_space();
    }
    if (h->p.RK_update == 1) {
        if (cmp && !tt) TRY(tracers_to_corners(h, h->rtr1, h->str1, true));
        if (!tt) TRY(smoother_time_T(h, h->T1));
        TRY(update_velocities(h));
        if (trc) derivs();
    }
    if (rat && !tt) stage_T(2, h->T1, h->T2);
    if (trc) stage_tracers(2, h->rtr1, h->str1, h->rtr2, h->str2, h->Ttr2);
    if (torder >= 3) {
        // ---- stage 3 ----
        if (tt) {
            if (cmp) restore_C();
            TRY(tracers_to_corners(h, h->rtr2, h->str2, true, h->Ttr2, h->T0));
            tracer_space();
        }
        if (h->p.RK_update == 1) {
            if (cmp && !tt) { restore_C(); TRY(tracers_to_corners(h, h->rtr2, h->str2, true)); }
            if (!tt) TRY(smoother_time_T(h, h->T2));
            TRY(update_velocities(h));
            if (trc) derivs();
        }
        if (rat && !tt) stage_T(3, h->T2, h->T1);
        if (trc) stage_tracers(3, h->rtr2, h->str2, h->rtr1, h->str1, h->Ttr1);
        // ---- stage 4 ----
        if (tt) {
            if (cmp) restore_C();
            TRY(tracers_to_corners(h, h->rtr1, h->str1, true, h->Ttr1, h->T0));
            tracer_space();
        }
        if (h->p.RK_update == 1) {
            if (cmp && !tt) { restore_C(); TRY(tracers_to_corners(h, h->rtr1, h->str1, true)); }
            if (!tt) TRY(smoother_time_T(h, h->T1));
            TRY(update_velocities(h));
            if (trc) derivs();
        }
        if (rat && !tt) stage_T(4, h->T1, h->T1);
        if (trc) stage_tracers(4, h->rtr1, h->str1, nullptr, nullptr, nullptr);
    }
    // ---- wrap up ----
    if (cmp) restore_C();
    if (trc) TRY(tracers_to_corners(h, h->rtr, h->str, true, tt ? h->Ttr : nullptr, h->T0));
    if (tt) copy_plane(h, h->T, h->Tratio);
    else TRY(smoother_time_T(h, h->T));
    return sync_point(h, [h]() {
        TRY(flags_result(h));
        h->dt = h->hs->dt;
        return TC_OK;
    });
}

// stats (basics.f90:236-324)
tc_status stats_row(Handle* h, tc_stats_row* row);

tc_status stats(Handle* h, tc_stats_row* row) {
    launch_strain(h->st, h->L1, h->P, h->u, h->w, h->strain);
    launch_stats(h->st, h->L1, h->P, h->kent, h->T, h->u, h->w, h->conduct, cur_vis(h, 1), h->strain, h->Cnew,
                 h->nempty, h->rows, h->ds);
    TRY(sync_point(h, [h]() { return stats_row(h, &h->stats_row); }));
    if (!h->capturing && row) *row = h->stats_row;
    return TC_OK;
}

// the stats.dat row from the last read of the device scalars
tc_status stats_row(Handle* h, tc_stats_row* row) {
    std::memset(row, 0, sizeof(*row));
    const double asp = h->p.aspect;
    const DevScalars& s = *h->hs;
    if (h->p.comp == 1) {
        for (int t = 0; t < h->ntype; t++) row->Cavg[t] = s.integ[t] / asp;
        if (h->tstep == 0)
            for (int t = 0; t < h->ntype; t++) h->mass[t] = row->Cavg[t];
        for (int t = 0; t < h->ntype; t++) row->ent[t] = s.integ[4 + t] / asp / h->mass[t];
    }
    if (h->p.comp == 1 || h->p.tracer == 1) {
        row->empty_cells = s.empty_cells;
        row->tracer_min = s.nempty_min;
        row->tracer_max = s.nempty_max;
    }
    row->vrms = std::pow(s.integ[8] / asp, 0.5);
    row->mobility = std::pow(s.integ[11] / asp, 0.5) / row->vrms;
    row->strain_max = s.strain_max;
    if (h->p.RaT != 0.0) {
        row->Tavg = s.integ[9] / asp;
        row->RaT_avg = s.integ[10] / asp;
        row->Nu = s.integ[12] / s.integ[13];
        row->Nu_bot = s.integ[14] / asp;
        row->q1 = s.integ[15]; row->q2 = s.integ[16]; row->q3 = s.integ[17]; row->q4 = s.integ[18];
    }
    row->time = h->time;
    row->tstep = h->tstep;
    if (h->time == 0.0 && h->p.equalize == 1)
        for (int t = 0; t < h->ntype; t++) h->Cinit[t] = row->Cavg[t];
    row->n_eta = h->n_eta;
    row->n_temp = h->n_temp;
    row->eig_fine = h->eig_fine;
    for (int t = 0; t < TC_MAX_TYPES; t++) row->n_comp[t] = h->n_comp[t];
    return TC_OK;
}

// ---------------------------------------------------------------------------
// creation
// ---------------------------------------------------------------------------
tc_status create(Handle* h, const tc_params* in) {
    h->p = *in;
    tc_params& p = h->p;
    if (p.order != 2) { h->err = "the GPU path implements order=2"; return TC_ERR_UNSUPPORTED; }
    if (p.gridX < 0 || p.gridX > 2 || p.gridZ < 0 || p.gridZ > 2) { h->err = "gridX and gridZ must be 0..2"; return TC_ERR_ARG; }
    if (p.gridZ == 2 && (p.nbound < 2 || p.nz - 2 * p.nbound + 2 <= 0)) {
        h->err = "gridZ = 2 needs 2 <= nbound and nz > 2 nbound - 2";
        return TC_ERR_ARG;
    }
    if (p.ivis < -1 || p.ivis > 3) { h->err = "ivis must be -1..3"; return TC_ERR_ARG; }
    if (p.iterate_order != 1) { h->err = "iterate_order must be 1"; return TC_ERR_UNSUPPORTED; }
    if (p.RaT == 0.0) { h->err = "the GPU path implements thermal or thermochemical convection (RaT != 0)"; return TC_ERR_UNSUPPORTED; }
    if (p.torder != 2 && p.torder != 4) return TC_ERR_UNSUPPORTED;
    if (p.grids < 2 || p.grids > 6) return TC_ERR_ARG;
    if (p.comp == 1 && (p.ntype < 1 || p.ntype > TC_MAX_TYPES)) return TC_ERR_ARG;
    if (p.tracer != 0 && p.tracer != 1) return TC_ERR_ARG;
    if (p.non_Newtonian != 0 && p.non_Newtonian != 1) return TC_ERR_ARG;
    if (p.equalize != 0 && p.equalize != 1) return TC_ERR_ARG;
    if (p.equalize == 1 && p.comp == 0 && p.tracer == 0) { h->err = "equalize needs tracers"; return TC_ERR_ARG; }
    if (p.equalize_threads < 0 || p.equalize_threads > 1024) return TC_ERR_ARG;
    if (p.non_Newtonian == 1 && (p.solver_precision != 0 || p.learned_guess != 0)) {
        h->err = "the non-Newtonian iteration runs in FP64 without the learned start";
        return TC_ERR_UNSUPPORTED;
    }
    if (p.tracer == 1 && p.Tbot != 0 && p.Tbot != 1) { h->err = "temperature tracers need Tbot = 0 or 1"; return TC_ERR_ARG; }
    if (p.Nmulti < 1 || p.max_cycles < 1 || p.nx < 8 || p.nz < 8 || p.aspect <= 0.0) return TC_ERR_ARG;
    if (p.solver_precision != 0 && p.solver_precision != 1) return TC_ERR_ARG;
    if (p.learned_guess < 0 || p.learned_guess > 3 || p.learned_smooth < 0 || p.learned_smooth > 64) return TC_ERR_ARG;
    if (p.cycle_correction < 0 || p.cycle_correction > 4) return TC_ERR_ARG;
    if (p.non_Newtonian == 1 && p.cycle_correction != 0) {
        h->err = "the cycle correction runs on Newtonian solves";
        return TC_ERR_UNSUPPORTED;
    }
    h->nx = p.nx; h->nz = p.nz; h->grids = p.grids;
    {
        const long nb = (long)((p.nx + 2 + BX - 1) / BX) * (long)((p.nz + 2 + BY - 1) / BY);
        if (nb > TC_MAX_RED_BLOCKS) { h->err = "grid too large for the reduction scratch"; return TC_ERR_UNSUPPORTED; }
    }
    h->ntype = (p.comp == 1) ? p.ntype : 0;
    // compute_smoothing_parameters (multigrid_cycle.f90:131-173)
    if (p.ivis == 0 || p.RaT == 0.0) h->delta_T = 2.0;
    else h->delta_T = (p.visT != 1.0) ? std::log(p.delta_visT) / std::log(p.visT) : 2.0;
    if (p.vis_iter < 1) { h->err = "vis_iter must be >= 1"; return TC_ERR_ARG; }
    for (int t = 0; t < TC_MAX_TYPES; t++) h->delta_C[t] = 2.0;
    if (p.comp == 1) {
        for (int t = 0; t < p.ntype; t++)
            if (p.conduct_factor[t] != 1.0)
                h->delta_C[t] = std::fabs(std::log(p.delta_visC[t]) / std::log(1.0 / p.conduct_factor[t]));
        if (p.ivis == 2)
            for (int t = 0; t < p.ntype; t++)
                if (p.visC[t] != 1.0) h->delta_C[t] = std::fabs(std::log(p.delta_visC[t]) / std::log(p.visC[t]));
    }
    // multigrid_setup
    tcs::optimize_grid(h->nx, h->nz, h->grids, p.mingrid);
    std::vector<int> tab = tcs::cycle_table(h->grids);
    if (tab.empty()) return TC_ERR_ARG;
    h->nsteps = (int)tab.size();
    h->multi.assign(h->nsteps + 2, 0);
    for (int i = 0; i < h->nsteps; i++) h->multi[i + 1] = tab[i];
    h->multi[0] = h->multi[h->nsteps];
    h->multi[h->nsteps + 1] = h->multi[1];
    const int nx = h->nx, nz = h->nz, G = h->grids;
    for (int l = 1; l <= G; l++)
        if ((nx >> (l - 1)) < 4 || (nz >> (l - 1)) < 4) { h->err = "grid too coarse for the level count"; return TC_ERR_ARG; }
    // compute_basics
    tcs::LevSpacing s1;
    tcs::level_spacing(p.aspect, nx, nz, s1);
    h->grid_dr = s1.dr; h->grid_ds = s1.ds;
    h->ntr = (p.comp == 1 || p.tracer == 1) ? (int64_t)(nx + 1) * (nz + 1) * p.tpc : 0;
    const int nxc = nx >> (G - 1), nzc = nz >> (G - 1);
    h->ngrid_coarse = (nxc + 1) * (nzc + 1);
    tcs::coarse_bandwidth(nxc, nzc, 2, 1, h->kl, h->ku);
    // FD coefficients and eigenvalue bases
    tcs::FD fd;
    tcs::fd_coefficients(2, fd);
    tcs::derivative_eigenvalues(fd, 1, h->eb);
    // build_grid (grid.f90): coordinates and metrics
    tcs::GridMetrics gm;
    tcs::grid_metrics(p.aspect, nx, nz, p.gridX, p.gridZ, p.spaceX, p.spaceZ, p.thickness, p.nbound, fd, gm);
    const bool stretched = (p.gridX != 0 || p.gridZ != 0);
    h->xg_h = gm.xg;
    h->zg_h = gm.zg;
    // entrainment_setup (composition.f90:582-591)
    h->kent = 0;
    for (int k = 0; k <= nz; k++)
        if (gm.zg[(size_t)(k + gm.pad)] <= p.dent) h->kent = k;
    // ---- physics scalars ----
    Phys& P = h->P;
    P.nx = nx; P.nz = nz; P.ntype = h->ntype; P.comp = p.comp; P.ivis = p.ivis; P.Tbot = p.Tbot; P.Vbc = p.Vbc;
    P.torder = p.torder; P.tracer = p.tracer; P.aspect = p.aspect; P.dr = s1.dr; P.ds = s1.ds; P.dr2 = s1.dr2; P.ds2 = s1.ds2;
    P.dro2 = 0.5 * s1.dr; P.dso2 = 0.5 * s1.ds; P.RaT = p.RaT;
    P.rdr = 1.0 / s1.dr; P.rds = 1.0 / s1.ds;
    P.lnvisT = std::log(p.visT); P.lnvisP = std::log(p.visP); P.visT2 = p.visT * p.visT; P.H = p.H;
    P.visT = p.visT; P.yield = p.yield; P.yield_gradient = p.yield_gradient; P.yield_depth = p.yield_depth;
    for (int t = 0; t < TC_MAX_TYPES; t++) {
        P.RaC[t] = p.RaC[t]; P.lnvisC[t] = (p.visC[t] > 0.0) ? std::log(p.visC[t]) : 0.0; P.Htype[t] = p.Htype[t];
        P.lncf[t] = (p.conduct_factor[t] > 0.0) ? std::log(1.0 / p.conduct_factor[t]) : 0.0;
    }
    P.courantT = p.courantT; P.courantC = p.courantC;
    P.Tr_max = h->eb.Tr / s1.dr; P.Ts_max = h->eb.Tr / s1.ds;
    P.Trr_max = -h->eb.Trr / s1.dr2; P.Tss_max = -h->eb.Trr / s1.ds2;
    P.M = Metric{};
    P.M.on = stretched ? 1 : 0;
    P.M.gx = (p.gridX != 0) ? 1 : 0;
    P.M.gz = (p.gridZ != 0) ? 1 : 0;
    // ---- stream ----
    cudaGetDevice(&h->device);
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return TC_ERR_CUDA; }
    h->own_stream = true;
    h->graphs = new CycleGraphs();
    h->no_graphs = (std::getenv("TC_NO_GRAPHS") != nullptr);
    h->no_device_loop = (std::getenv("TC_HOST_LOOP") != nullptr);
    h->fuse_visits = (std::getenv("TC_NO_FUSED_VISITS") == nullptr) && visit_cluster_setup() > 0;
    // ---- allocations ----
    h->L1 = make_lay(nx, nz);
    const size_t pl = h->L1.plane;
    double** fine[] = {&h->T, &h->T0, &h->T1, &h->T2, &h->SF, &h->Tvis, &h->Tvis2, &h->Tbuoy, &h->u, &h->w,
                       &h->du, &h->dw, &h->conduct, &h->conduct_r, &h->conduct_s, &h->dts, &h->strain};
    for (double** q : fine) TRY(dalloc_t(h, q, pl));
    for (int t = 0; t < h->ntype; t++) {
        TRY(dalloc_t(h, &h->Cnew[t], pl)); TRY(dalloc_t(h, &h->C0[t], pl)); TRY(dalloc_t(h, &h->Cvis[t], pl));
        TRY(dalloc_t(h, &h->Cvis2[t], pl)); TRY(dalloc_t(h, &h->Cbuoy[t], pl));
    }
    TRY(dalloc_t(h, &h->counts, pl * (size_t)(h->ntype + 1)));
    TRY(dalloc_t(h, &h->nempty, pl));
    TRY(dalloc_t(h, &h->zg, (size_t)nz + 1 + 2 * (SP + 1)));
    if (h->ntr > 0) {
        double** tr[] = {&h->rtr, &h->str, &h->rtr0, &h->str0, &h->rtr1, &h->str1, &h->rtr2, &h->str2};
        for (double** q : tr) TRY(dalloc_t(h, q, (size_t)h->ntr));
        TRY(dalloc_t(h, &h->ttype, (size_t)h->ntr));
        TRY(dalloc_t(h, &h->perm, (size_t)h->ntr));
        launch_iota(h->st, h->ntr, h->perm);  // a valid permutation before any upload
        for (int q = 0; q < 2; q++) TRY(dalloc_t(h, &h->itmp[q], (size_t)h->ntr));
        TRY(dalloc_t(h, &h->sort_cnt, pl));
        TRY(dalloc_t(h, &h->sort_off, pl));
        TRY(dalloc_t(h, &h->sort_bsum, (pl + 1023) / 1024));
    }
    if (p.equalize == 1 && h->ntr > 0) {
        const int NR = (p.equalize_threads > 0) ? p.equalize_threads : 1;
        const size_t nc = (size_t)(nx + 1) * (nz + 1);
        h->eq_NR = NR;
        TRY(dalloc_t(h, &h->eq_iperm, (size_t)h->ntr));
        TRY(dalloc_t(h, &h->eq_ids, (size_t)h->ntr));
        TRY(dalloc_t(h, &h->eq_nex, nc));
        TRY(dalloc_t(h, &h->eq_off, nc + 1));
        TRY(dalloc_t(h, &h->eq_cur, nc));
        TRY(dalloc_t(h, &h->eq_cnt, nc));
        TRY(dalloc_t(h, &h->eq_seeds, (size_t)4 * NR));
        TRY(dalloc_t(h, &h->eq_isv, (size_t)NR * (h->ntype + 1)));
        TRY(dalloc_t(h, &h->eq_isv2, (size_t)NR * (h->ntype + 1)));
        TRY(dalloc_t(h, &h->eq_nfr, (size_t)NR * (h->ntype + 1)));
        TRY(dalloc_t(h, &h->eq_nxl, (size_t)nx + 1));
        TRY(dalloc_t(h, &h->eq_nzl, (size_t)nz + 1));
        TRY(dalloc_t(h, &h->eq_sc, (size_t)64));
        if (p.tracer == 1) { TRY(dalloc_t(h, &h->eq_Td, pl)); TRY(dalloc_t(h, &h->eq_dTd, pl)); }
        // mzran seeds of each OpenMP thread (basics.f90:198-212), laid out [4][NR]
        std::vector<int32_t> sd((size_t)4 * NR);
        sd[0] = 521288629; sd[NR] = 362436069; sd[2 * NR] = 16163801; sd[3 * NR] = 1131199299;
        for (int j = 1; j < NR; j++) {
            int32_t r = sd[j - 1] - sd[2 * NR + j - 1];
            if (r < 0) r += 2147483579;
            sd[j] = sd[NR + j - 1];
            sd[NR + j] = sd[2 * NR + j - 1];
            sd[2 * NR + j] = r;
            sd[3 * NR + j] = (int32_t)(69069u * (uint32_t)sd[3 * NR + j - 1] + 1013904243u);
        }
        CK(cudaMemcpy(h->eq_seeds, sd.data(), sizeof(int32_t) * sd.size(), cudaMemcpyHostToDevice));
    }
    if (p.tracer == 1 && h->ntr > 0) {
        double** tq[] = {&h->Ttr, &h->Ttr0, &h->Ttr1, &h->Ttr2};
        for (double** q : tq) TRY(dalloc_t(h, q, (size_t)h->ntr));
        double** tf[] = {&h->Tratio, &h->tsa, &h->dT};
        for (double** q : tf) TRY(dalloc_t(h, q, pl));
        TRY(dalloc_t(h, &h->tsum, 2 * pl));
    }
    const int ldab = 2 * h->kl + h->ku + 1;
    TRY(dalloc_t(h, &h->band, (size_t)ldab * h->ngrid_coarse));
    TRY(dalloc_t(h, &h->rowb, (size_t)h->ngrid_coarse));
    h->coarse_banded = h->ngrid_coarse > kCoarseInverseMax;
    if (!h->coarse_banded) {
        TRY(dalloc_t(h, &h->ainv, (size_t)h->ngrid_coarse * h->ngrid_coarse));
        TRY(dalloc_t(h, &h->bvec, (size_t)(h->ngrid_coarse + 8) * h->ngrid_coarse));
        // interior unknowns p = i*(nzc+1) + k in increasing order, with their offsets
        const Lay Lc = make_lay(nx >> (G - 1), nz >> (G - 1));
        std::vector<int> cq, cx;
        for (int i = 1; i <= Lc.a - 1; i++)
            for (int k = 1; k <= Lc.b - 1; k++) {
                cq.push_back(i * (Lc.b + 1) + k);
                cx.push_back((int)IX(Lc, i, k));
            }
        h->coarse_m = (int)cq.size();
        TRY(dalloc_t(h, &h->coarse_q, cq.size()));
        TRY(dalloc_t(h, &h->coarse_x, cx.size()));
        CK(cudaMemcpy(h->coarse_q, cq.data(), sizeof(int) * cq.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->coarse_x, cx.data(), sizeof(int) * cx.size(), cudaMemcpyHostToDevice));
    }
    TRY(dalloc_t(h, &h->ipiv, (size_t)h->ngrid_coarse));
    if (h->fuse_visits) TRY(dalloc_t(h, &h->ctab, (size_t)128 * 4096));
    TRY(dalloc_t(h, &h->rows, (size_t)8 * (nz + 1)));
    TRY(dalloc_t(h, &h->rs.part, (size_t)4 * TC_MAX_RED_BLOCKS));
    TRY(dalloc_t(h, &h->rs.count, (size_t)8));
    TRY(dalloc_t(h, &h->ds, (size_t)1));
    e = cudaMallocHost((void**)&h->hs, sizeof(DevScalars));
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return TC_ERR_ALLOC; }
    std::memset(h->hs, 0, sizeof(DevScalars));
    if (stretched) {
        // the metric arrays, each over fine index -pad..n+pad
        const std::vector<double>* xs[7] = {&gm.xr, &gm.xrr, &gm.xrrr, &gm.xrrrr, &gm.xr3, &gm.xr4, &gm.dxr};
        const std::vector<double>* zs_[7] = {&gm.zs, &gm.zss, &gm.zsss, &gm.zssss, &gm.zs3, &gm.zs4, &gm.dzs};
        const double** xd[7] = {&P.M.xr, &P.M.xrr, &P.M.xrrr, &P.M.xrrrr, &P.M.xr3, &P.M.xr4, &P.M.dxr};
        const double** zd[7] = {&P.M.zs, &P.M.zss, &P.M.zsss, &P.M.zssss, &P.M.zs3, &P.M.zs4, &P.M.dzs};
        for (int q = 0; q < 7; q++) {
            double* dx = nullptr;
            double* dz = nullptr;
            TRY(dalloc_t(h, &dx, xs[q]->size()));
            TRY(dalloc_t(h, &dz, zs_[q]->size()));
            CK(cudaMemcpy(dx, xs[q]->data(), sizeof(double) * xs[q]->size(), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(dz, zs_[q]->data(), sizeof(double) * zs_[q]->size(), cudaMemcpyHostToDevice));
            *xd[q] = dx;
            *zd[q] = dz;
        }
    }
    // ---- levels ----
    const int odi[TC_NCOEF] = TC_OFFSETS_DI, odk[TC_NCOEF] = TC_OFFSETS_DK;
    auto Dv = [&](const double* D, int j) { return (j < -3 || j > 3) ? 0.0 : D[j + 3]; };
    int n_sms = 0;
    CK(cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, h->device));
    for (int l = 1; l <= G; l++) {
        Level& lv = h->lev[l];
        lv.L = make_lay(nx >> (l - 1), nz >> (l - 1));
        const size_t lp = lv.L.plane;
        for (int q = 0; q < 2; q++) { TRY(dalloc_t(h, &lv.err[q], lp)); TRY(dalloc_t(h, &lv.vis[q], lp)); }
        lv.ecur = 0; lv.vcur = 0;
        double** lf[] = {&lv.vx, &lv.vz, &lv.vxx, &lv.vzz, &lv.vxz, &lv.dt_vis, &lv.dt_stream, &lv.ratio, &lv.rhs,
                         &lv.res, &lv.cA, &lv.cB};
        for (double** q : lf) TRY(dalloc_t(h, q, lp));
        for (int q = 0; q < 6; q++) TRY(dalloc_t(h, &lv.bak[q], lp));
        TRY(dalloc_t(h, &lv.coef, lp * TC_NCOEF));
        lv.sweep_bx = BX;
        lv.sweep_by = BY;
        lv.fuse = 1;
        lv.visit_cfg = 0;
        lv.blk = 0;
        // mixed solve, a level below the first that no cluster visit covers:
        // six sweeps per launch of the tiled smoother when its tiles fit one
        // wave (measured faster than one launch per sweep at 512x128; slower
        // at 1024x256, and in FP64, where the redundant halo work costs FP64
        // issue slots)
        if (p.solver_precision == 1 && l > 1 && !(h->fuse_visits && visit_cluster_fits(lv.L, p.Nmulti, 1)) &&
            sweep_blk_tiles(lv.L) <= n_sms)
            lv.blk = 6;
        lv.coef32 = lv.dts32 = lv.cA32 = lv.cB32 = lv.rhs32 = lv.res32 = nullptr;
        lv.e32[0] = lv.e32[1] = nullptr;
        lv.e32cur = 0;
        lv.g32 = nullptr;
        if (p.solver_precision == 1) {
            TRY(dalloc_t(h, &lv.coef32, lp * TC_NCOEF));
            float** f32[] = {&lv.dts32, &lv.cA32, &lv.cB32, &lv.rhs32, &lv.res32, &lv.e32[0], &lv.e32[1]};
            for (float** q : f32) TRY(dalloc_t(h, q, lp));
        }
        tcs::LevSpacing s;
        tcs::level_spacing(p.aspect, lv.L.a, lv.L.b, s);
        LevConst& c = lv.c;
        c.dr = s.dr; c.ds = s.ds; c.dr2 = s.dr2; c.ds2 = s.ds2; c.dr3 = s.dr3; c.ds3 = s.ds3; c.dr4 = s.dr4;
        c.ds4 = s.ds4; c.drds = s.drds; c.drds2 = s.drds2; c.dr2ds = s.dr2ds; c.dr2ds2 = s.dr2ds2;
        {
            auto pow2 = [](double v) { int e; return v > 0.0 && std::frexp(v, &e) == 0.5; };
            c.recip = (pow2(c.dr) && pow2(c.ds) && pow2(c.dr2) && pow2(c.ds2) && pow2(c.drds)) ? 1 : 0;
            c.rdr = 1.0 / c.dr; c.rds = 1.0 / c.ds; c.rdr2 = 1.0 / c.dr2; c.rds2 = 1.0 / c.ds2; c.rdrds = 1.0 / c.drds;
        }
        // scaled bounds (test_eigenvalues / iterate_local_time_steps preamble)
        const double Ts = h->eb.Tr / s.ds, Tss = -h->eb.Trr / s.ds2, Tsss = h->eb.Trrr / s.ds3,
                     Tssss = h->eb.Trrrr / s.ds4, Trr = -h->eb.Trr / s.dr2, Trrr = h->eb.Trrr / s.dr3,
                     Trrrr = h->eb.Trrrr / s.dr4, Trs = -h->eb.Trs / s.drds, Trrss = h->eb.Trrss / s.dr2ds2,
                     Trss = h->eb.Trrs / s.drds2, Trrs = h->eb.Trrs / s.dr2ds;
        (void)Ts;
        c.eK1 = Trr - Tss; c.eK2 = Trrrr + Tssss; c.eTrrss = Trrss; c.eTrs = Trs;
        c.eK5 = Trrr + Trss; c.eK6 = Tsss + Trrs;
        c.M = P.M;
        c.mf = 1 << (l - 1);
        c.e = EigScaled{h->eb.Tr / s.dr, Ts, Trr, Tss, Trrr, Tsss, Trrrr, Tssss, Trs, Trrs, Trss, Trrss};
        for (int d = 0; d < TC_NCOEF; d++) {
            const int di = odi[d], dk = odk[d];
            double Srr = 0, Sss = 0, Srrr = 0, Ssss = 0, Srrrr = 0, Sssss = 0;
            if (dk == 0) { Srr = Dv(fd.D2, di) / s.dr2; Srrr = Dv(fd.D3, di) / s.dr3; Srrrr = Dv(fd.D4, di) / s.dr4; }
            if (di == 0) { Sss = Dv(fd.D2, dk) / s.ds2; Ssss = Dv(fd.D3, dk) / s.ds3; Sssss = Dv(fd.D4, dk) / s.ds4; }
            const bool in1 = (di >= -1 && di <= 1 && dk >= -1 && dk <= 1);
            const double Srs = in1 ? (Dv(fd.D1, dk) * Dv(fd.D1, di)) / s.drds : 0.0;
            const double Srss = in1 ? (Dv(fd.D2, dk) * Dv(fd.D1, di)) / s.drds2 : 0.0;
            const double Srrs = in1 ? (Dv(fd.D1, dk) * Dv(fd.D2, di)) / s.dr2ds : 0.0;
            const double Srrss = in1 ? (Dv(fd.D2, dk) * Dv(fd.D2, di)) / s.dr2ds2 : 0.0;
            c.fold[d][0] = Srr - Sss;
            c.fold[d][1] = Srrrr + Sssss;
            c.fold[d][2] = Srrss;
            c.fold[d][3] = Srs;
            c.fold[d][4] = Srrr + Srss;
            c.fold[d][5] = Ssss + Srrs;
            // the same single-tap derivatives unreduced (stream_space, build = 1)
            const double Sr = (dk == 0) ? Dv(fd.D1, di) / s.dr : 0.0;
            const double Ss = (di == 0) ? Dv(fd.D1, dk) / s.ds : 0.0;
            const double q[12] = {Sr, Srr, Srrr, Srrrr, Ss, Sss, Ssss, Sssss, Srs, Srrs, Srss, Srrss};
            for (int j = 0; j < 12; j++) lv.mfold.w[d][j] = q[j];
        }
        // level 1 of the mixed solve sweeps from the five viscosity fields
        // (k_sweep_g32) when the stencil's structural zeros hold
        lv.use_g32 = 0;
        if (p.solver_precision == 1 && l == 1 && !stretched && fold_g32_weights(c, &lv.gw)) {
            TRY(dalloc_t(h, &lv.g32, lp * 5));
            lv.use_g32 = 1;
        }
        // stability_vis_smoother (smoother.f90:465-508); uniform: eI = 0
        {
            const double Trr_l = -h->eb.Trr / s.dr2, Tss_l = -h->eb.Trr / s.ds2;
            const double Tr_l = h->eb.Tr / s.dr, Ts_l = h->eb.Tr / s.ds;
            std::vector<double> hv(lp, 0.0);
            for (int i = 0; i <= lv.L.a; i++)
                for (int k = 1; k <= lv.L.b - 1; k++) {
                    const int i1 = i * c.mf + gm.pad, k1 = k * c.mf + gm.pad;
                    const double x1 = gm.xr[(size_t)i1], x2 = gm.xrr[(size_t)i1];
                    const double z1 = gm.zs[(size_t)k1], z2 = gm.zss[(size_t)k1];
                    const double eR = std::fabs(Trr_l / (x1 * x1)) + std::fabs(Tss_l / (z1 * z1));
                    const double eI = std::fabs(x2 / gm.xr3[(size_t)i1]) * Tr_l + std::fabs(z2 / gm.zs3[(size_t)k1]) * Ts_l;
                    hv[IX(lv.L, i, k)] = 2.0 * eR / (eR * eR + eI * eI);
                }
            CK(cudaMemcpy(lv.dt_vis, hv.data(), lp * sizeof(double), cudaMemcpyHostToDevice));
        }
    }
    // the bottom of the W-cycle as precomputed matrices
    if (p.mg_coarse_matrix == 1 && p.mg_zero_coarse == 1 && p.non_Newtonian == 0 && G >= 3 && !h->coarse_banded &&
        p.Nmulti <= 128 &&
        subcycle_fits(h->lev[G - 1].L, h->lev[G].L)) {
        const int S = G - 1;
        h->sub_k.assign(h->nsteps + 2, 0);
        h->sub_end.assign(h->nsteps + 2, 0);
        bool need[5] = {false, false, false, false, false};
        bool ok = true;
        for (int pp = 2; pp <= h->nsteps && ok; pp++) {
            if (h->multi[pp] != S || h->multi[pp - 1] != S - 1) continue;
            int k = 0, q = pp;
            while (q + 1 <= h->nsteps + 1 && h->multi[q + 1] >= S) {
                q++;
                if (h->multi[q] == G) k++;
            }
            // the pattern must be S (G S)^k and end before the cycle does
            for (int t = pp; t <= q; t++)
                if (h->multi[t] != ((t - pp) % 2 == 0 ? S : G)) ok = false;
            if (q > h->nsteps || h->multi[q] != S || k < 1 || k > 4) ok = false;
            if (!ok) break;
            h->sub_k[pp] = k;
            h->sub_end[pp] = q;
            need[k] = true;
            h->sub_kmax = std::max(h->sub_kmax, k);
        }
        if (ok && h->sub_kmax > 0) {
            const size_t nS = (size_t)(h->lev[S].L.a - 1) * (h->lev[S].L.b - 1);
            for (int k = 1; k <= 4; k++)
                if (need[k]) TRY(dalloc_t(h, &h->subM[k - 1], nS * nS));
            TRY(dalloc_t(h, &h->sub_tab, 4 * (size_t)p.Nmulti));
            TRY(dalloc_t(h, &h->sub_ctab, (size_t)p.Nmulti * nS));
            h->sub_m32 = (p.solver_precision == 1);
            if (h->sub_m32) TRY(dalloc_t(h, &h->sub_ac, (size_t)h->coarse_m * h->coarse_m));
            h->sub_on = true;
        }
    }
    // corrections after the level-1 visit: psi at the previous one, the network's direction
    if (p.cycle_correction != 0 || p.learned_guess == 3) {
        if (p.cycle_correction != 0) TRY(dalloc_t(h, &h->acc_prev, pl));
        if (p.cycle_correction >= 3) {
            TRY(dalloc_t(h, &h->win_p, pl * TC_WIN));
            TRY(dalloc_t(h, &h->win_ap, pl * TC_WIN));
            TRY(dalloc_t(h, &h->win_rn, pl));
            TRY(dalloc_t(h, &h->win_rp, pl));
            TRY(dalloc_t(h, &h->win_adnn, pl));
        }
        TRY(dalloc_t(h, &h->acc_dnn, pl));
    }
    // Chebyshev factors of the filter loops (smoother.f90: the same
    // expressions the host loops evaluate), for the device-side loops
    {
        auto cheb = [](int Niter, int n, double lb, double la) {
            const int ntemp = Niter - n + 1;
            return 2.0 / (-lb - la + (lb - la) * std::cos((double)(2 * ntemp - 1) * kPi / (double)(2 * Niter)));
        };
        std::vector<double> tb((size_t)kTabVis0 + p.vis_iter + 11);
        for (int n = 1; n <= 6; n++) {
            tb[kTabVisA1 + n - 1] = cheb(6, n, -5.0, -2.0);
            tb[kTabVisB + n - 1] = cheb(6, n, -2.0, -1.0);
        }
        for (int n = 1; n <= p.vis_iter; n++) tb[kTabVis0 + n - 1] = cheb(p.vis_iter, n, -2.0, -1.0);
        for (int n = 1; n <= 10; n++) tb[tab_c10(h) + n - 1] = cheb(10, n, -5.0, -1.0);
        tb[tab_c1(h)] = cheb(1, 1, -5.0, -1.0);
        TRY(dalloc_t(h, &h->flt_tab, tb.size()));
        CK(cudaMemcpy(h->flt_tab, tb.data(), sizeof(double) * tb.size(), cudaMemcpyHostToDevice));
    }
    // stability_RK4_smoother: dts_array (smoother.f90:423-462)
    {
        const double Tr_max = h->eb.Tr / s1.dr, Ts_max = h->eb.Tr / s1.ds;
        const double Trr_max = -h->eb.Trr / s1.dr2, Tss_max = -h->eb.Trr / s1.ds2;
        std::vector<double> hv(pl, 0.0);
        for (int i = 0; i <= nx; i++)
            for (int k = 0; k <= nz; k++) {
                const size_t i1 = (size_t)(i + gm.pad), k1 = (size_t)(k + gm.pad);
                const double x1 = gm.xr[i1], z1 = gm.zs[k1];
                const double eR = std::fabs(Trr_max / (x1 * x1)) + std::fabs(Tss_max / (z1 * z1));
                const double eI = std::fabs(gm.xrr[i1] / gm.xr3[i1]) * Tr_max + std::fabs(gm.zss[k1] / gm.zs3[k1]) * Ts_max;
                hv[IX(h->L1, i, k)] = 2.0 * eR / (eR * eR + eI * eI);
            }
        CK(cudaMemcpy(h->dts, hv.data(), pl * sizeof(double), cudaMemcpyHostToDevice));
    }
    // zg (grid.f90:46-109, restart=0 coordinates)
    {
        static_assert(SP + 1 == 3, "zg is indexed k + 3");
        CK(cudaMemcpy(h->zg, gm.zg.data(), gm.zg.size() * sizeof(double), cudaMemcpyHostToDevice));
        h->zg += gm.pad;  // kernels index zg[k], k >= -3
    }
    CK(cudaDeviceSynchronize());
    return TC_OK;
}

// Fortran-layout (nx+5)x(nz+5) host array <-> padded device plane
tc_status put_field(Handle* h, double* dev, const double* host) {
    const size_t ni = (size_t)h->nx + 1 + 2 * SP, nk = (size_t)h->nz + 1 + 2 * SP;
    CK(cudaMemcpy2DAsync(dev, h->L1.ld * sizeof(double), host, ni * sizeof(double), ni * sizeof(double), nk,
                         cudaMemcpyHostToDevice, h->st));
    return TC_OK;
}
tc_status get_field(Handle* h, double* host, const double* dev) {
    const size_t ni = (size_t)h->nx + 1 + 2 * SP, nk = (size_t)h->nz + 1 + 2 * SP;
    CK(cudaMemcpy2DAsync(host, ni * sizeof(double), dev, h->L1.ld * sizeof(double), ni * sizeof(double), nk,
                         cudaMemcpyDeviceToHost, h->st));
    return TC_OK;
}

tc_status upload(Handle* h, const double* T, const double* Cn, const double* SF, const double* r, const double* s,
                 const int32_t* tt, int64_t n, const double* Ttr = nullptr) {
    if (!T || !SF) return TC_ERR_ARG;
    if (h->p.comp == 1 && (n != h->ntr || !r || !s || !tt)) return TC_ERR_ARG;
    if (h->p.tracer == 1 && (n != h->ntr || !r || !s || !Ttr)) {
        h->err = "temperature tracers need rtr, str and Ttr (tc_upload_state_ex)";
        return TC_ERR_ARG;
    }
    TRY(put_field(h, h->T, T));
    TRY(put_field(h, h->SF, SF));
    const size_t ni = (size_t)h->nx + 1 + 2 * SP, nk = (size_t)h->nz + 1 + 2 * SP;
    std::vector<double> tmp;
    for (int t = 0; t < h->ntype; t++) {
        if (Cn) {
            tmp.resize(ni * nk);
            for (size_t x = 0; x < ni * nk; x++) tmp[x] = Cn[x * h->ntype + t];
            TRY(put_field(h, h->Cnew[t], tmp.data()));
            CK(cudaStreamSynchronize(h->st));
        } else {
            CK(cudaMemsetAsync(h->Cnew[t], 0, sizeof(double) * h->L1.plane, h->st));
        }
    }
    if (h->p.comp == 1 || h->p.tracer == 1) {
        CK(cudaMemcpyAsync(h->rtr, r, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
        CK(cudaMemcpyAsync(h->str, s, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
        if (h->p.comp == 1) CK(cudaMemcpyAsync(h->ttype, tt, sizeof(int32_t) * h->ntr, cudaMemcpyHostToDevice, h->st));
        else CK(cudaMemsetAsync(h->ttype, 0, sizeof(int32_t) * h->ntr, h->st));  // all ambient
        if (h->p.tracer == 1)
            CK(cudaMemcpyAsync(h->Ttr, Ttr, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
        launch_iota(h->st, h->ntr, h->perm);
    }
    CK(cudaMemsetAsync(h->ds, 0, sizeof(DevScalars), h->st));
    launch_enforce_T(h->st, h->L1, h->T, h->p.Tbot);
    launch_stream_bcs(h->st, h->lev[1], h->SF, h->p.Vbc);
    for (int t = 0; t < h->ntype; t++) launch_enforce_comp(h->st, h->L1, h->Cnew[t], h->Cnew[t]);
    for (int l = 2; l <= h->grids; l++)
        for (int q = 0; q < 2; q++) CK(cudaMemsetAsync(h->lev[l].err[q], 0, sizeof(double) * h->lev[l].L.plane, h->st));
    h->uploaded = true;
    if (h->p.comp == 1 || h->p.tracer == 1)
        TRY(tracers_to_corners(h, h->rtr, h->str, false, h->p.tracer == 1 ? h->Ttr : nullptr, h->T));
    TRY(smoother_time_T(h, h->T));
    if (h->p.comp != 0) TRY(smoother_time(h));
    load_conductivity_array(h);
    TRY(check_flags(h));
    return TC_OK;
}

// ---------------------------------------------------------------------------
// the whole timestep as one graph launch
// ---------------------------------------------------------------------------
void drop_step_graphs(Handle* h) {
    for (auto& kv : h->step_graphs) {
        if (kv.second && kv.second->ge) cudaGraphExecDestroy(kv.second->ge);
        delete kv.second;
    }
    h->step_graphs.clear();
    h->epoch++;
}

// The step can run as one captured graph: every loop of it on the device,
// no host branch on a device value, and everything the first step builds
// (cycle and filter graphs, coarse factors, sub-cycle tables) in place.
// `own`: the handle's own step graph (tc_set_step_graph) rather than an
// ensemble's.
bool step_graph_ready(const Handle* h, bool own) {
    if ((own && !h->step_graph) || h->step_graph_failed || !h->uploaded || h->st == nullptr) return false;
    if (h->no_graphs || h->no_device_loop || h->flt_failed || !h->flt_dev_state || h->wait_test) return false;
    if (h->p.non_Newtonian == 1 || h->p.equalize == 1) return false;
    if (h->p.learned_guess == 1 || h->p.learned_guess == 2) return false;
    if (h->rec_raw && h->rec_count < h->rec_cap) return false;
    if (h->tstep < 1 || h->time == 0.0 || !h->lu_valid || (h->sub_on && !h->sub_valid)) return false;
    return h->graphs != nullptr && h->graphs->loop != nullptr;
}

// what a captured step needs before its capture begins (allocations are
// not allowed inside one)
tc_status step_graph_prepare(Handle* h) {
    if (!h->hsnap) CK(cudaMallocHost((void**)&h->hsnap, sizeof(DevScalars) * kMaxSnap));
    if (!h->body_st) CK(cudaStreamCreateWithFlags(&h->body_st, cudaStreamNonBlocking));
    return TC_OK;
}

// One step (multigrid, velocities, stats, energy_time; the order of tc_step)
// enqueued on h->st, which is capturing; the host work that follows each
// launch goes to sg->post, the kernels outside the WHILE bodies to
// sg->n_static.
tc_status capture_step(Handle* h, StepGraph* sg) {
    const long long before = t_launches;
    h->deferred.clear();
    h->nsnap = 0;
    h->enq_err = cudaSuccess;
    h->capturing = true;
    tc_status s = multigrid(h);
    if (s == TC_OK) {
        compute_velocities(h);
        s = stats(h, nullptr);
    }
    if (s == TC_OK) s = energy_time(h);
    h->capturing = false;
    sg->n_static = t_launches - before;
    g_launches.fetch_sub(sg->n_static);
    t_launches = before;
    sg->post = std::move(h->deferred);
    h->deferred.clear();
    if (s == TC_OK && h->enq_err != cudaSuccess) s = TC_ERR_CUDA;
    h->enq_err = cudaSuccess;
    return s;
}

tc_status build_step_graph(Handle* h, StepGraph** out) {
    TRY(step_graph_prepare(h));
    StepGraph* sg = new StepGraph();
    if (cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        delete sg;
        cudaGetLastError();
        return TC_ERR_CUDA;
    }
    tc_status s = capture_step(h, sg);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (s == TC_OK && (e != cudaSuccess || g == nullptr)) s = TC_ERR_CUDA;
    if (s == TC_OK && cudaGraphInstantiate(&sg->ge, g, 0) != cudaSuccess) s = TC_ERR_CUDA;
    if (g) cudaGraphDestroy(g);
    if (s != TC_OK) {
        delete sg;
        cudaGetLastError();
        return s;
    }
    *out = sg;
    return TC_OK;
}

// The host's part of a step after its graph ran: the deferred reads in the
// eager step's order (the first error stops them, as it stops that step),
// then the outputs and the clock.
tc_status finish_step(Handle* h, const StepGraph& sg, tc_stats_row* row, int32_t* cycles, double* dt_out) {
    tc_status s = TC_OK;
    for (const auto& f : sg.post) {
        s = f();
        if (s != TC_OK) break;
    }
    h->graph_steps++;
    if (cycles) *cycles = (s == TC_OK || h->cycles_acc > 0) ? h->cycles_acc : h->last_cycles;
    if (s != TC_OK) return s;
    if (row) *row = h->stats_row;
    if (dt_out) *dt_out = h->dt;
    h->time = h->time + h->dt;
    h->tstep += 1;
    return TC_OK;
}

// tc_step as one graph launch: the step's graph for this sort flag (captured
// on first use), one synchronisation, then the deferred host work.  False in
// *ran when the step must run eagerly (a capture the CUDA runtime refused).
tc_status step_as_graph(Handle* h, tc_stats_row* row, int32_t* cycles, double* dt_out, bool* ran) {
    *ran = false;
    const int key = sorts_this_step(h) ? 1 : 0;
    StepGraph* sg = nullptr;
    auto it = h->step_graphs.find(key);
    if (it != h->step_graphs.end()) {
        sg = it->second;
    } else if (build_step_graph(h, &sg) == TC_OK) {
        h->step_graphs[key] = sg;
    } else {
        h->step_graph_failed = true;
        return TC_OK;
    }
    *ran = true;
    h->cycles_acc = 0;
    CK(cudaGraphLaunch(sg->ge, h->st));
    tc_note_launch(sg->n_static);
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    return finish_step(h, *sg, row, cycles, dt_out);
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
struct tc_handle {
    Handle h;
};

namespace {
// time one replay of the launches `fn` enqueues, captured as a CUDA graph (ms)
template <class F>
tc_status graph_time(Handle* h, F&& fn, double* ms_out) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    const long long before = t_launches;
    h->enq_err = cudaSuccess;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    fn();
    CK(cudaStreamEndCapture(h->st, &g));
    g_launches.fetch_sub(t_launches - before);
    t_launches = before;
    if (h->enq_err != cudaSuccess) {
        cudaGraphDestroy(g);
        CK(h->enq_err);
    }
    cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaGraphLaunch(ge, h->st));
    CK(cudaEventRecord(e0, h->st));
    CK(cudaGraphLaunch(ge, h->st));
    CK(cudaEventRecord(e1, h->st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    *ms_out = ms;
    return TC_OK;
}
}  // namespace

// An ensemble whose timestep is one graph launch: the cases' captured steps
// as independent branches of one graph (fork from a root stream onto every
// case's stream, join back), cached by the case list (each handle's address
// and process-unique id), each case's configuration epoch and sort flag.
struct tc_ensemble {
    struct Entry {
        std::vector<tc_handle*> hs;
        std::vector<long long> uids, epochs;
        std::vector<int> sorts;
        cudaGraphExec_t ge = nullptr;
        std::vector<StepGraph> cases;
        long long n_static = 0;
    };
    int nthreads = 1;
    int device = 0;
    cudaStream_t root = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    std::vector<Entry*> cache;  // most recent last, at most kCache
    long long graph_steps = 0, eager_steps = 0;
    bool failed = false;
    static constexpr size_t kCache = 4;
};

namespace {
void drop_entry(tc_ensemble::Entry* en) {
    if (en->ge) cudaGraphExecDestroy(en->ge);
    delete en;
}

tc_ensemble::Entry* build_entry(tc_ensemble* e, tc_handle* const* hs, int n) {
    auto* en = new tc_ensemble::Entry();
    en->hs.assign(hs, hs + n);
    en->cases.resize((size_t)n);
    for (int i = 0; i < n; i++) {
        Handle* h = &hs[i]->h;
        if (step_graph_prepare(h) != TC_OK) {
            drop_entry(en);
            return nullptr;
        }
        en->uids.push_back(h->uid);
        en->epochs.push_back(h->epoch);
        en->sorts.push_back(sorts_this_step(h) ? 1 : 0);
    }
    while (e->join.size() < (size_t)n) {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            drop_entry(en);
            return nullptr;
        }
        e->join.push_back(ev);
    }
    if (cudaStreamBeginCapture(e->root, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        drop_entry(en);
        return nullptr;
    }
    bool ok = cudaEventRecord(e->fork, e->root) == cudaSuccess;
    for (int i = 0; i < n && ok; i++) {
        Handle* h = &hs[i]->h;
        ok = cudaStreamWaitEvent(h->st, e->fork, 0) == cudaSuccess && capture_step(h, &en->cases[(size_t)i]) == TC_OK;
        en->n_static += en->cases[(size_t)i].n_static;
        ok = ok && cudaEventRecord(e->join[(size_t)i], h->st) == cudaSuccess &&
             cudaStreamWaitEvent(e->root, e->join[(size_t)i], 0) == cudaSuccess;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(e->root, &g);
    ok = ok && ee == cudaSuccess && g != nullptr && cudaGraphInstantiate(&en->ge, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        drop_entry(en);
        return nullptr;
    }
    return en;
}
}  // namespace

extern "C" {

void tc_default_params(tc_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->nx = 200; p->nz = 200; p->aspect = 1.0; p->order = 2;
    p->gridX = 0; p->gridZ = 0; p->spaceX = 1.0; p->spaceZ = 1.0; p->thickness = 0.1; p->nbound = 8;
    p->non_Newtonian = 0; p->iterate_order = 1; p->tolerance = 1.0e-3; p->Nmulti = 70; p->mingrid = 4;
    p->grids = 2; p->eig_ratio = 4.0; p->vis_iter = 12; p->max_cycles = 1000;
    p->torder = 4; p->courant = 0.99; p->courantT = 0.99; p->courantC = 0.99; p->courant_stream = 0.99;
    p->RK_update = 1; p->dt_manual = 0.5;
    p->comp = 1; p->ntype = 1; p->tpc = 30; p->dist_factor = 1.0e-4;
    p->Tbot = 0; p->Vbc = 0; p->dlayer = 0.1; p->dent = 0.1;
    p->RaT = 1.0e3 / 3.0; p->H = 0.0;
    for (int t = 0; t < TC_MAX_TYPES; t++) {
        p->RaC[t] = 0.0; p->conduct_factor[t] = 1.0; p->Htype[t] = 0.0; p->visC[t] = 1.0; p->delta_visC[t] = 2.0;
    }
    p->eig_ratio_min = 4.0; p->ivis = 2; p->visP = 1.0; p->visT = 3.0e4; p->delta_visT = 100.0;
    p->yield = 15.0; p->yield_gradient = 0.0; p->yield_depth = 0.1;
    p->tracer_sort_interval = 10;
}

void tc_abi_sizes(int32_t sizes[3]) {
    sizes[0] = (int32_t)sizeof(tc_params);
    sizes[1] = (int32_t)sizeof(tc_stats_row);
    sizes[2] = (int32_t)sizeof(tc_info);
}

tc_status tc_create(const tc_params* p, tc_handle** out) {
    if (!p || !out) return TC_ERR_ARG;
    *out = nullptr;
    tc_handle* H = new (std::nothrow) tc_handle();
    if (!H) return TC_ERR_ALLOC;
    H->h.uid = ++g_handle_uid;
    tc_status s = create(&H->h, p);
    if (s != TC_OK) {
        static thread_local std::string last;
        last = H->h.err;
        tc_destroy(H);
        return s;
    }
    *out = H;
    return TC_OK;
}

tc_status tc_attach_net(tc_handle* H, tc_net* net) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    tc_net_impl* n = tcnn_impl(net);
    if (n) {
        int nh = 0, nw = 0;
        net_dims(n, &nh, &nw);
        if (nh != h->nz || nw != h->nx) return TC_ERR_ARG;
        if (!h->guess) TRY(dalloc_t(h, &h->guess, h->L1.plane));
        if (!h->nn_raw) TRY(dalloc_t(h, &h->nn_raw, (size_t)3 * h->nx * h->nz));
    }
    h->net = n;
    drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_record_solves(tc_handle* H, float* raw, float* sf_new, int32_t capacity) {
    if (!H || capacity < 0 || (capacity > 0 && (!raw || !sf_new))) return TC_ERR_ARG;
    Handle* h = &H->h;
    h->rec_raw = capacity > 0 ? raw : nullptr;
    h->rec_sf = capacity > 0 ? sf_new : nullptr;
    h->rec_cap = capacity;
    h->rec_count = 0;
    drop_step_graphs(h);
    return TC_OK;
}

int32_t tc_record_count(const tc_handle* H) { return H ? H->h.rec_count : 0; }

tc_status tc_guess_stats(const tc_handle* H, int64_t* used, int64_t* offered) {
    if (!H) return TC_ERR_ARG;
    if (used) *used = H->h.guess_used;
    if (offered) *offered = H->h.guess_offered;
    return TC_OK;
}

tc_status tc_destroy(tc_handle* H) {
    if (!H) return TC_OK;
    Handle* h = &H->h;
    if (h->st) cudaStreamSynchronize(h->st);
    for (void* q : h->allocs) cudaFree(q);
    if (h->eq_donor) cudaFree(h->eq_donor);
    if (h->hs) cudaFreeHost(h->hs);
    if (h->graphs) {
        if (h->graphs->l1) cudaGraphExecDestroy(h->graphs->l1);
        if (h->graphs->rest) cudaGraphExecDestroy(h->graphs->rest);
        if (h->graphs->loop) cudaGraphExecDestroy(h->graphs->loop);
        delete h->graphs;
    }
    for (auto& kv : h->flt_graphs)
        if (kv.second) cudaGraphExecDestroy(kv.second);
    drop_step_graphs(h);
    if (h->hsnap) cudaFreeHost(h->hsnap);
    if (h->body_st) cudaStreamDestroy(h->body_st);
    if (h->own_stream && h->st) cudaStreamDestroy(h->st);
    delete H;
    return TC_OK;
}

tc_status tc_get_info(const tc_handle* H, tc_info* info) {
    if (!H || !info) return TC_ERR_ARG;
    const Handle* h = &H->h;
    std::memset(info, 0, sizeof(*info));
    info->nx = h->nx; info->nz = h->nz; info->span = SP; info->span_interp = 1; info->grids = h->grids;
    info->nsteps = h->nsteps; info->ntr = h->ntr; info->ngrid_coarse = h->ngrid_coarse; info->kl = h->kl;
    info->ku = h->ku;
    for (int l = 1; l <= h->grids && l <= 8; l++) { info->nx_grid[l - 1] = h->lev[l].L.a; info->nz_grid[l - 1] = h->lev[l].L.b; }
    info->dr = h->grid_dr; info->ds = h->grid_ds;
    return TC_OK;
}

tc_status tc_grid_metrics(const tc_params* p, double* x5, double* z5) {
    if (!p || !x5 || !z5 || p->nx < 4 || p->nz < 4) return TC_ERR_ARG;
    tcs::FD fd;
    tcs::fd_coefficients(2, fd);
    tcs::GridMetrics g;
    tcs::grid_metrics(p->aspect, p->nx, p->nz, p->gridX, p->gridZ, p->spaceX, p->spaceZ, p->thickness, p->nbound, fd,
                      g);
    const std::vector<double>* xs[5] = {&g.xr, &g.xrr, &g.xrrr, &g.xrrrr, &g.dxr};
    const std::vector<double>* zs[5] = {&g.zs, &g.zss, &g.zsss, &g.zssss, &g.dzs};
    for (int q = 0; q < 5; q++) {
        std::copy(xs[q]->begin(), xs[q]->end(), x5 + (size_t)q * (p->nx + 7));
        std::copy(zs[q]->begin(), zs[q]->end(), z5 + (size_t)q * (p->nz + 7));
    }
    return TC_OK;
}

tc_status tc_grid_coordinates(const tc_handle* H, double* xg, double* zg) {
    if (!H || !xg || !zg) return TC_ERR_ARG;
    std::copy(H->h.xg_h.begin(), H->h.xg_h.end(), xg);
    std::copy(H->h.zg_h.begin(), H->h.zg_h.end(), zg);
    return TC_OK;
}

tc_status tc_get_params(const tc_handle* H, tc_params* p) {
    if (!H || !p) return TC_ERR_ARG;
    *p = H->h.p;
    return TC_OK;
}

tc_status tc_set_stream(tc_handle* H, void* stream) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->own_stream && h->st) cudaStreamDestroy(h->st);
    h->own_stream = false;
    h->st = (cudaStream_t)stream;
    drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_upload_state(tc_handle* H, const double* T, const double* Cnew, const double* SF, const double* rtr,
                          const double* str, const int32_t* Ttype, int64_t ntr) {
    if (!H) return TC_ERR_ARG;
    return upload(&H->h, T, Cnew, SF, rtr, str, Ttype, ntr);
}

tc_status tc_upload_state_ex(tc_handle* H, const double* T, const double* Cnew, const double* SF, const double* rtr,
                             const double* str, const int32_t* Ttype, const double* Ttr, int64_t ntr) {
    if (!H) return TC_ERR_ARG;
    return upload(&H->h, T, Cnew, SF, rtr, str, Ttype, ntr, Ttr);
}

tc_status tc_equalize_row(const tc_handle* H, int64_t* out, int32_t cap, int32_t* len) {
    if (!H || !len) return TC_ERR_ARG;
    const Handle* h = &H->h;
    if ((int32_t)h->eq_row.size() > cap || (!out && !h->eq_row.empty())) return TC_ERR_ARG;
    for (size_t q = 0; q < h->eq_row.size(); q++) out[q] = h->eq_row[q];
    *len = (int32_t)h->eq_row.size();
    return TC_OK;
}

tc_status tc_download_tracer_temperature(tc_handle* H, double* Ttr) {
    if (!H || !Ttr) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (h->p.tracer != 1 || !h->Ttr) return TC_ERR_ARG;
    TRY(download_tracers(h, nullptr, nullptr, nullptr, Ttr));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

tc_status tc_download_state(tc_handle* H, double* T, double* Cnew, double* SF, double* rtr, double* str,
                            int32_t* Ttype) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (T) TRY(get_field(h, T, h->T));
    if (SF) TRY(get_field(h, SF, h->SF));
    if (Cnew && h->ntype > 0) {
        const size_t ni = (size_t)h->nx + 1 + 2 * SP, nk = (size_t)h->nz + 1 + 2 * SP;
        std::vector<double> tmp(ni * nk);
        for (int t = 0; t < h->ntype; t++) {
            TRY(get_field(h, tmp.data(), h->Cnew[t]));
            CK(cudaStreamSynchronize(h->st));
            for (size_t x = 0; x < ni * nk; x++) Cnew[x * h->ntype + t] = tmp[x];
        }
    }
    if (h->p.comp == 1 || h->p.tracer == 1) TRY(download_tracers(h, rtr, str, h->p.comp == 1 ? Ttype : nullptr));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

tc_status tc_set_clock(tc_handle* H, int32_t tstep, double time) {
    if (!H) return TC_ERR_ARG;
    H->h.tstep = tstep;
    H->h.time = time;
    return TC_OK;
}

tc_status tc_multigrid(tc_handle* H, int32_t* cycles_out) {
    if (!H) return TC_ERR_ARG;
    tc_status s = multigrid(&H->h);
    if (cycles_out) *cycles_out = H->h.last_cycles;
    return s;
}

tc_status tc_compute_velocities(tc_handle* H) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    compute_velocities(h);
    CK(cudaGetLastError());
    return TC_OK;
}

tc_status tc_stats(tc_handle* H, tc_stats_row* row) {
    if (!H || !row) return TC_ERR_ARG;
    return stats(&H->h, row);
}

tc_status tc_energy_time(tc_handle* H, double* dt_out) {
    if (!H) return TC_ERR_ARG;
    tc_status s = energy_time(&H->h);
    if (dt_out) *dt_out = H->h.dt;
    return s;
}

tc_status tc_step(tc_handle* H, tc_stats_row* row, int32_t* cycles, double* dt_out) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (step_graph_ready(h, true)) {
        bool ran = false;
        const tc_status s = step_as_graph(h, row, cycles, dt_out, &ran);
        if (ran || s != TC_OK) return s;
    }
    h->cycles_acc = 0;
    tc_status s = multigrid(h);
    if (cycles) *cycles = h->last_cycles;
    if (s != TC_OK) return s;
    compute_velocities(h);
    tc_stats_row tmp;
    TRY(stats(h, row ? row : &tmp));
    s = energy_time(h);
    if (cycles) *cycles = h->cycles_acc;
    if (s != TC_OK) return s;
    if (dt_out) *dt_out = h->dt;
    h->time = h->time + h->dt;
    h->tstep += 1;
    return TC_OK;
}


tc_status tc_autotune(tc_handle* H, int32_t* choices) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    const bool mixed = (h->p.solver_precision == 1);
    const int G = h->grids;
    // candidate block shapes (at most 256 threads: the kernels' launch bounds)
    const int shapes[][2] = {{32, 8}, {64, 4}, {128, 2}, {256, 1}, {32, 4}, {16, 16}, {64, 2}, {16, 8}};
    for (int l = 1; l < G; l++) {
        Level& lv = h->lev[l];
        // the timed sweeps and visits change the level's corrections: keep a copy
        const size_t bytes = lv.L.plane * (mixed ? sizeof(float) : sizeof(double));
        void* save[2] = {nullptr, nullptr};
        for (int q = 0; q < 2; q++) {
            CK(cudaMalloc(&save[q], bytes));
            CK(cudaMemcpyAsync(save[q], mixed ? (void*)lv.e32[q] : (void*)lv.err[q], bytes, cudaMemcpyDeviceToDevice,
                               h->st));
        }
        // block shape of the per-sweep smoother kernel
        double best = 1e30;
        int bb = 0;
        for (int c = 0; c < (int)(sizeof(shapes) / sizeof(shapes[0])); c++) {
            lv.sweep_bx = shapes[c][0];
            lv.sweep_by = shapes[c][1];
            double ms = 0;
            TRY(graph_time(h, [&]() {
                for (int n = 0; n < 20; n++) {
                    if (mixed) launch_sweep32(h->st, lv, lv.e32[0], lv.e32[1], 1.0f, 0, 0.f, h->p.Vbc);
                    else launch_sweep(h->st, lv, lv.err[0], lv.err[1], 1.0, 0, 0.0, h->p.Vbc);
                }
            }, &ms));
            if (ms < best) { best = ms; bb = c; }
        }
        lv.sweep_bx = shapes[bb][0];
        lv.sweep_by = shapes[bb][1];
        // unfused visits: 1..6 sweeps per launch (tiled smoother for 2..6;
        // FP64 at most 2); then one cluster launch per visit in each shape
        // that fits (points per strip x CTAs)
        auto time_visits = [&](double* ms) {
            return graph_time(h, [&]() {
                for (int v = 0; v < 2; v++) {
                    if (mixed) iterate_stream32(h, l, 1);
                    else iterate_stream(h, l, 1);
                }
            }, ms);
        };
        lv.fuse = 0;
        lv.visit_cfg = 0;
        double best_v = 1e30;
        int best_blk = 0;
        const bool gf = lv.g32 && lv.use_g32;
        for (int blk = 0; blk <= (mixed ? (gf ? 3 : 6) : 2); blk++) {
            if (gf && blk == 1) continue;  // field sweeps: 0 (one per launch), 2 or 3 per launch
            lv.blk = blk;
            double ms = 0;
            TRY(time_visits(&ms));
            if (ms < best_v) { best_v = ms; best_blk = blk; }
        }
        lv.blk = best_blk;
        int best_cfg = -1;  // -1 = unfused
        if (l > 1 && h->fuse_visits && visit_cluster_fits(lv.L, h->p.Nmulti, mixed ? 1 : 0)) {
            lv.fuse = 1;
            std::vector<int> cfgs = {0};
            for (int p : {1, 2})
                for (int c : {1, 2, 4, 8, 16}) cfgs.push_back(100 * p + c);
            for (int cfg : cfgs) {
                if (!visit_cluster_fits(lv.L, h->p.Nmulti, mixed ? 1 : 0, cfg)) continue;
                lv.visit_cfg = cfg;
                double ms = 0;
                TRY(time_visits(&ms));
                if (ms < best_v) { best_v = ms; best_cfg = cfg; }
            }
        }
        lv.fuse = (best_cfg >= 0) ? 1 : 0;
        lv.visit_cfg = (best_cfg > 0) ? best_cfg : 0;
        for (int q = 0; q < 2; q++) {
            CK(cudaMemcpyAsync(mixed ? (void*)lv.e32[q] : (void*)lv.err[q], save[q], bytes, cudaMemcpyDeviceToDevice,
                               h->st));
        }
        CK(cudaStreamSynchronize(h->st));
        for (int q = 0; q < 2; q++) cudaFree(save[q]);
        if (choices) {
            choices[3 * (l - 1) + 0] = lv.sweep_bx;
            choices[3 * (l - 1) + 1] = lv.sweep_by;
            choices[3 * (l - 1) + 2] = lv.fuse ? (lv.visit_cfg ? lv.visit_cfg : 1) : (lv.blk > 0 ? 1000 + lv.blk : 0);
        }
    }
    // the cycle graphs bake in launch shapes: capture again at the next solve
    CycleGraphs& cg = *h->graphs;
    if (cg.l1) cudaGraphExecDestroy(cg.l1);
    if (cg.rest) cudaGraphExecDestroy(cg.rest);
    if (cg.loop) cudaGraphExecDestroy(cg.loop);
    cg.l1 = cg.rest = cg.loop = nullptr;
    drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_set_launch_shapes(tc_handle* H, const int32_t* choices) {
    if (!H || !choices) return TC_ERR_ARG;
    Handle* h = &H->h;
    const bool mixed = (h->p.solver_precision == 1);
    const int G = h->grids;
    for (int l = 1; l < G; l++) {
        const int bx = choices[3 * (l - 1)], by = choices[3 * (l - 1) + 1], v = choices[3 * (l - 1) + 2];
        if (bx < 1 || by < 1 || bx * by > 256 || (bx * by) % 32 != 0 || v < 0) return TC_ERR_ARG;
        if (v > 1000) {
            if (!(v == 1001 || v == 1002 || (v >= 1003 && v <= 1006 && mixed))) return TC_ERR_ARG;
        } else if (v > 1 &&
                   (l == 1 || !h->fuse_visits || !visit_cluster_fits(h->lev[l].L, h->p.Nmulti, mixed ? 1 : 0, v))) {
            return TC_ERR_ARG;
        }
    }
    for (int l = 1; l < G; l++) {
        Level& lv = h->lev[l];
        lv.sweep_bx = choices[3 * (l - 1)];
        lv.sweep_by = choices[3 * (l - 1) + 1];
        const int v = choices[3 * (l - 1) + 2];
        lv.fuse = (v != 0 && v < 1000) ? 1 : 0;
        lv.visit_cfg = (v > 1 && v < 1000) ? v : 0;
        lv.blk = (v > 1000) ? v - 1000 : 0;
    }
    CycleGraphs& cg = *h->graphs;
    if (cg.l1) cudaGraphExecDestroy(cg.l1);
    if (cg.rest) cudaGraphExecDestroy(cg.rest);
    if (cg.loop) cudaGraphExecDestroy(cg.loop);
    cg.l1 = cg.rest = cg.loop = nullptr;
    drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_ensemble_step(tc_handle* const* hs, int32_t n, int32_t nthreads, tc_stats_row* rows, int32_t* cycles,
                           double* dts, tc_status* status) {
    if (!hs || n < 1 || nthreads < 1) return TC_ERR_ARG;
    for (int i = 0; i < n; i++)
        if (!hs[i]) return TC_ERR_ARG;
    std::atomic<int> next{0};
    std::vector<tc_status> st((size_t)n, TC_OK);
    auto work = [&]() {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n) break;
            cudaSetDevice(hs[i]->h.device);
            st[(size_t)i] = tc_step(hs[i], rows ? &rows[i] : nullptr, cycles ? &cycles[i] : nullptr,
                                    dts ? &dts[i] : nullptr);
        }
    };
    const int T = nthreads < n ? nthreads : n;
    std::vector<std::thread> pool;
    for (int t = 1; t < T; t++) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    tc_status first = TC_OK;
    for (int i = 0; i < n; i++) {
        if (status) status[i] = st[(size_t)i];
        if (first == TC_OK && st[(size_t)i] != TC_OK) first = st[(size_t)i];
    }
    return first;
}

tc_status tc_set_step_graph(tc_handle* H, int32_t on) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    h->step_graph = (on != 0);
    h->step_graph_failed = false;
    if (!h->step_graph) drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_step_graph_info(const tc_handle* H, int64_t* graph_steps, int32_t* state) {
    if (!H) return TC_ERR_ARG;
    const Handle* h = &H->h;
    if (graph_steps) *graph_steps = h->graph_steps;
    if (state) *state = h->step_graph_failed ? 2 : (h->step_graph ? 1 : 0);
    return TC_OK;
}

tc_status tc_ensemble_create(int32_t nthreads, tc_ensemble** out) {
    if (!out || nthreads < 1) return TC_ERR_ARG;
    auto* e = new tc_ensemble();
    e->nthreads = nthreads;
    cudaGetDevice(&e->device);
    if (cudaStreamCreateWithFlags(&e->root, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess) {
        tc_ensemble_destroy(e);
        return TC_ERR_CUDA;
    }
    *out = e;
    return TC_OK;
}

tc_status tc_ensemble_run(tc_ensemble* e, tc_handle* const* hs, int32_t n, tc_stats_row* rows, int32_t* cycles,
                          double* dts, tc_status* status) {
    if (!e || !hs || n < 1) return TC_ERR_ARG;
    bool ready = !e->failed;
    for (int i = 0; i < n; i++) {
        if (!hs[i]) return TC_ERR_ARG;
        ready = ready && step_graph_ready(&hs[i]->h, false) && hs[i]->h.device == e->device;
    }
    tc_ensemble::Entry* en = nullptr;
    if (ready) {
        const std::vector<tc_handle*> key(hs, hs + n);
        for (auto* c : e->cache) {
            if (c->hs != key) continue;
            bool same = true;
            for (int i = 0; i < n && same; i++)
                same = c->uids[(size_t)i] == hs[i]->h.uid && c->epochs[(size_t)i] == hs[i]->h.epoch &&
                       c->sorts[(size_t)i] == (sorts_this_step(&hs[i]->h) ? 1 : 0);
            if (same) en = c;
        }
        if (!en) {
            cudaSetDevice(e->device);
            en = build_entry(e, hs, n);
            if (en) {
                e->cache.push_back(en);
                if (e->cache.size() > tc_ensemble::kCache) {
                    drop_entry(e->cache.front());
                    e->cache.erase(e->cache.begin());
                }
            } else {
                e->failed = true;  // the CUDA runtime refused the capture: the thread pool from now on
            }
        }
    }
    if (!en) {
        e->eager_steps++;
        return tc_ensemble_step(hs, n, e->nthreads, rows, cycles, dts, status);
    }
    for (int i = 0; i < n; i++) hs[i]->h.cycles_acc = 0;
    cudaSetDevice(e->device);
    if (cudaGraphLaunch(en->ge, e->root) != cudaSuccess) return TC_ERR_CUDA;
    tc_note_launch(en->n_static);
    if (cudaStreamSynchronize(e->root) != cudaSuccess || cudaGetLastError() != cudaSuccess) return TC_ERR_CUDA;
    tc_status first = TC_OK;
    for (int i = 0; i < n; i++) {
        const tc_status s = finish_step(&hs[i]->h, en->cases[(size_t)i], rows ? &rows[i] : nullptr,
                                        cycles ? &cycles[i] : nullptr, dts ? &dts[i] : nullptr);
        if (status) status[i] = s;
        if (first == TC_OK && s != TC_OK) first = s;
    }
    e->graph_steps++;
    return first;
}

tc_status tc_ensemble_info(const tc_ensemble* e, int64_t* graph_steps, int64_t* eager_steps) {
    if (!e) return TC_ERR_ARG;
    if (graph_steps) *graph_steps = e->graph_steps;
    if (eager_steps) *eager_steps = e->eager_steps;
    return TC_OK;
}

tc_status tc_ensemble_destroy(tc_ensemble* e) {
    if (!e) return TC_OK;
    if (e->root) cudaStreamSynchronize(e->root);
    for (auto* c : e->cache) drop_entry(c);
    for (auto ev : e->join) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->root) cudaStreamDestroy(e->root);
    delete e;
    return TC_OK;
}

tc_status tc_step_host(tc_handle* H, double* T, double* Cnew, double* SF, double* rtr, double* str,
                       const int32_t* Ttype, int64_t ntr, tc_stats_row* row, int32_t* cycles, double* dt_out) {
    if (!H || !T || !SF) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    if (h->p.tracer == 1) {
        h->err = "tc_step_host carries no tracer temperatures: use tc_step with tc_download_tracer_temperature";
        return TC_ERR_UNSUPPORTED;
    }
    if (h->p.comp == 1 && (ntr != h->ntr || !rtr || !str || !Ttype || !Cnew)) return TC_ERR_ARG;
    TRY(put_field(h, h->T, T));
    TRY(put_field(h, h->SF, SF));
    if (h->ntype == 1) TRY(put_field(h, h->Cnew[0], Cnew));
    if (h->p.comp == 1) {
        CK(cudaMemcpyAsync(h->rtr, rtr, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
        CK(cudaMemcpyAsync(h->str, str, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
        CK(cudaMemcpyAsync(h->ttype, Ttype, sizeof(int32_t) * h->ntr, cudaMemcpyHostToDevice, h->st));
        launch_iota(h->st, h->ntr, h->perm);
    }
    tc_status s = tc_step(H, row, cycles, dt_out);
    if (s != TC_OK) return s;
    TRY(get_field(h, T, h->T));
    TRY(get_field(h, SF, h->SF));
    if (h->ntype == 1) TRY(get_field(h, Cnew, h->Cnew[0]));
    if (h->p.comp == 1) TRY(download_tracers(h, rtr, str, nullptr));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

tc_status tc_time_sweep(tc_handle* H, int32_t level, int32_t nsweeps, double* ms_per_sweep) {
    if (!H || !ms_per_sweep || nsweeps < 1) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (level < 1 || level >= h->grids) return TC_ERR_ARG;
    Level& lv = h->lev[level];
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // sweeps read the current buffer and write the other one; the state is
    // untouched.  The mixed solve times its FP32 smoother kernel.
    const bool mixed = (h->p.solver_precision == 1);
    auto sweep = [&]() {
        if (mixed) launch_sweep32(h->st, lv, lv.e32[lv.e32cur], lv.e32[1 - lv.e32cur], 1.0f, 0, 0.0f, h->p.Vbc);
        else launch_sweep(h->st, lv, lv.err[lv.ecur], lv.err[1 - lv.ecur], 1.0, 0, 0.0, h->p.Vbc);
    };
    // the sweeps are captured in a CUDA graph and replayed, as the solver
    // runs them (per-launch host overhead would otherwise dominate)
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    const long long before = t_launches;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    for (int n = 0; n < nsweeps; n++) sweep();
    CK(cudaStreamEndCapture(h->st, &g));
    g_launches.fetch_sub(t_launches - before);
    t_launches = before;
    cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    CK(cudaGraphLaunch(ge, h->st));
    CK(cudaEventRecord(e0, h->st));
    CK(cudaGraphLaunch(ge, h->st));
    CK(cudaEventRecord(e1, h->st));
    CK(cudaEventSynchronize(e1));
    cudaGraphExecDestroy(ge);
    tc_note_launch(2LL * nsweeps);
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_sweep = (double)ms / nsweeps;
    return TC_OK;
}

tc_status tc_time_visit(tc_handle* H, int32_t level, int32_t reps, double* ms_per_visit) {
    if (!H || !ms_per_visit || reps < 1) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    if (level < 1 || level >= h->grids) return TC_ERR_ARG;
    const bool mixed = (h->p.solver_precision == 1);
    auto visit = [&]() {
        if (level == 1 && mixed) enqueue_l1_mixed(h, 0);
        else if (mixed) iterate_stream32(h, level, 0);
        else iterate_stream(h, level, 0);
    };
    // one visit launched directly (counted), then reps visits captured in a
    // CUDA graph and replayed, as the solver runs them (per-launch host
    // overhead would otherwise dominate the many-launch visits)
    h->enq_err = cudaSuccess;
    const long long n0 = t_launches;
    visit();
    CK(h->enq_err);
    const long long per_visit = t_launches - n0;
    double ms = 0.0;
    TRY(graph_time(h, [&]() {
        for (int n = 0; n < reps; n++) visit();
    }, &ms));
    tc_note_launch(per_visit * reps);
    *ms_per_visit = ms / reps;
    return TC_OK;
}

tc_status tc_time_subcycle(tc_handle* H, int32_t k, int32_t reps, double* ms_per_apply) {
    if (!H || !ms_per_apply || reps < 1 || k < 1 || k > 4) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    if (!h->sub_on || h->subM[k - 1] == nullptr) return TC_ERR_UNSUPPORTED;
    const int S = h->grids - 1;
    const bool mixed = (h->p.solver_precision == 1);
    void* err = mixed ? (void*)cur_e32(h, S) : (void*)cur_err(h, S);
    auto apply = [&]() {
        launch_subcycle_apply(h->st, h->lev[S], h->subM[k - 1], mixed ? 1 : 0, h->sub_m32 ? 1 : 0, err, h->p.Vbc);
    };
    apply();
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, h->st));
    for (int n = 0; n < reps; n++) apply();
    CK(cudaEventRecord(e1, h->st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_apply = (double)ms / reps;
    return TC_OK;
}

tc_status tc_debug_wait_test(tc_handle* H, int32_t on) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    h->wait_test = (on != 0);
    // the cycle graphs bake in the visits' parameters: capture again
    CycleGraphs& cg = *h->graphs;
    if (cg.l1) cudaGraphExecDestroy(cg.l1);
    if (cg.rest) cudaGraphExecDestroy(cg.rest);
    if (cg.loop) cudaGraphExecDestroy(cg.loop);
    cg.l1 = cg.rest = cg.loop = nullptr;
    drop_step_graphs(h);
    return TC_OK;
}

tc_status tc_debug_sweep_fields(tc_handle* H, int32_t fields) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (h->lev[1].g32 == nullptr) return TC_ERR_UNSUPPORTED;
    h->lev[1].use_g32 = fields ? 1 : 0;
    CycleGraphs& cg = *h->graphs;
    if (cg.l1) cudaGraphExecDestroy(cg.l1);
    if (cg.rest) cudaGraphExecDestroy(cg.rest);
    if (cg.loop) cudaGraphExecDestroy(cg.loop);
    cg.l1 = cg.rest = cg.loop = nullptr;
    drop_step_graphs(h);
    return TC_OK;
}

int64_t tc_kernel_launches(void) { return (int64_t)g_launches.load(); }

tc_status tc_download_velocities(tc_handle* H, double* u, double* w) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    // (-1:nx+1, -1:nz+1) sub-box of the padded plane
    const size_t ni = (size_t)h->nx + 3, nk = (size_t)h->nz + 3;
    const size_t off = IX(h->L1, -1, -1);
    if (u) CK(cudaMemcpy2DAsync(u, ni * sizeof(double), h->u + off, h->L1.ld * sizeof(double), ni * sizeof(double), nk,
                                cudaMemcpyDeviceToHost, h->st));
    if (w) CK(cudaMemcpy2DAsync(w, ni * sizeof(double), h->w + off, h->L1.ld * sizeof(double), ni * sizeof(double), nk,
                                cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

tc_status tc_tracers_to_corners(tc_handle* H, const double* rtr, const double* str) {
    if (!H || !rtr || !str) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (h->p.comp != 1) return TC_ERR_UNSUPPORTED;
    // positions in the reference's order, gathered into the cell order of
    // the tracer types
    CK(cudaMemcpyAsync(h->rtr1, rtr, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->str1, str, sizeof(double) * h->ntr, cudaMemcpyHostToDevice, h->st));
    launch_perm_gather(h->st, h->ntr, h->perm, h->rtr1, h->rtr2);
    launch_perm_gather(h->st, h->ntr, h->perm, h->str1, h->str2);
    TRY(tracers_to_corners(h, h->rtr2, h->str2, true));
    return check_flags(h);
}

tc_status tc_compute_strain_rate_invariant(tc_handle* H) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    launch_strain(h->st, h->L1, h->P, h->u, h->w, h->strain);
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    return TC_OK;
}

tc_status tc_compute_viscosity(tc_handle* H, int32_t level) {
    if (!H) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (!h->uploaded) return TC_ERR_STATE;
    if (level < 1 || level > h->grids) return TC_ERR_ARG;
    TRY(compute_viscosity(h, level));
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    return TC_OK;
}

tc_status tc_tracer_order(tc_handle* H, int32_t* perm) {
    if (!H || !perm) return TC_ERR_ARG;
    Handle* h = &H->h;
    if (h->ntr <= 0 || !h->perm) return TC_ERR_STATE;
    CK(cudaMemcpyAsync(perm, h->perm, sizeof(int32_t) * (size_t)h->ntr, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

tc_status tc_download_counts(tc_handle* H, int32_t* count_type) {
    if (!H || !count_type) return TC_ERR_ARG;
    Handle* h = &H->h;
    const int nt = h->ntype + 1;
    std::vector<int> hv(h->L1.plane * (size_t)nt);
    CK(cudaMemcpyAsync(hv.data(), h->counts, hv.size() * sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const int ni = h->nx + 1 + 2 * SP, nk = h->nz + 1 + 2 * SP;
    for (int kk = 0; kk < nk; kk++)
        for (int ii = 0; ii < ni; ii++)
            for (int t = 0; t < nt; t++)
                count_type[((size_t)kk * ni + ii) * nt + t] = hv[(size_t)t * h->L1.plane + (size_t)ii + (size_t)kk * h->L1.ld];
    return TC_OK;
}

tc_status tc_debug_field(tc_handle* H, const char* name, int32_t level, int32_t type, double* out) {
    if (!H || !name || !out) return TC_ERR_ARG;
    Handle* h = &H->h;
    std::string n(name);
    const double* src = nullptr;
    Lay L = h->L1;
    auto ty = [&](double* const* a) -> const double* { return (type >= 1 && type <= h->ntype) ? a[type - 1] : nullptr; };
    if (level >= 1 && level <= h->grids) {
        Level& lv = h->lev[level];
        if (n == "vis_grid") src = lv.vis[lv.vcur];
        else if (n == "vis_x") src = lv.vx;
        else if (n == "vis_z") src = lv.vz;
        else if (n == "vis_xx") src = lv.vxx;
        else if (n == "vis_zz") src = lv.vzz;
        else if (n == "vis_xz") src = lv.vxz;
        else if (n == "dt_stream") src = lv.dt_stream;
        else if (n == "ratio") src = lv.ratio;
        else if (n == "RHS") src = lv.rhs;
        else if (n == "error") src = lv.err[lv.ecur];
        else if (n == "residual") src = lv.res;
        else if (n == "dt_vis") src = lv.dt_vis;
        if (src) L = lv.L;
    }
    if (!src) {
        if (n == "T") src = h->T;
        else if (n == "SF") src = h->SF;
        else if (n == "Tvis") src = h->Tvis;
        else if (n == "Tbuoy") src = h->Tbuoy;
        else if (n == "u") src = h->u;
        else if (n == "w") src = h->w;
        else if (n == "conduct") src = h->conduct;
        else if (n == "conduct_r") src = h->conduct_r;
        else if (n == "conduct_s") src = h->conduct_s;
        else if (n == "DERr_u") src = h->du;
        else if (n == "DERr_w") src = h->dw;
        else if (n == "dts_array") src = h->dts;
        else if (n == "strain") src = h->strain;
        else if (n == "Tratio") src = h->Tratio;
        else if (n == "tracer_space_array") src = h->tsa;
        else if (n == "Cnew") src = ty(h->Cnew);
        else if (n == "Cvis") src = ty(h->Cvis);
        else if (n == "Cbuoy") src = ty(h->Cbuoy);
    }
    if (!src) return TC_ERR_ARG;
    const size_t ni = (size_t)L.a + 1 + 2 * SP, nk = (size_t)L.b + 1 + 2 * SP;
    CK(cudaMemcpy2DAsync(out, ni * sizeof(double), src, L.ld * sizeof(double), ni * sizeof(double), nk,
                         cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return TC_OK;
}

const char* tc_last_error(const tc_handle* H) {
    if (!H) return "";
    return H->h.err.c_str();
}

}  // extern "C"
