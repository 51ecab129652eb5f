// k_noalloc.cu -- tc_stats_noalloc: the stats.dat integrals computed from
// device arrays the caller owns, without allocating anything.
//
// Who needs it: a host that owns every device allocation itself -- for
// example an OpenACC or CUDA Fortran port of the reference that keeps T, u,
// w, C, ... in its own memory pool, or an application running under a fixed
// device-memory budget -- and therefore cannot let a library call cudaMalloc
// (or create a tc_handle, which allocates).  The caller passes the input
// arrays and the output row; the only other memory used is the fixed-size
// buffer below.
//
// Scratch: one file-scope __device__ array (rows of per-k integrals, the
// integral results, and three reduction integers), 229,712 bytes.  Every
// GPU that loads this library holds one copy until the process exits.  It
// limits nz to TC_NOALLOC_MAX_NZ; larger inputs are rejected with
// TC_ERR_TOO_LARGE.  All calls share the array and it keeps the last
// call's contents; the reduction integers are re-initialised at the start
// of every call.  Two calls whose work overlaps on the GPU (different
// streams, or different host threads without ordering) race on it.
//
// Set-up: the array's host-side name is only a stand-in, not a device
// address, so the entry point looks up the device address once per device
// (cudaGetSymbolAddress, with that device current) on its first call there
// and caches it together with the device's current context.  A call that
// finds another context current on that device (after cudaDeviceReset, or
// when the primary context was released and created again, which may load
// the module at another address) looks the address up again.  Make the first
// call on a device before capturing any stream on it.
//
// Errors: the launches' own return codes and the stream synchronisation are
// checked; the runtime's last-error state is neither read nor cleared, so an
// error that the caller's own code left pending stays the caller's.
//
// The kernels are a variant of k_stats_rows / k_stats_final (k_field.cu)
// that read the reference's own array layouts (no padding) and take their
// scratch from the fixed array; the arithmetic and its order are the same,
// so the row equals tc_stats' row for the same fields.
#include "tc_device.cuh"

#include <cmath>
#include <cstring>
#include <mutex>

#define TC_NOALLOC_ROWS 7

namespace {

struct NoAllocScratch {
    double rows[TC_NOALLOC_ROWS * (TC_NOALLOC_MAX_NZ + 1)];
    double integ[32];
    double strain_max;
    int nempty_min, nempty_max, empty_cells, pad;
};

static __device__ __align__(256) NoAllocScratch tc_noalloc_scratch;

struct RefLayout {
    int nx, nz, ldT, ldU, ntype;
    __device__ __forceinline__ size_t t(int i, int k) const { return (size_t)(i + 2) + (size_t)(k + 2) * ldT; }
    __device__ __forceinline__ size_t u(int i, int k) const { return (size_t)(i + 1) + (size_t)(k + 1) * ldU; }
};

struct Consts {
    double dr, ds, RaT;
};

__global__ void k_na_rows(RefLayout R, Consts c, const double* __restrict__ T, const double* __restrict__ u,
                          const double* __restrict__ w, const double* __restrict__ cd,
                          const double* __restrict__ vis, const double* __restrict__ Cn, NoAllocScratch* S) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = R.nx, nz = R.nz;
    if (k > nz) return;
    auto f = [&](int q, int i) -> double {
        if (q < 4) return (q < R.ntype) ? Cn[(size_t)q + (size_t)R.ntype * R.t(i, k)] : 0.0;
        if (q == 4) { size_t x = R.u(i, k); return u[x] * u[x] + w[x] * w[x]; }
        size_t x = R.t(i, k);
        if (q == 5) return T[x];
        return c.RaT / cd[x] / vis[x];
    };
    for (int q = 0; q < TC_NOALLOC_ROWS; q++) {
        double fint = 0.0;
        bool active = !((q < 4 && q >= R.ntype) || (q >= 5 && c.RaT == 0.0));
        if (active) {
            double fprev = f(q, 0);
            for (int i = 0; i <= nx - 1; i++) {
                double fn = f(q, i + 1);
                fint = fint + 0.5 * (fprev * 1.0 + fn * 1.0) * c.dr;
                fprev = fn;
            }
        }
        S->rows[(size_t)q * (nz + 1) + k] = fint;
    }
}

__global__ void k_na_final(RefLayout R, Consts c, int kent, const double* __restrict__ T,
                           const double* __restrict__ u, const double* __restrict__ w,
                           const double* __restrict__ cd, NoAllocScratch* S) {
    const int nx = R.nx, nz = R.nz;
    const int t = threadIdx.x;
    const size_t ldT = (size_t)R.ldT;
    if (t < TC_NOALLOC_ROWS + 4) {
        int q = (t < TC_NOALLOC_ROWS) ? t : (t - TC_NOALLOC_ROWS);
        int k0 = (t < TC_NOALLOC_ROWS) ? 0 : kent;
        bool active = !(q < 4 && q >= R.ntype) && !(t >= TC_NOALLOC_ROWS && q >= 4);
        if (active) {
            const double* f = S->rows + (size_t)q * (nz + 1);
            double fint = 0.0;
            for (int k = k0; k <= nz - 1; k++) fint = fint + 0.5 * (f[k] * 1.0 + f[k + 1] * 1.0) * c.ds;
            int slot = (t < TC_NOALLOC_ROWS) ? ((q < 4) ? q : (q - 4 + 8)) : (4 + q);
            S->integ[slot] = fint;
        }
    } else if (t == 16) {
        double a = 0.0, b = 0.0, cc = 0.0, m = 0.0;
        auto top = [&](int i) { size_t x = R.u(i, nz); return u[x] * u[x] + w[x] * w[x]; };
        auto Tzs = [&](int i) { size_t x = R.t(i, nz); return (-0.5 * T[x - ldT] + 0.5 * T[x + ldT]) / c.ds / 1.0; };
        auto Tzb = [&](int i) { size_t x = R.t(i, 0); return (-0.5 * T[x - ldT] + 0.5 * T[x + ldT]) / c.ds / 1.0; };
        for (int i = 0; i <= nx - 1; i++) {
            m = m + 0.5 * (top(i) * 1.0 + top(i + 1) * 1.0) * c.dr;
            if (c.RaT != 0.0) {
                double ai = -cd[R.t(i, nz)] * Tzs(i), ai1 = -cd[R.t(i + 1, nz)] * Tzs(i + 1);
                a = a + 0.5 * (ai * 1.0 + ai1 * 1.0) * c.dr;
                double bi = T[R.t(i, 0)], bi1 = T[R.t(i + 1, 0)];
                b = b + 0.5 * (bi * 1.0 + bi1 * 1.0) * c.dr;
                double ci = -cd[R.t(i, 0)] * Tzb(i), ci1 = -cd[R.t(i + 1, 0)] * Tzb(i + 1);
                cc = cc + 0.5 * (ci * 1.0 + ci1 * 1.0) * c.dr;
            }
        }
        S->integ[11] = m;
        S->integ[12] = a;
        S->integ[13] = b;
        S->integ[14] = cc;
        if (c.RaT != 0.0) {
            auto dz = [&](int i, int kk) { size_t x = R.t(i, kk); return -0.5 * T[x - ldT] + 0.5 * T[x + ldT]; };
            S->integ[15] = -(cd[R.t(0, nz)] * dz(0, nz)) / c.ds / 1.0;
            S->integ[16] = -(cd[R.t(nx, nz)] * dz(nx, nz)) / c.ds / 1.0;
            S->integ[17] = -(cd[R.t(nx, 0)] * dz(nx, 0)) / c.ds / 1.0;
            S->integ[18] = -(cd[R.t(0, 0)] * dz(0, 0)) / c.ds / 1.0;
        }
        // strain-rate invariant on the top row (compute_strain_rate_invariant)
        double smax = -INFINITY;
        const size_t ldU = (size_t)R.ldU;
        for (int i = 0; i <= nx; i++) {
            size_t x = R.u(i, nz);
            double ur = (-0.5 * u[x - 1] + 0.5 * u[x + 1]) / c.dr;
            double us = (-0.5 * u[x - ldU] + 0.5 * u[x + ldU]) / c.ds;
            double wr = (-0.5 * w[x - 1] + 0.5 * w[x + 1]) / c.dr;
            double ws = (-0.5 * w[x - ldU] + 0.5 * w[x + ldU]) / c.ds;
            double qv = 0.5 * (2.0 * (ur * ur + ws * ws) + (us + wr) * (us + wr));
            smax = fmax(smax, sqrt(qv));
        }
        S->strain_max = smax;
    }
}

__global__ void k_na_nempty_init(NoAllocScratch* S) {
    S->nempty_min = 0x7fffffff;
    S->nempty_max = -0x7fffffff;
    S->empty_cells = 0;
}

__global__ void k_na_nempty(RefLayout R, const int* __restrict__ ne, NoAllocScratch* S) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    __shared__ int smin, smax, szero;
    if (threadIdx.x == 0) { smin = 0x7fffffff; smax = -0x7fffffff; szero = 0; }
    __syncthreads();
    if (i <= R.nx) {
        int v = ne[R.t(i, k)];
        atomicMin(&smin, v);
        atomicMax(&smax, v);
        if (v == 0) atomicAdd(&szero, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMin(&S->nempty_min, smin);
        atomicMax(&S->nempty_max, smax);
        atomicAdd(&S->empty_cells, szero);
    }
}

std::mutex g_na_mutex;
NoAllocScratch* g_na_ptr[256] = {};
void* g_na_ctx[256] = {};

// cuCtxGetCurrent from the driver, reached through the runtime so that the
// library needs no link against libcuda.
typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn g_ctx_get = nullptr;
bool g_ctx_get_tried = false;

// Device address of the fixed array on the current device: looked up on the
// first call per device (with that device current) and again whenever the
// device's current context differs from the one the address was found in.
cudaError_t na_scratch(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    // make the runtime bind the device's primary context before reading it
    e = cudaFree(nullptr);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_ctx_get_tried) {
        g_ctx_get_tried = true;
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get = (CtxGetCurrentFn)fn;
    }
    void* ctx = nullptr;
    if (g_ctx_get == nullptr || g_ctx_get(&ctx) != 0 || ctx == nullptr) {
        // no context identity available: look the address up on every call
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, tc_noalloc_scratch);
        if (e != cudaSuccess) return e;
        *out = (NoAllocScratch*)p;
        return cudaSuccess;
    }
    if (g_na_ptr[dev] == nullptr || g_na_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, tc_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_ptr[dev] = (NoAllocScratch*)p;
        g_na_ctx[dev] = ctx;
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

// One launch whose status is its own return code (the runtime's last-error
// state is left alone).
template <typename... A>
cudaError_t na_launch(void (*kern)(A...), dim3 grid, dim3 block, cudaStream_t st, A... args) {
    void* argv[] = {(void*)&args...};
    return cudaLaunchKernel((const void*)kern, grid, block, argv, 0, st);
}

}  // namespace

extern "C" tc_status tc_stats_noalloc(const double* T, const double* u, const double* w, const double* conduct,
                                      const double* vis, const double* Cnew, const int32_t* nempty, int32_t nx,
                                      int32_t nz, int32_t ntype, double aspect, double RaT, int32_t kent,
                                      const double* mass, tc_stats_row* row, void* stream) {
    if (!T || !u || !w || !conduct || !vis || !row || nx < 2 || nz < 2 || aspect <= 0.0) return TC_ERR_ARG;
    if (ntype < 0 || ntype > TC_MAX_TYPES || (ntype > 0 && (!Cnew || !nempty)) || kent < 0 || kent > nz)
        return TC_ERR_ARG;
    if (nz > TC_NOALLOC_MAX_NZ) return TC_ERR_TOO_LARGE;
    NoAllocScratch* S = nullptr;
    if (na_scratch(&S) != cudaSuccess) return TC_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    RefLayout R{nx, nz, nx + 5, nx + 3, ntype};
    Consts c{aspect / (double)nx, 1.0 / (double)nz, RaT};
    // the tracer-count statistics follow the reference's rule: computed when
    // comp = 1 or tracer = 1 (basics.f90:263-267), which the caller states by
    // passing nempty (required with compositional types, NULL otherwise)
    const bool counts = (nempty != nullptr);
    cudaError_t e = na_launch(k_na_rows, dim3((unsigned)((nz + 1 + 63) / 64)), dim3(64), st, R, c, T, u, w, conduct,
                              vis, Cnew, S);
    if (e == cudaSuccess) e = na_launch(k_na_final, dim3(1), dim3(32), st, R, c, kent, T, u, w, conduct, S);
    if (e == cudaSuccess && counts) e = na_launch(k_na_nempty_init, dim3(1), dim3(1), st, S);
    if (e == cudaSuccess && counts)
        e = na_launch(k_na_nempty, dim3((unsigned)((nx + 1 + 127) / 128), (unsigned)(nz + 1)), dim3(128), st, R,
                      nempty, S);
    if (e != cudaSuccess) return TC_ERR_CUDA;
    tc_note_launch(counts ? 4 : 2);
    double integ[32];
    double smax = 0.0;
    int ints[3] = {0, 0, 0};
    if (cudaMemcpyAsync(integ, S->integ, sizeof(integ), cudaMemcpyDeviceToHost, st) != cudaSuccess) return TC_ERR_CUDA;
    if (cudaMemcpyAsync(&smax, &S->strain_max, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TC_ERR_CUDA;
    if (cudaMemcpyAsync(ints, &S->nempty_min, sizeof(ints), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TC_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return TC_ERR_CUDA;
    std::memset(row, 0, sizeof(*row));
    // final divisions and roots exactly as stats (basics.f90:236-324)
    for (int t = 0; t < ntype; t++) row->Cavg[t] = integ[t] / aspect;
    for (int t = 0; t < ntype; t++) row->ent[t] = (mass && mass[t] != 0.0) ? integ[4 + t] / aspect / mass[t] : 0.0;
    if (counts) {
        row->tracer_min = ints[0];
        row->tracer_max = ints[1];
        row->empty_cells = ints[2];
    }
    row->vrms = std::pow(integ[8] / aspect, 0.5);
    row->mobility = std::pow(integ[11] / aspect, 0.5) / row->vrms;
    row->strain_max = smax;
    if (RaT != 0.0) {
        row->Tavg = integ[9] / aspect;
        row->RaT_avg = integ[10] / aspect;
        row->Nu = integ[12] / integ[13];
        row->Nu_bot = integ[14] / aspect;
        row->q1 = integ[15]; row->q2 = integ[16]; row->q3 = integ[17]; row->q4 = integ[18];
    }
    return TC_OK;
}
