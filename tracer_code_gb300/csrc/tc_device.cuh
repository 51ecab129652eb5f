// tc_device.cuh -- device helpers shared by the kernel files.
//
// All kernels are compiled with --fmad=false: plain a*b+c in this code is a
// rounded multiply followed by a rounded add, exactly as in the reference's
// x86-64 gfortran build, so the kernels that the tests compare bit-for-bit
// with the CPU restatement (velocities, Taylor interpolation, RK updates,
// histograms, smoothers) reproduce its rounding.  Where bit-equality is not
// required (the folded multigrid operator) fma() is written explicitly.
#pragma once

#include "tc_internal.h"

#include <math.h>

#define BX 32
#define BY 8

struct Range2 {
    int i0, i1, k0, k1;  // inclusive
};

inline dim3 grid_for(const Range2& r) {
    int ni = r.i1 - r.i0 + 1, nk = r.k1 - r.k0 + 1;
    if (ni < 1) ni = 1;
    if (nk < 1) nk = 1;
    return dim3((unsigned)((ni + BX - 1) / BX), (unsigned)((nk + BY - 1) / BY), 1);
}
inline int nblocks_of(const Range2& r) {
    dim3 g = grid_for(r);
    return (int)(g.x * g.y);
}

#define RANGE_IK(r)                                    \
    const int i = (r).i0 + (int)(blockIdx.x * BX + threadIdx.x); \
    const int k = (r).k0 + (int)(blockIdx.y * BY + threadIdx.y); \
    const bool inr = (i <= (r).i1) && (k <= (r).k1);

enum { RED_SUM = 0, RED_MIN = 1, RED_MAX = 2 };

__device__ __forceinline__ double red_apply(int op, double a, double b) {
    if (op == RED_SUM) return a + b;
    if (op == RED_MIN) return fmin(a, b);
    return fmax(a, b);
}
__device__ __forceinline__ double red_identity(int op) {
    if (op == RED_SUM) return 0.0;
    if (op == RED_MIN) return INFINITY;
    return -INFINITY;
}

// Block-level reduction of v (one value per thread, any 1-D/2-D block of at
// most 1024 threads) followed by a deterministic grid-level finish: each
// block stores its partial; the last block to arrive (counter) folds the
// partials in block order and writes *out, then re-arms the counter.
// Every thread of every block must call this exactly once.
__device__ __forceinline__ void reduce_to(int op, double v, double* part, unsigned int* count, double* out,
                                          double scale_div1 = 1.0, double scale_div2 = 1.0) {
    __shared__ double sh[32];
    __shared__ bool last;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nth = blockDim.x * blockDim.y;
    const int bid = blockIdx.x + blockIdx.y * gridDim.x;
    const int nb = gridDim.x * gridDim.y;
    for (int off = 16; off > 0; off >>= 1) v = red_apply(op, v, __shfl_down_sync(0xffffffffu, v, off));
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        double x = (tid < ((nth + 31) >> 5)) ? sh[tid] : red_identity(op);
        for (int off = 16; off > 0; off >>= 1) x = red_apply(op, x, __shfl_down_sync(0xffffffffu, x, off));
        if (tid == 0) {
            part[bid] = x;
            __threadfence();
            unsigned int t = atomicAdd(count, 1u);
            last = (t == (unsigned int)(nb - 1));
        }
    }
    __syncthreads();
    if (last) {
        __threadfence();
        if (tid < 32) {
            double x = red_identity(op);
            // lane-strided partial folds in fixed order, then a fixed tree
            for (int b = tid; b < nb; b += 32) x = red_apply(op, x, __ldcg(part + b));
            for (int off = 16; off > 0; off >>= 1) x = red_apply(op, x, __shfl_down_sync(0xffffffffu, x, off));
            if (tid == 0) {
                if (op == RED_SUM) x = x / scale_div1 / scale_div2;
                *out = x;
                *count = 0u;
            }
        }
    }
}

// Host-side count of kernels this library enqueues (tc_kernel_launches).
void tc_note_launch(long long n = 1);

struct CPtrs {
    const double* p[TC_MAX_TYPES];
};
struct CPtrsW {
    double* p[TC_MAX_TYPES];
};
