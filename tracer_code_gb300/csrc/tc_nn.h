// tc_nn.h -- internal interface of the learned initial guess (network kernels).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_device.cuh"

// input channels per K stage of a conv with `cin` input channels (a multiple of 16)
__host__ __device__ inline int conv_kc(int cin) { return cin % 64 == 0 ? 64 : (cin % 32 == 0 ? 32 : 16); }

// k_conv.cu: 3x3 conv of NHWC BF16 on tcgen05 (see the file header); 0 = launched
int conv3x3_launch(cudaStream_t s, const __nv_bfloat16* x, int nb, int H, int W, int cin_tot, int cin_off, int cin,
                   const __nv_bfloat16* wpack, const float* bias, int N, int relu, __nv_bfloat16* out, int cout_tot,
                   int cout_off, int cout_store, int* fail, const int* test_flag = nullptr);

// A channel window of an NHWC BF16 tensor: channels [off, off+c) of ctot.
struct View {
    __nv_bfloat16* p;
    int ctot, off, c;
};
