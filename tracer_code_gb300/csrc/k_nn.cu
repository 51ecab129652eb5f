// k_nn.cu -- the learned initial guess: a 4-level convolutional
// encoder-decoder (channels 32/64/128/128, two 3x3 convolutions per level,
// 2x2 average pooling, nearest upsampling, skip connections by channel
// concatenation, 1x1 output head), its training (forward, backward, Adam)
// and its use as the multigrid initial guess.
//
// Data: NHWC BF16 activations and weights, FP32 accumulation (tensor cores
// through k_conv.cu for every 3x3 forward convolution and for the
// backward-data convolutions, which are forward convolutions with flipped,
// transposed weights), FP32 master weights, gradients and Adam moments.
// Weight gradients are reductions over pixels on the CUDA cores with a
// deterministic two-pass sum (per-chunk partials, then a fixed-order sum).
//
// Input channels (per image, H = nz rows, W = nx columns of grid nodes
// i = 0..nx-1, k = 0..nz-1): log10 viscosity standardised per image, the
// streamfunction RHS divided by its RMS, and the previous streamfunction
// divided by its RMS s.  The target and the output are (SF_new - SF_prev)/s
// on the interior nodes, so the guess is SF_prev + s * output.
#include "nn_conv.cuh"
#include "tc_nn.h"

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

typedef __nv_bfloat16 bf16;

namespace {

// ---- layer table ---------------------------------------------------------------
struct ConvSpec {
    int cin, cout;  // real channels (the first layer's input is padded to 16 in the tensor)
    int lev;        // resolution level 0..3 (H >> lev)
};
const ConvSpec kConv[14] = {
    {3, 32, 0},    {32, 32, 0},    // enc0a, enc0b -> U0[64:96]
    {32, 64, 1},   {64, 64, 1},    // enc1a, enc1b -> U1[128:192]
    {64, 128, 2},  {128, 128, 2},  // enc2a, enc2b -> U2[128:256]
    {128, 128, 3}, {128, 128, 3},  // bottleneck
    {256, 128, 2}, {128, 128, 2},  // dec2a (U2), dec2b
    {192, 64, 1},  {64, 64, 1},    // dec1a (U1), dec1b
    {96, 32, 0},   {32, 32, 0},    // dec0a (U0), dec0b
};
const int kHeadC = 32;

inline int pad16(int c) { return (c + 15) / 16 * 16; }
inline int npow(int c) { return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : 256; }

// ---- weight packing --------------------------------------------------------------
// forward: wp[i = tap*nch + ch][j][co][e] = W[co][tap][ch*kc + j*8 + e]
__global__ void k_pack_fwd(const float* __restrict__ W, int cout, int cin, int cin_p, int N, bf16* __restrict__ wp) {
    const int kc = conv_kc(cin_p), nch = cin_p / kc;
    const size_t total = (size_t)9 * cin_p * N;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % 8);
        const int co = (int)((t / 8) % N);
        const size_t r = t / (8 * (size_t)N);  // (i, j)
        const int j = (int)(r % (kc / 8));
        const int i = (int)(r / (kc / 8));
        const int tap = i / nch, ch = i % nch;
        const int ci = ch * kc + j * 8 + e;
        const float v = (co < cout && ci < cin) ? W[((size_t)co * 9 + tap) * cin + ci] : 0.f;
        wp[t] = __float2bfloat16(v);
    }
}
// backward data: the forward kernel on dZ (cout channels) producing cin
// channels: wp[i = tap*nch + ch][j][ci][e] = W[co = ch*kc + j*8 + e][8 - tap][ci]
__global__ void k_pack_bwd(const float* __restrict__ W, int cout, int cin, int N, bf16* __restrict__ wp) {
    const int kc = conv_kc(cout), nch = cout / kc;
    const size_t total = (size_t)9 * cout * N;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % 8);
        const int ci = (int)((t / 8) % N);
        const size_t r = t / (8 * (size_t)N);
        const int j = (int)(r % (kc / 8));
        const int i = (int)(r / (kc / 8));
        const int tap = i / nch, ch = i % nch;
        const int co = ch * kc + j * 8 + e;
        const float v = (ci < cin) ? W[((size_t)co * 9 + (8 - tap)) * cin + ci] : 0.f;
        wp[t] = __float2bfloat16(v);
    }
}

// ---- elementwise ------------------------------------------------------------------
__device__ __forceinline__ float bf(const bf16 v) { return __bfloat162float(v); }

// dZ = dY * (Y > 0), dZ contiguous with c channels
__global__ void k_relu_mask(View dY, View Y, size_t npx, bf16* __restrict__ dZ) {
    const int c = dY.c;
    const size_t total = npx * c;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const size_t p = t / c;
        const int ch = (int)(t % c);
        const float y = bf(Y.p[p * Y.ctot + Y.off + ch]);
        dZ[t] = y > 0.f ? dY.p[p * dY.ctot + dY.off + ch] : __float2bfloat16(0.f);
    }
}
// out (half resolution) = 2x2 mean of in
__global__ void k_pool(View in, int nb, int H, int W, View out) {
    const int c = in.c, h = H / 2, w = W / 2;
    const size_t total = (size_t)nb * h * w * c;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(t % c);
        size_t q = t / c;
        const int x = (int)(q % w);
        q /= w;
        const int y = (int)(q % h);
        const int n = (int)(q / h);
        float s = 0.f;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                s += bf(in.p[(((size_t)n * H + 2 * y + a) * W + 2 * x + b) * in.ctot + in.off + ch]);
        out.p[(((size_t)n * h + y) * w + x) * out.ctot + out.off + ch] = __float2bfloat16(0.25f * s);
    }
}
// dIn (full resolution view) += dOut / 4 spread over each 2x2 block
__global__ void k_pool_bwd_add(View dout, int nb, int H, int W, View din) {
    const int c = din.c, h = H / 2, w = W / 2;
    const size_t total = (size_t)nb * H * W * c;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(t % c);
        size_t q = t / c;
        const int x = (int)(q % W);
        q /= W;
        const int y = (int)(q % H);
        const int n = (int)(q / H);
        bf16& d = din.p[(((size_t)n * H + y) * W + x) * din.ctot + din.off + ch];
        const float g = bf(dout.p[(((size_t)n * h + y / 2) * w + x / 2) * dout.ctot + dout.off + ch]);
        d = __float2bfloat16(bf(d) + 0.25f * g);
    }
}
// out (full resolution view) = nearest upsampling of in (half resolution)
// nearest upsampling, eight channels (16 bytes) per thread: channel counts,
// offsets and totals are multiples of 8
__global__ void k_up(View in, int nb, int H, int W, View out) {
    const int c8 = in.c / 8, h = H / 2, w = W / 2;
    const int total = nb * H * W * c8;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int ch = (t % c8) * 8;
        int q = t / c8;
        const int x = q % W;
        q /= W;
        const int y = q % H;
        const int n = q / H;
        *reinterpret_cast<uint4*>(out.p + (((size_t)n * H + y) * W + x) * out.ctot + out.off + ch) =
            *reinterpret_cast<const uint4*>(in.p + (((size_t)n * h + y / 2) * w + x / 2) * in.ctot + in.off + ch);
    }
}
// dIn (half resolution) = sum over each 2x2 block of dOut (full resolution view)
__global__ void k_up_bwd(View dout, int nb, int H, int W, View din) {
    const int c = din.c, h = H / 2, w = W / 2;
    const size_t total = (size_t)nb * h * w * c;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(t % c);
        size_t q = t / c;
        const int x = (int)(q % w);
        q /= w;
        const int y = (int)(q % h);
        const int n = (int)(q / h);
        float s = 0.f;
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++)
                s += bf(dout.p[(((size_t)n * H + 2 * y + a) * W + 2 * x + b) * dout.ctot + dout.off + ch]);
        din.p[(((size_t)n * h + y) * w + x) * din.ctot + din.off + ch] = __float2bfloat16(s);
    }
}

// ---- weight gradient of a 3x3 conv (CUDA cores, FP32) ------------------------------
// Block (chunk, co tile of 32, ci tile of CI): pixels of rows y0..y0+7, columns
// x0..x0+63 of one image; partial[chunk][co][tap][ci], bias partial[chunk][co].
template <int CI>
__global__ void __launch_bounds__(256) k_conv_dw(View X, const bf16* __restrict__ dZ, int nb, int H, int W, int cout,
                                                 int cin, float* __restrict__ pw, float* __restrict__ pb) {
    constexpr int PX = 64, RY = 8, CPT = CI / 8;
    __shared__ float Xs[3][PX + 2][CI];
    __shared__ float Zs[PX][32];
    const int tid = threadIdx.x, co_l = tid & 31, cg = tid >> 5;
    const int co0 = blockIdx.y * 32, ci0 = blockIdx.z * CI;
    const int cx = (W + PX - 1) / PX, cy = (H + RY - 1) / RY;
    int q = blockIdx.x;
    const int bxi = q % cx;
    q /= cx;
    const int byi = q % cy;
    const int n = q / cy;
    const int x0 = bxi * PX, y0 = byi * RY;
    float acc[9][CPT];
    float bacc = 0.f;
#pragma unroll
    for (int t = 0; t < 9; t++)
#pragma unroll
        for (int c = 0; c < CPT; c++) acc[t][c] = 0.f;
    for (int y = y0; y < y0 + RY && y < H; y++) {
        for (int e = tid; e < 3 * (PX + 2) * CI; e += 256) {
            const int c = e % CI, xx = (e / CI) % (PX + 2), r = e / (CI * (PX + 2));
            const int gy = y - 1 + r, gx = x0 - 1 + xx, ci = ci0 + c;
            float v = 0.f;
            if (gy >= 0 && gy < H && gx >= 0 && gx < W && ci < cin)
                v = bf(X.p[(((size_t)n * H + gy) * W + gx) * X.ctot + X.off + ci]);
            Xs[r][xx][c] = v;
        }
        for (int e = tid; e < PX * 32; e += 256) {
            const int c = e % 32, xx = e / 32, gx = x0 + xx, co = co0 + c;
            float v = 0.f;
            if (gx < W && co < cout) v = bf(dZ[(((size_t)n * H + y) * W + gx) * cout + co]);
            Zs[xx][c] = v;
        }
        __syncthreads();
        for (int px = 0; px < PX; px++) {
            const float z = Zs[px][co_l];
            bacc += z;
#pragma unroll
            for (int t = 0; t < 9; t++) {
                const float* xr = &Xs[t / 3][px + t % 3][cg * CPT];
#pragma unroll
                for (int c = 0; c < CPT; c++) acc[t][c] = fmaf(z, xr[c], acc[t][c]);
            }
        }
        __syncthreads();
    }
    const int co = co0 + co_l;
    if (co < cout) {
        float* dst = pw + (size_t)blockIdx.x * cout * 9 * cin;
#pragma unroll
        for (int t = 0; t < 9; t++)
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                const int ci = ci0 + cg * CPT + c;
                if (ci < cin) dst[((size_t)co * 9 + t) * cin + ci] = acc[t][c];
            }
        if (blockIdx.z == 0 && cg == 0) pb[(size_t)blockIdx.x * cout + co] = bacc;
    }
}
// out[j] = sum_k part[k][j] in fixed order
__global__ void k_reduce_parts(const float* __restrict__ part, int nparts, size_t len, float* __restrict__ out) {
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < len; j += (size_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < nparts; k++) s += part[(size_t)k * len + j];
        out[j] = s;
    }
}

// ---- head, loss, optimiser ---------------------------------------------------------
// out[p] = b + sum_c w[c] * D[p][c]
__global__ void k_head(const bf16* __restrict__ D, const float* __restrict__ wb, size_t npx, float* __restrict__ out) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x) {
        float s = wb[kHeadC];
        for (int c = 0; c < kHeadC; c++) s = fmaf(wb[c], bf(D[p * kHeadC + c]), s);
        out[p] = s;
    }
}
// dD[p][c] = dout[p] * w[c]; per-block partials of dw (32) and db (1)
__global__ void __launch_bounds__(256) k_head_bwd(const bf16* __restrict__ D, const float* __restrict__ wb,
                                                  const float* __restrict__ dout, size_t npx, bf16* __restrict__ dD,
                                                  float* __restrict__ part) {
    __shared__ float red[8][kHeadC + 1];
    float acc[kHeadC + 1];
    for (int c = 0; c <= kHeadC; c++) acc[c] = 0.f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x) {
        const float g = dout[p];
        for (int c = 0; c < kHeadC; c++) {
            dD[p * kHeadC + c] = __float2bfloat16(g * wb[c]);
            acc[c] = fmaf(g, bf(D[p * kHeadC + c]), acc[c]);
        }
        acc[kHeadC] += g;
    }
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int c = 0; c <= kHeadC; c++) {
        float v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x <= kHeadC) {
        float v = 0.f;
        for (int w = 0; w < 8; w++) v += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * (kHeadC + 1) + threadIdx.x] = v;
    }
}
// masked MSE over interior nodes (x >= 1, y >= 1): per-block partial sums and dout
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ out, const float* __restrict__ tgt, int nb,
                                              int H, int W, float inv_count, float* __restrict__ dout,
                                              float* __restrict__ part) {
    __shared__ float red[8];
    float s = 0.f;
    const size_t npx = (size_t)nb * H * W;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % W), y = (int)((p / W) % H);
        float g = 0.f;
        if (x >= 1 && y >= 1) {
            const float d = out[p] - tgt[p];
            s = fmaf(d, d, s);
            g = 2.f * d * inv_count;
        }
        dout[p] = g;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float v = 0.f;
        for (int w = 0; w < 8; w++) v += red[w];
        part[blockIdx.x] = v * inv_count;
    }
}
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
        const float gj = g[j];
        const float mj = b1 * m[j] + (1.f - b1) * gj;
        const float vj = b2 * v[j] + (1.f - b2) * gj * gj;
        m[j] = mj;
        v[j] = vj;
        p[j] -= lr * (mj / c1) / (sqrtf(vj / c2) + eps);
    }
}

// ---- inputs ---------------------------------------------------------------------------
// per-image statistics of the three raw channels (raw[n][3][H][W]):
// st[n] = {mean c0, std c0, rms c1, rms c2}.  kStatParts blocks per image
// write FP64 partial sums; one warp per image folds them in block order.
constexpr int kStatParts = 64;
__global__ void __launch_bounds__(256) k_stats_part(const float* __restrict__ raw, int H, int W,
                                                    double* __restrict__ part) {
    __shared__ double red[8][4];
    const int n = blockIdx.y, b = blockIdx.x;
    const size_t hw = (size_t)H * W;
    const float* r = raw + (size_t)n * 3 * hw;
    double s0 = 0, q0 = 0, q1 = 0, q2 = 0;
    for (size_t p = (size_t)b * blockDim.x + threadIdx.x; p < hw; p += (size_t)kStatParts * blockDim.x) {
        const double a = r[p], bb = r[hw + p], c = r[2 * hw + p];
        s0 += a;
        q0 += a * a;
        q1 += bb * bb;
        q2 += c * c;
    }
    double v[4] = {s0, q0, q1, q2};
    for (int k = 0; k < 4; k++) {
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0;
        for (int w = 0; w < 8; w++) t += red[w][threadIdx.x];
        part[((size_t)n * kStatParts + b) * 4 + threadIdx.x] = t;
    }
}
__global__ void k_stats_fin(const double* __restrict__ part, int H, int W, float* __restrict__ st) {
    const int n = blockIdx.x, lane = threadIdx.x;
    const double hw = (double)H * W;
    double t[4];
    for (int k = 0; k < 4; k++) {
        double v = 0;
        for (int b = lane; b < kStatParts; b += 32) v += part[((size_t)n * kStatParts + b) * 4 + k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        t[k] = v;
    }
    if (lane == 0) {
        const double mean = t[0] / hw, var = t[1] / hw - mean * mean;
        st[4 * n + 0] = (float)mean;
        st[4 * n + 1] = (float)sqrt(var > 1e-12 ? var : 1e-12);
        st[4 * n + 2] = (float)sqrt(t[2] / hw > 1e-60 ? t[2] / hw : 1e-60);
        st[4 * n + 3] = (float)sqrt(t[3] / hw > 1e-60 ? t[3] / hw : 1e-60);
    }
}
// x16[n][y][x][16] = normalised channels, zero padded to 16
__global__ void k_input(const float* __restrict__ raw, const float* __restrict__ st, int nb, int H, int W,
                        bf16* __restrict__ x16) {
    const size_t hw = (size_t)H * W, total = (size_t)nb * hw;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(t / hw);
        const size_t p = t % hw;
        const float* r = raw + (size_t)n * 3 * hw;
        const float* s = st + 4 * n;
        __align__(16) bf16 v[16];
        for (int c = 0; c < 16; c++) v[c] = __float2bfloat16(0.f);
        v[0] = __float2bfloat16((r[p] - s[0]) / s[1]);
        v[1] = __float2bfloat16(r[hw + p] / s[2]);
        v[2] = __float2bfloat16(r[2 * hw + p] / s[3]);
        uint4* d = reinterpret_cast<uint4*>(x16 + t * 16);
        d[0] = reinterpret_cast<const uint4*>(v)[0];
        d[1] = reinterpret_cast<const uint4*>(v)[1];
    }
}
// target[n][p] = (sf_new - sf_prev) / rms(sf_prev)
__global__ void k_target(const float* __restrict__ raw, const float* __restrict__ sf_new, const float* __restrict__ st,
                         int nb, int H, int W, float* __restrict__ tgt) {
    const size_t hw = (size_t)H * W, total = (size_t)nb * hw;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(t / hw);
        const size_t p = t % hw;
        tgt[t] = (sf_new[t] - raw[(size_t)n * 3 * hw + 2 * hw + p]) / st[4 * n + 3];
    }
}

inline unsigned nblk(size_t n, int per = 256) {
    size_t b = (n + per - 1) / per;
    if (b > 4096) b = 4096;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace

// ---- the network object -------------------------------------------------------------------
struct tc_net_impl {
    int nbmax = 0, H = 0, W = 0;
    cudaStream_t st = nullptr;
    // parameters: per conv layer W[cout][9][cin] then b[cout]; head w[32], b
    std::vector<size_t> woff, boff;
    size_t head_off = 0, nparam = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    int adam_t = 0;
    bf16* wpf[14] = {};
    bf16* wpb[14] = {};
    // activations (bf16 NHWC) and gradients
    bf16 *x16 = nullptr, *A0 = nullptr, *U0 = nullptr, *P0 = nullptr, *A1 = nullptr, *U1 = nullptr, *P1 = nullptr,
         *A2 = nullptr, *U2 = nullptr, *P2 = nullptr, *A3 = nullptr, *B3 = nullptr, *D2a = nullptr, *D2b = nullptr,
         *D1a = nullptr, *D1b = nullptr, *D0a = nullptr, *D0b = nullptr;
    bf16 *dA0 = nullptr, *dU0 = nullptr, *dP0 = nullptr, *dA1 = nullptr, *dU1 = nullptr, *dP1 = nullptr,
         *dA2 = nullptr, *dU2 = nullptr, *dP2 = nullptr, *dA3 = nullptr, *dB3 = nullptr, *dD2a = nullptr,
         *dD2b = nullptr, *dD1a = nullptr, *dD1b = nullptr, *dD0a = nullptr, *dD0b = nullptr, *dZ = nullptr;
    float *out = nullptr, *dout = nullptr, *tgt = nullptr, *stats = nullptr, *part = nullptr, *lossp = nullptr;
    double* statp = nullptr;   // per-block partial sums of the input statistics
    size_t part_len = 0;
    int* fail = nullptr;
    int* never = nullptr;      // a word that stays 0 (timeout-path test)
    bool wait_test = false;    // tcnn_debug_wait_test: convs wait on `never` first
    std::vector<void*> allocs;
    std::string err;
};

namespace {

template <class T>
bool nalloc(tc_net_impl* n, T** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T) + 64) != cudaSuccess) return false;
    cudaMemset(q, 0, count * sizeof(T) + 64);
    n->allocs.push_back(q);
    *p = (T*)q;
    return true;
}

size_t px_at(const tc_net_impl* n, int lev, int nb) { return (size_t)nb * (n->H >> lev) * (n->W >> lev); }

View V(bf16* p, int ctot, int off, int c) { return View{p, ctot, off, c}; }

// one 3x3 conv layer forward: input view -> output view, bias + ReLU
int conv_fwd(tc_net_impl* n, int l, int nb, View in, View out) {
    const ConvSpec& s = kConv[l];
    const int H = n->H >> s.lev, W = n->W >> s.lev;
    const int cin_p = (l == 0) ? 16 : s.cin;
    return conv3x3_launch(n->st, in.p, nb, H, W, in.ctot, in.off, cin_p, n->wpf[l], n->p + n->boff[l], npow(s.cout),
                          1, out.p, out.ctot, out.off, s.cout, n->fail, n->wait_test ? n->never : nullptr);
}

// backward of layer l given dY (view, same shape as its output) and Y:
// weight/bias gradients into n->g, and (unless l == 0) dX into view dX
int conv_bwd(tc_net_impl* n, int l, int nb, View X, View Y, View dY, View dX) {
    const ConvSpec& s = kConv[l];
    const int H = n->H >> s.lev, W = n->W >> s.lev;
    const size_t npx = (size_t)nb * H * W;
    k_relu_mask<<<nblk(npx * s.cout), 256, 0, n->st>>>(dY, Y, npx, n->dZ); tc_note_launch();
    const int cx = (W + 63) / 64, cy = (H + 7) / 8, nchunk = nb * cx * cy;
    const int CI = (s.cin <= 16) ? 16 : 32;
    dim3 grid((unsigned)nchunk, (unsigned)(s.cout / 32), (unsigned)((s.cin + CI - 1) / CI));
    float* pw = n->part;
    float* pb = n->part + (size_t)nchunk * s.cout * 9 * s.cin;
    if ((size_t)nchunk * (s.cout * 9 * s.cin + s.cout) > n->part_len) return 10;
    if (CI == 16) k_conv_dw<16><<<grid, 256, 0, n->st>>>(X, n->dZ, nb, H, W, s.cout, s.cin, pw, pb);
    else k_conv_dw<32><<<grid, 256, 0, n->st>>>(X, n->dZ, nb, H, W, s.cout, s.cin, pw, pb);
    tc_note_launch();
    const size_t lw = (size_t)s.cout * 9 * s.cin;
    k_reduce_parts<<<nblk(lw), 256, 0, n->st>>>(pw, nchunk, lw, n->g + n->woff[l]); tc_note_launch();
    k_reduce_parts<<<nblk(s.cout), 256, 0, n->st>>>(pb, nchunk, (size_t)s.cout, n->g + n->boff[l]); tc_note_launch();
    if (l == 0) return 0;
    return conv3x3_launch(n->st, n->dZ, nb, H, W, s.cout, 0, s.cout, n->wpb[l], nullptr, npow(s.cin), 0, dX.p,
                          dX.ctot, dX.off, s.cin, n->fail, n->wait_test ? n->never : nullptr);
}

void pack_all(tc_net_impl* n) {
    for (int l = 0; l < 14; l++) {
        const ConvSpec& s = kConv[l];
        const int cin_p = (l == 0) ? 16 : s.cin;
        k_pack_fwd<<<nblk((size_t)9 * cin_p * npow(s.cout)), 256, 0, n->st>>>(n->p + n->woff[l], s.cout, s.cin, cin_p,
                                                                               npow(s.cout), n->wpf[l]);
        tc_note_launch();
        if (l > 0) {
            k_pack_bwd<<<nblk((size_t)9 * s.cout * npow(s.cin)), 256, 0, n->st>>>(n->p + n->woff[l], s.cout, s.cin,
                                                                                   npow(s.cin), n->wpb[l]);
            tc_note_launch();
        }
    }
}

}  // namespace

int net_forward(tc_net_impl* n, int nb) {
    const int H = n->H, W = n->W;
    int r = 0;
    // the failure flag reports this pass (and a backward pass that follows it)
    if (cudaMemsetAsync(n->fail, 0, sizeof(int), n->st) != cudaSuccess) return 1;
    r |= conv_fwd(n, 0, nb, V(n->x16, 16, 0, 16), V(n->A0, 32, 0, 32));
    r |= conv_fwd(n, 1, nb, V(n->A0, 32, 0, 32), V(n->U0, 96, 64, 32));
    k_pool<<<nblk(px_at(n, 1, nb) * 32), 256, 0, n->st>>>(V(n->U0, 96, 64, 32), nb, H, W, V(n->P0, 32, 0, 32));
    r |= conv_fwd(n, 2, nb, V(n->P0, 32, 0, 32), V(n->A1, 64, 0, 64));
    r |= conv_fwd(n, 3, nb, V(n->A1, 64, 0, 64), V(n->U1, 192, 128, 64));
    k_pool<<<nblk(px_at(n, 2, nb) * 64), 256, 0, n->st>>>(V(n->U1, 192, 128, 64), nb, H / 2, W / 2,
                                                          V(n->P1, 64, 0, 64));
    r |= conv_fwd(n, 4, nb, V(n->P1, 64, 0, 64), V(n->A2, 128, 0, 128));
    r |= conv_fwd(n, 5, nb, V(n->A2, 128, 0, 128), V(n->U2, 256, 128, 128));
    k_pool<<<nblk(px_at(n, 3, nb) * 128), 256, 0, n->st>>>(V(n->U2, 256, 128, 128), nb, H / 4, W / 4,
                                                           V(n->P2, 128, 0, 128));
    r |= conv_fwd(n, 6, nb, V(n->P2, 128, 0, 128), V(n->A3, 128, 0, 128));
    r |= conv_fwd(n, 7, nb, V(n->A3, 128, 0, 128), V(n->B3, 128, 0, 128));
    k_up<<<nblk(px_at(n, 2, nb) * 16), 256, 0, n->st>>>(V(n->B3, 128, 0, 128), nb, H / 4, W / 4,
                                                         V(n->U2, 256, 0, 128));
    r |= conv_fwd(n, 8, nb, V(n->U2, 256, 0, 256), V(n->D2a, 128, 0, 128));
    r |= conv_fwd(n, 9, nb, V(n->D2a, 128, 0, 128), V(n->D2b, 128, 0, 128));
    k_up<<<nblk(px_at(n, 1, nb) * 16), 256, 0, n->st>>>(V(n->D2b, 128, 0, 128), nb, H / 2, W / 2,
                                                         V(n->U1, 192, 0, 128));
    r |= conv_fwd(n, 10, nb, V(n->U1, 192, 0, 192), V(n->D1a, 64, 0, 64));
    r |= conv_fwd(n, 11, nb, V(n->D1a, 64, 0, 64), V(n->D1b, 64, 0, 64));
    k_up<<<nblk(px_at(n, 0, nb) * 8), 256, 0, n->st>>>(V(n->D1b, 64, 0, 64), nb, H, W, V(n->U0, 96, 0, 64));
    r |= conv_fwd(n, 12, nb, V(n->U0, 96, 0, 96), V(n->D0a, 32, 0, 32));
    r |= conv_fwd(n, 13, nb, V(n->D0a, 32, 0, 32), V(n->D0b, 32, 0, 32));
    k_head<<<nblk(px_at(n, 0, nb)), 256, 0, n->st>>>(n->D0b, n->p + n->head_off, px_at(n, 0, nb), n->out);
    tc_note_launch(7);  // pools, upsamplings, head
    return r;
}

int net_backward(tc_net_impl* n, int nb) {
    const int H = n->H, W = n->W;
    int r = 0;
    const size_t np0 = px_at(n, 0, nb);
    const unsigned hb = nblk(np0, 256) > 512 ? 512 : nblk(np0, 256);
    k_head_bwd<<<hb, 256, 0, n->st>>>(n->D0b, n->p + n->head_off, n->dout, np0, n->dD0b, n->part);
    k_reduce_parts<<<1, 64, 0, n->st>>>(n->part, (int)hb, (size_t)(kHeadC + 1), n->g + n->head_off);
    tc_note_launch(2);
    r |= conv_bwd(n, 13, nb, V(n->D0a, 32, 0, 32), V(n->D0b, 32, 0, 32), V(n->dD0b, 32, 0, 32), V(n->dD0a, 32, 0, 32));
    r |= conv_bwd(n, 12, nb, V(n->U0, 96, 0, 96), V(n->D0a, 32, 0, 32), V(n->dD0a, 32, 0, 32), V(n->dU0, 96, 0, 96));
    k_up_bwd<<<nblk(px_at(n, 1, nb) * 64), 256, 0, n->st>>>(V(n->dU0, 96, 0, 64), nb, H, W, V(n->dD1b, 64, 0, 64));
    r |= conv_bwd(n, 11, nb, V(n->D1a, 64, 0, 64), V(n->D1b, 64, 0, 64), V(n->dD1b, 64, 0, 64), V(n->dD1a, 64, 0, 64));
    r |= conv_bwd(n, 10, nb, V(n->U1, 192, 0, 192), V(n->D1a, 64, 0, 64), V(n->dD1a, 64, 0, 64),
                  V(n->dU1, 192, 0, 192));
    k_up_bwd<<<nblk(px_at(n, 2, nb) * 128), 256, 0, n->st>>>(V(n->dU1, 192, 0, 128), nb, H / 2, W / 2,
                                                             V(n->dD2b, 128, 0, 128));
    r |= conv_bwd(n, 9, nb, V(n->D2a, 128, 0, 128), V(n->D2b, 128, 0, 128), V(n->dD2b, 128, 0, 128),
                  V(n->dD2a, 128, 0, 128));
    r |= conv_bwd(n, 8, nb, V(n->U2, 256, 0, 256), V(n->D2a, 128, 0, 128), V(n->dD2a, 128, 0, 128),
                  V(n->dU2, 256, 0, 256));
    k_up_bwd<<<nblk(px_at(n, 3, nb) * 128), 256, 0, n->st>>>(V(n->dU2, 256, 0, 128), nb, H / 4, W / 4,
                                                             V(n->dB3, 128, 0, 128));
    r |= conv_bwd(n, 7, nb, V(n->A3, 128, 0, 128), V(n->B3, 128, 0, 128), V(n->dB3, 128, 0, 128),
                  V(n->dA3, 128, 0, 128));
    r |= conv_bwd(n, 6, nb, V(n->P2, 128, 0, 128), V(n->A3, 128, 0, 128), V(n->dA3, 128, 0, 128),
                  V(n->dP2, 128, 0, 128));
    k_pool_bwd_add<<<nblk(px_at(n, 2, nb) * 128), 256, 0, n->st>>>(V(n->dP2, 128, 0, 128), nb, H / 4, W / 4,
                                                                   V(n->dU2, 256, 128, 128));
    r |= conv_bwd(n, 5, nb, V(n->A2, 128, 0, 128), V(n->U2, 256, 128, 128), V(n->dU2, 256, 128, 128),
                  V(n->dA2, 128, 0, 128));
    r |= conv_bwd(n, 4, nb, V(n->P1, 64, 0, 64), V(n->A2, 128, 0, 128), V(n->dA2, 128, 0, 128), V(n->dP1, 64, 0, 64));
    k_pool_bwd_add<<<nblk(px_at(n, 1, nb) * 64), 256, 0, n->st>>>(V(n->dP1, 64, 0, 64), nb, H / 2, W / 2,
                                                                  V(n->dU1, 192, 128, 64));
    r |= conv_bwd(n, 3, nb, V(n->A1, 64, 0, 64), V(n->U1, 192, 128, 64), V(n->dU1, 192, 128, 64),
                  V(n->dA1, 64, 0, 64));
    r |= conv_bwd(n, 2, nb, V(n->P0, 32, 0, 32), V(n->A1, 64, 0, 64), V(n->dA1, 64, 0, 64), V(n->dP0, 32, 0, 32));
    k_pool_bwd_add<<<nblk(px_at(n, 0, nb) * 32), 256, 0, n->st>>>(V(n->dP0, 32, 0, 32), nb, H, W,
                                                                  V(n->dU0, 96, 64, 32));
    r |= conv_bwd(n, 1, nb, V(n->A0, 32, 0, 32), V(n->U0, 96, 64, 32), V(n->dU0, 96, 64, 32), V(n->dA0, 32, 0, 32));
    r |= conv_bwd(n, 0, nb, V(n->x16, 16, 0, 16), V(n->A0, 32, 0, 32), V(n->dA0, 32, 0, 32), V(n->dA0, 32, 0, 32));
    tc_note_launch(6);
    return r;
}

int net_create(tc_net_impl* n, int nbmax, int H, int W, uint64_t seed) {
    if (nbmax < 1 || H % 16 || W % 16 || H < 16 || W < 16) return 1;
    // every level must tile into 128-pixel blocks of bx x by pixels (k_conv.cu)
    for (int lev = 0; lev < 4; lev++) {
        const int h = H >> lev, w = W >> lev, bx = w < 128 ? w : 128;
        if (128 % bx || w % bx || h % (128 / bx)) return 1;
    }
    n->nbmax = nbmax;
    n->H = H;
    n->W = W;
    size_t off = 0;
    for (int l = 0; l < 14; l++) {
        n->woff.push_back(off);
        off += (size_t)kConv[l].cout * 9 * kConv[l].cin;
        n->boff.push_back(off);
        off += kConv[l].cout;
    }
    n->head_off = off;
    off += kHeadC + 1;
    n->nparam = off;
    if (!nalloc(n, &n->p, off) || !nalloc(n, &n->g, off) || !nalloc(n, &n->m, off) || !nalloc(n, &n->v, off))
        return 2;
    // He-normal initial weights, zero biases
    std::vector<float> h(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < 14; l++) {
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (9.0 * kConv[l].cin)));
        for (size_t j = 0; j < (size_t)kConv[l].cout * 9 * kConv[l].cin; j++) h[n->woff[l] + j] = (float)nd(rng);
    }
    {
        std::normal_distribution<double> nd(0.0, 0.1 * std::sqrt(1.0 / kHeadC));
        for (int c = 0; c < kHeadC; c++) h[n->head_off + c] = (float)nd(rng);
    }
    cudaMemcpy(n->p, h.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    for (int l = 0; l < 14; l++) {
        const int cin_p = (l == 0) ? 16 : kConv[l].cin;
        if (!nalloc(n, &n->wpf[l], (size_t)9 * cin_p * npow(kConv[l].cout))) return 2;
        if (l > 0 && !nalloc(n, &n->wpb[l], (size_t)9 * kConv[l].cout * npow(kConv[l].cin))) return 2;
    }
    const size_t p0 = (size_t)nbmax * H * W, p1 = p0 / 4, p2 = p0 / 16, p3 = p0 / 64;
    struct B { bf16** a; bf16** d; size_t n; };
    B bufs[] = {{&n->A0, &n->dA0, p0 * 32},   {&n->U0, &n->dU0, p0 * 96},   {&n->P0, &n->dP0, p1 * 32},
                {&n->A1, &n->dA1, p1 * 64},   {&n->U1, &n->dU1, p1 * 192},  {&n->P1, &n->dP1, p2 * 64},
                {&n->A2, &n->dA2, p2 * 128},  {&n->U2, &n->dU2, p2 * 256},  {&n->P2, &n->dP2, p3 * 128},
                {&n->A3, &n->dA3, p3 * 128},  {&n->B3, &n->dB3, p3 * 128},  {&n->D2a, &n->dD2a, p2 * 128},
                {&n->D2b, &n->dD2b, p2 * 128}, {&n->D1a, &n->dD1a, p1 * 64}, {&n->D1b, &n->dD1b, p1 * 64},
                {&n->D0a, &n->dD0a, p0 * 32}, {&n->D0b, &n->dD0b, p0 * 32}};
    for (B& b : bufs)
        if (!nalloc(n, b.a, b.n) || !nalloc(n, b.d, b.n)) return 2;
    if (!nalloc(n, &n->x16, p0 * 16) || !nalloc(n, &n->dZ, p0 * 32)) return 2;
    if (!nalloc(n, &n->out, p0) || !nalloc(n, &n->dout, p0) || !nalloc(n, &n->tgt, p0) ||
        !nalloc(n, &n->stats, (size_t)4 * nbmax) || !nalloc(n, &n->statp, (size_t)4 * kStatParts * nbmax) ||
        !nalloc(n, &n->lossp, 4096) || !nalloc(n, &n->fail, 4) ||
        !nalloc(n, &n->never, 4))
        return 2;
    // weight-gradient partials: the largest chunks * (cout*9*cin + cout) over layers
    size_t mx = 0;
    for (int l = 0; l < 14; l++) {
        const int h = H >> kConv[l].lev, w = W >> kConv[l].lev;
        const size_t ch = (size_t)nbmax * ((w + 63) / 64) * ((h + 7) / 8);
        const size_t need = ch * ((size_t)kConv[l].cout * 9 * kConv[l].cin + kConv[l].cout);
        if (need > mx) mx = need;
    }
    mx = mx > (size_t)4096 * (kHeadC + 1) ? mx : (size_t)4096 * (kHeadC + 1);
    n->part_len = mx;
    if (!nalloc(n, &n->part, mx)) return 2;
    pack_all(n);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 3;
}

void net_prepare(tc_net_impl* n, const float* raw, int nb) {
    k_stats_part<<<dim3(kStatParts, nb), 256, 0, n->st>>>(raw, n->H, n->W, n->statp);
    k_stats_fin<<<nb, 32, 0, n->st>>>(n->statp, n->H, n->W, n->stats);
    k_input<<<nblk((size_t)nb * n->H * n->W), 256, 0, n->st>>>(raw, n->stats, nb, n->H, n->W, n->x16);
    tc_note_launch(3);
}

int net_loss(tc_net_impl* n, const float* raw, const float* sf_new, int nb, float* loss_host) {
    k_target<<<nblk((size_t)nb * n->H * n->W), 256, 0, n->st>>>(raw, sf_new, n->stats, nb, n->H, n->W, n->tgt);
    const float inv = 1.f / ((float)nb * (n->H - 1) * (n->W - 1));
    const unsigned nbk = 1024;
    k_loss<<<nbk, 256, 0, n->st>>>(n->out, n->tgt, nb, n->H, n->W, inv, n->dout, n->lossp);
    k_reduce_parts<<<1, 32, 0, n->st>>>(n->lossp, (int)nbk, 1, n->lossp + 2048);
    tc_note_launch(3);
    if (loss_host) {
        if (cudaMemcpyAsync(loss_host, n->lossp + 2048, sizeof(float), cudaMemcpyDeviceToHost, n->st) != cudaSuccess)
            return 1;
        if (cudaStreamSynchronize(n->st) != cudaSuccess) return 1;
    }
    return 0;
}

void net_adam(tc_net_impl* n, float lr, float b1, float b2, float eps) {
    n->adam_t++;
    const float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
    k_adam<<<nblk(n->nparam), 256, 0, n->st>>>(n->p, n->g, n->m, n->v, n->nparam, lr, b1, b2, eps, c1, c2);
    tc_note_launch();
    pack_all(n);
}

void net_destroy(tc_net_impl* n) {
    for (void* q : n->allocs) cudaFree(q);
    n->allocs.clear();
}

// ---- solver side: fields <-> network images ---------------------------------------------
namespace {
// raw[3][nz][nx] from the level-1 FP64 fields (image row k, column i)
__global__ void k_fields_to_raw(Lay L, const double* __restrict__ vis, const double* __restrict__ rhs,
                                const double* __restrict__ SF, float* __restrict__ raw) {
    const int W = L.a, H = L.b;
    const size_t hw = (size_t)H * W;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < hw; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % W), k = (int)(t / W);
        const size_t x = IX(L, i, k);
        const double v = vis[x];
        raw[t] = (float)log10(v > 1e-300 ? v : 1e-300);
        raw[hw + t] = (float)rhs[x];
        raw[2 * hw + t] = (float)SF[x];
    }
}
__global__ void k_field_to_img(Lay L, const double* __restrict__ S, float* __restrict__ img) {
    const int W = L.a, H = L.b;
    const size_t hw = (size_t)H * W;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < hw; t += (size_t)gridDim.x * blockDim.x)
        img[t] = (float)S[IX(L, (int)(t % W), (int)(t / W))];
}
// guess = SF + s * out on the interior nodes, with the stream BCs' ghosts
__global__ void k_guess(Lay L, const double* __restrict__ SF, const float* __restrict__ out,
                        const float* __restrict__ st, double* __restrict__ G, int Vbc) {
    const int W = L.a, H = L.b;
    const double s = st[3];
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)H * W;
         t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % W), k = (int)(t / W);
        if (i < 1 || k < 1) continue;
        store_stream<double>(L, G, i, k, SF[IX(L, i, k)] + s * (double)out[t], Vbc);
    }
}
}  // namespace

void nn_fields_to_raw(cudaStream_t s, const Lay& L, const double* vis, const double* rhs, const double* SF,
                      float* raw) {
    k_fields_to_raw<<<nblk((size_t)L.a * L.b), 256, 0, s>>>(L, vis, rhs, SF, raw); tc_note_launch();
}
void nn_field_to_img(cudaStream_t s, const Lay& L, const double* S, float* img) {
    k_field_to_img<<<nblk((size_t)L.a * L.b), 256, 0, s>>>(L, S, img); tc_note_launch();
}
namespace {
// one pass of the separable (1,2,1)/4 x (1,2,1)/4 filter on the interior
// nodes of an H x W image (boundary nodes i = 0, k = 0 and the absent
// i = W, k = H count as zero)
__global__ void k_binomial(const float* __restrict__ in, int H, int W, float* __restrict__ out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)H * W;
         t += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(t % W), y = (int)(t / W);
        if (x < 1 || y < 1) { out[t] = 0.f; continue; }
        auto v = [&](int yy, int xx) { return (xx < 1 || yy < 1 || xx >= W || yy >= H) ? 0.f : in[(size_t)yy * W + xx]; };
        float s = 0.f;
        const float w[3] = {0.25f, 0.5f, 0.25f};
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++) s += w[a + 1] * w[b + 1] * v(y + a, x + b);
        out[t] = s;
    }
}
}  // namespace

// network guess from the level-1 fields into G (a zeroed plane: walls stay 0)
int nn_guess(tc_net_impl* n, cudaStream_t s, const Lay& L, const double* vis, const double* rhs, const double* SF,
             float* raw, double* G, int Vbc, int smooth) {
    if (n->H != L.b || n->W != L.a) return 1;
    cudaStream_t keep = n->st;
    n->st = s;
    nn_fields_to_raw(s, L, vis, rhs, SF, raw);
    net_prepare(n, raw, 1);
    const int r = net_forward(n, 1);
    float* o = n->out;
    for (int f = 0; f < smooth; f++) {
        float* dst = (o == n->out) ? n->dout : n->out;
        k_binomial<<<nblk((size_t)L.a * L.b), 256, 0, s>>>(o, L.b, L.a, dst); tc_note_launch();
        o = dst;
    }
    k_guess<<<nblk((size_t)L.a * L.b), 256, 0, s>>>(L, SF, o, n->stats, G, Vbc); tc_note_launch();
    n->st = keep;
    return r;
}

// ---- accessors for the C ABI (tc_nn_api.cu) ------------------------------------------------
tc_net_impl* net_new() { return new tc_net_impl(); }
void net_delete(tc_net_impl* n) { delete n; }
cudaStream_t& net_stream(tc_net_impl* n) { return n->st; }
int64_t net_nparam(const tc_net_impl* n) { return (int64_t)n->nparam; }
float* net_params(tc_net_impl* n) { return n->p; }
float* net_grads(tc_net_impl* n) { return n->g; }
float* net_out(tc_net_impl* n) { return n->out; }
int net_nbmax(const tc_net_impl* n) { return n->nbmax; }
int* net_fail(tc_net_impl* n) { return n->fail; }
void net_set_wait_test(tc_net_impl* n, bool on) { n->wait_test = on; }
size_t net_npx(const tc_net_impl* n, int nb) { return (size_t)nb * n->H * n->W; }
int net_repack(tc_net_impl* n) {
    pack_all(n);
    return cudaStreamSynchronize(n->st) == cudaSuccess ? 0 : 1;
}
int net_loss_value(tc_net_impl* n, float* host) {
    if (cudaMemcpyAsync(host, n->lossp + 2048, sizeof(float), cudaMemcpyDeviceToHost, n->st) != cudaSuccess) return 1;
    return cudaStreamSynchronize(n->st) == cudaSuccess ? 0 : 1;
}

// one convolution for tests: packs w (FP32 [cout][9][cin]) and runs the layer kernel
int nn_conv_test(const uint16_t* x, int nb, int H, int W, int cin, const float* w, const float* b, int cout, int relu,
                 uint16_t* y) {
    if (cin % 16 || !(cout == 32 || cout == 64 || cout == 128 || cout == 256)) return 1;
    bf16* wp = nullptr;
    int* fail = nullptr;
    if (cudaMalloc(&wp, sizeof(bf16) * 9 * cin * cout) != cudaSuccess) return 2;
    if (cudaMalloc(&fail, sizeof(int)) != cudaSuccess) { cudaFree(wp); return 2; }
    cudaMemset(fail, 0, sizeof(int));
    k_pack_fwd<<<nblk((size_t)9 * cin * cout), 256>>>(w, cout, cin, cin, cout, wp);
    tc_note_launch();
    int r = conv3x3_launch(0, (const bf16*)x, nb, H, W, cin, 0, cin, wp, b, cout, relu, (bf16*)y, cout, 0, cout, fail);
    int f = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) r = 5;
    cudaMemcpy(&f, fail, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(wp);
    cudaFree(fail);
    if (r == 0 && f) r = 6;
    return r;
}
void net_dims(const tc_net_impl* n, int* H, int* W) {
    *H = n->H;
    *W = n->W;
}
