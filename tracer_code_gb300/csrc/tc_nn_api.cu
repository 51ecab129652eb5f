// tc_nn_api.cu -- C ABI of the learned initial guess (tracer_nn.h).
#include "tc_nn.h"
#include "tracer_nn.h"

#include <vector>

struct tc_net_impl;
int net_create(tc_net_impl* n, int nbmax, int H, int W, uint64_t seed);
int net_forward(tc_net_impl* n, int nb);
int net_backward(tc_net_impl* n, int nb);
void net_prepare(tc_net_impl* n, const float* raw, int nb);
int net_loss(tc_net_impl* n, const float* raw, const float* sf_new, int nb, float* loss_host);
void net_adam(tc_net_impl* n, float lr, float b1, float b2, float eps);
void net_destroy(tc_net_impl* n);
tc_net_impl* net_new();
void net_delete(tc_net_impl* n);
cudaStream_t& net_stream(tc_net_impl* n);
int64_t net_nparam(const tc_net_impl* n);
float* net_params(tc_net_impl* n);
float* net_grads(tc_net_impl* n);
float* net_out(tc_net_impl* n);
int net_nbmax(const tc_net_impl* n);
int* net_fail(tc_net_impl* n);
void net_set_wait_test(tc_net_impl* n, bool on);
int net_repack(tc_net_impl* n);
size_t net_npx(const tc_net_impl* n, int nb);
int net_loss_value(tc_net_impl* n, float* host);
int nn_conv_test(const uint16_t* x, int nb, int H, int W, int cin, const float* w, const float* b, int cout, int relu,
                 uint16_t* y);

struct tc_net {
    tc_net_impl* impl;
};
tc_net_impl* tcnn_impl(tc_net* n) { return n ? n->impl : nullptr; }

static tc_status chk_fail(tc_net* net) {
    int f = 0;
    if (cudaMemcpyAsync(&f, net_fail(net->impl), sizeof(int), cudaMemcpyDeviceToHost, net_stream(net->impl)) !=
        cudaSuccess)
        return TC_ERR_CUDA;
    if (cudaStreamSynchronize(net_stream(net->impl)) != cudaSuccess) return TC_ERR_CUDA;
    return f ? TC_ERR_DEVICE_TIMEOUT : TC_OK;
}

extern "C" {

tc_status tcnn_create(int32_t nb_max, int32_t H, int32_t W, uint64_t seed, tc_net** out) {
    if (!out) return TC_ERR_ARG;
    tc_net_impl* n = net_new();
    const int r = net_create(n, nb_max, H, W, seed);
    if (r != 0) {
        net_destroy(n);
        net_delete(n);
        return r == 1 ? TC_ERR_ARG : (r == 2 ? TC_ERR_ALLOC : TC_ERR_CUDA);
    }
    *out = new tc_net{n};
    return TC_OK;
}
tc_status tcnn_destroy(tc_net* net) {
    if (!net) return TC_ERR_ARG;
    net_destroy(net->impl);
    net_delete(net->impl);
    delete net;
    return TC_OK;
}
tc_status tcnn_debug_wait_test(tc_net* net, int32_t on) {
    if (!net) return TC_ERR_ARG;
    net_set_wait_test(net->impl, on != 0);
    return TC_OK;
}
tc_status tcnn_set_stream(tc_net* net, void* stream) {
    if (!net) return TC_ERR_ARG;
    net_stream(net->impl) = (cudaStream_t)stream;
    return TC_OK;
}
int64_t tcnn_param_count(const tc_net* net) { return net ? net_nparam(net->impl) : 0; }
tc_status tcnn_get_params(tc_net* net, float* host) {
    if (!net || !host) return TC_ERR_ARG;
    if (cudaMemcpy(host, net_params(net->impl), sizeof(float) * net_nparam(net->impl), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return TC_ERR_CUDA;
    return TC_OK;
}
tc_status tcnn_set_params(tc_net* net, const float* host) {
    if (!net || !host) return TC_ERR_ARG;
    if (cudaMemcpy(net_params(net->impl), host, sizeof(float) * net_nparam(net->impl), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return TC_ERR_CUDA;
    return net_repack(net->impl) == 0 ? TC_OK : TC_ERR_CUDA;
}
tc_status tcnn_get_grads(tc_net* net, float* host) {
    if (!net || !host) return TC_ERR_ARG;
    if (cudaMemcpy(host, net_grads(net->impl), sizeof(float) * net_nparam(net->impl), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return TC_ERR_CUDA;
    return TC_OK;
}
tc_status tcnn_forward(tc_net* net, const float* raw, int32_t nb, float* out) {
    if (!net || !raw || !out || nb < 1 || nb > net_nbmax(net->impl)) return TC_ERR_ARG;
    net_prepare(net->impl, raw, nb);
    if (net_forward(net->impl, nb) != 0) return TC_ERR_CUDA;
    if (cudaMemcpyAsync(out, net_out(net->impl), sizeof(float) * net_npx(net->impl, nb), cudaMemcpyDeviceToDevice,
                        net_stream(net->impl)) != cudaSuccess)
        return TC_ERR_CUDA;
    return chk_fail(net);
}
tc_status tcnn_loss_backward(tc_net* net, const float* raw, const float* sf_new, int32_t nb, float* loss_host) {
    if (!net || !raw || !sf_new || nb < 1 || nb > net_nbmax(net->impl)) return TC_ERR_ARG;
    net_prepare(net->impl, raw, nb);
    if (net_forward(net->impl, nb) != 0) return TC_ERR_CUDA;
    if (net_loss(net->impl, raw, sf_new, nb, nullptr) != 0) return TC_ERR_CUDA;
    if (net_backward(net->impl, nb) != 0) return TC_ERR_CUDA;
    if (loss_host && net_loss_value(net->impl, loss_host) != 0) return TC_ERR_CUDA;
    return chk_fail(net);
}
tc_status tcnn_adam(tc_net* net, float lr, float beta1, float beta2, float eps) {
    if (!net) return TC_ERR_ARG;
    net_adam(net->impl, lr, beta1, beta2, eps);
    return cudaGetLastError() == cudaSuccess ? TC_OK : TC_ERR_CUDA;
}

tc_status tcnn_conv3x3(const uint16_t* x, int32_t nb, int32_t H, int32_t W, int32_t cin, const float* w,
                       const float* b, int32_t cout, int32_t relu, uint16_t* y) {
    const int r = nn_conv_test(x, nb, H, W, cin, w, b, cout, relu, y);
    return r == 0 ? TC_OK : (r == 1 ? TC_ERR_ARG : (r == 6 ? TC_ERR_DEVICE_TIMEOUT : TC_ERR_CUDA));
}

}  // extern "C"
