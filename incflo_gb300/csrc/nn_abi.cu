// C ABI of the warm-start network: the tensor-core convolution entry points (used by the numerics
// tests against a PyTorch FP32 reference) and the surrogate object.
#include <cuda_runtime.h>

#include <mutex>

#include "gbp_internal.cuh"
#include "incflo_gb300.h"
#include "nn.h"

using namespace gbp;

namespace {

// one device error word per process for the synchronous test entry points
unsigned* test_err_word()
{
    static unsigned* w = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (!w && cudaMalloc(&w, sizeof(unsigned)) != cudaSuccess) w = nullptr;
    return w;
}

int finish_sync(unsigned* err, cudaStream_t st)
{
    unsigned h = 0;
    GBP_CUDA(cudaMemcpyAsync(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error("a bounded wait inside a tensor-core convolution ran out");
        return GBP_TIMEOUT;
    }
    return GBP_OK;
}

}  // namespace

extern "C" {

int gbp_nn_conv3d(const int dims[3], int nin, void* const in[], const int cin[], const void* w, int ntaps,
                  int flip, int cout, const float* bias, int nseg, void* const out[], void* const aux[],
                  const int seg_c[], int flags, void* stream)
{
    if (!dims || !in || !cin || !out || !seg_c || nin < 1 || nin > 2 || nseg < 1 || nseg > 2 || dims[0] < 1 ||
        dims[1] < 1 || dims[2] < 1) {
        set_error("gbp_nn_conv3d: bad arguments");
        return GBP_BAD_ARG;
    }
    unsigned* err = test_err_word();
    if (!err) return cuda_fail(cudaGetLastError(), "cudaMalloc(error word)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GBP_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    nn::ConvLaunch L{};
    L.g = nn::make_grid3(dims[0], dims[1], dims[2]);
    L.nin = nin;
    for (int i = 0; i < nin; ++i) {
        L.in[i] = static_cast<const __nv_bfloat16*>(in[i]);
        L.cin[i] = cin[i];
    }
    L.w = static_cast<const __nv_bfloat16*>(w);
    L.ntaps = ntaps;
    L.flip = flip;
    L.N = cout;
    L.bias = bias;
    L.nseg = nseg;
    for (int s = 0; s < nseg; ++s) {
        L.out[s] = static_cast<__nv_bfloat16*>(out[s]);
        L.aux[s] = aux ? static_cast<__nv_bfloat16*>(aux[s]) : nullptr;
        L.seg_c[s] = seg_c[s];
    }
    L.flags = flags;
    L.err = err;
    int rc = nn::conv3d(L, st);
    if (rc) return rc;
    return finish_sync(err, st);
}

int gbp_nn_conv3d_wgrad(const int dims[3], const void* in, int cin, int ci0, int cin_tot, const void* gout,
                        int cout, int ntaps, float* dw, void* stream)
{
    if (!dims || dims[0] < 1 || dims[1] < 1 || dims[2] < 1) {
        set_error("gbp_nn_conv3d_wgrad: bad arguments");
        return GBP_BAD_ARG;
    }
    unsigned* err = test_err_word();
    if (!err) return cuda_fail(cudaGetLastError(), "cudaMalloc(error word)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GBP_CUDA(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
    nn::WgradLaunch L{};
    L.g = nn::make_grid3(dims[0], dims[1], dims[2]);
    L.in = static_cast<const __nv_bfloat16*>(in);
    L.cin = cin;
    L.ci0 = ci0;
    L.cin_tot = cin_tot;
    L.gout = static_cast<const __nv_bfloat16*>(gout);
    L.cout = cout;
    L.ntaps = ntaps;
    L.dw = dw;
    L.err = err;
    int rc = nn::conv3d_wgrad(L, st);
    if (rc) return rc;
    return finish_sync(err, st);
}

}  // extern "C"
