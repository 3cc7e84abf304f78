// C ABI of the warm-start network: the tensor-core convolution entry points (used by the numerics
// tests against a PyTorch FP32 reference) and the surrogate object.
#include <cuda_runtime.h>

#include <mutex>
#include <new>
#include <vector>

#include "gbp_internal.cuh"
#include "incflo_gb300.h"
#include "nn.h"
#include "nn_unet.h"
#include "nodal_kernels.h"
#include "plan.h"

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

// One training pair kept on the device: the network input and the normalised target.
struct SurrogateSample {
    __nv_bfloat16* x0 = nullptr;
    float* target = nullptr;
};

struct gbp_surrogate {
    nn::UNet net;
    int dims[3] = {0, 0, 0};  // network grid of the samples
    int dom[3] = {0, 0, 0};   // unique nodes of the sampled level (the loss domain)
    std::vector<SurrogateSample> samples;
    double* scr = nullptr;    // device scratch: statistics, losses
    double* phi_prev = nullptr;
    size_t phi_prev_count = 0;
    SurrogateSample stream_pair;  // the pair of gbp_surrogate_train_step (built, used once, overwritten)
    long long stream_rows = 0;
    ~gbp_surrogate()
    {
        for (auto& q : samples) {
            cudaFree(q.x0);
            cudaFree(q.target);
        }
        if (stream_pair.x0) cudaFree(stream_pair.x0);
        if (stream_pair.target) cudaFree(stream_pair.target);
        if (scr) cudaFree(scr);
        if (phi_prev) cudaFree(phi_prev);
    }
};

namespace {

// (input, target) of the plan's last projection into q (sized for the plan's network grid): input rhs,
// sigma and phi_prev (may be null), target phi - phi_prev (phi without one)
int make_pair(gbp_surrogate* s, gbp_plan* plan, const gbp_array4* phi_prev, SurrogateSample& q, int dims[3])
{
    NodalSolver& ns = *plan->nodal;
    const NodalGeom& g = ns.geom0();
    cudaStream_t st = ns.stream();
    nn::net_dims(g, dims);
    const nn::Grid3 g0 = nn::make_grid3(dims[0], dims[1], dims[2]);
    const double* prev = nullptr;
    if (phi_prev && phi_prev->data) {
        if ((size_t)g.count > s->phi_prev_count) {
            if (s->phi_prev) cudaFree(s->phi_prev);
            s->phi_prev = nullptr;
            s->phi_prev_count = 0;
            GBP_CUDA(cudaMalloc(&s->phi_prev, sizeof(double) * g.count));
            s->phi_prev_count = g.count;
        }
        GBP_CUDA(cudaMemsetAsync(s->phi_prev, 0, sizeof(double) * g.count, st));
        nodal_load_phi(g, *phi_prev, s->phi_prev, st);
        prev = s->phi_prev;
    }
    GBP_CUDA(cudaMemsetAsync(q.x0, 0, (size_t)g0.R * nn::kInC * sizeof(__nv_bfloat16), st));
    GBP_CUDA(cudaMemsetAsync(q.target, 0, (size_t)g0.R * sizeof(float), st));
    // channel 0 = the residual of the previous solution in this projection's system (rhs itself without
    // one): the increment is A^-1 of it, the local problem the network learns
    const double* ch0 = prev ? ns.residual_of(prev) : ns.rhs64();
    int rc = nn::build_input<double>(g, ch0, ns.sigma64(), prev, g0, q.x0, s->scr, st);
    if (!rc) rc = nn::build_target(g, ns.phi64(), prev, g0, q.target, s->scr + 4, st);
    return rc;
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

int gbp_surrogate_create(int base_channels, unsigned long long seed, gbp_surrogate** out)
{
    if (!out) {
        set_error("gbp_surrogate_create: out is NULL");
        return GBP_BAD_ARG;
    }
    *out = nullptr;
    gbp_surrogate* s = new (std::nothrow) gbp_surrogate();
    if (!s) {
        set_error("gbp_surrogate_create: out of host memory");
        return GBP_BAD_ARG;
    }
    int rc = s->net.create(base_channels, seed);
    if (!rc && cudaMalloc(&s->scr, 64 * sizeof(double)) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "cudaMalloc");
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return GBP_OK;
}

int gbp_surrogate_destroy(gbp_surrogate* s)
{
    if (s) {
        cudaDeviceSynchronize();
        delete s;
    }
    return GBP_OK;
}

long long gbp_surrogate_num_params(const gbp_surrogate* s) { return s ? (long long)s->net.num_params() : 0; }

int gbp_surrogate_get_params(const gbp_surrogate* s, float* host, long long n)
{
    if (!s || !host) return GBP_BAD_ARG;
    return s->net.get_params(host, (size_t)n);
}

int gbp_surrogate_set_params(gbp_surrogate* s, const float* host, long long n)
{
    if (!s || !host) return GBP_BAD_ARG;
    return s->net.set_params(host, (size_t)n);
}

int gbp_surrogate_get_grads(const gbp_surrogate* s, float* host, long long n)
{
    if (!s || !host) return GBP_BAD_ARG;
    return s->net.get_grads(host, (size_t)n);
}

int gbp_surrogate_save(const gbp_surrogate* s, const char* path)
{
    if (!s || !path) return GBP_BAD_ARG;
    return s->net.save(path);
}

int gbp_surrogate_load(gbp_surrogate* s, const char* path)
{
    if (!s || !path) return GBP_BAD_ARG;
    return s->net.load(path);
}

int gbp_surrogate_train_pair(gbp_surrogate* s, const int dims[3], const int dom[3], const void* x0,
                             const float* target, float lr, double* loss, void* stream)
{
    if (!s || !dims || !dom || !x0 || !target) {
        set_error("gbp_surrogate_train_pair: bad arguments");
        return GBP_BAD_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = s->net.workspace(dims, true);
    if (rc) return rc;
    GBP_CUDA(cudaMemsetAsync(s->scr, 0, sizeof(double), st));
    GBP_CUDA(cudaMemsetAsync(s->net.err_word(), 0, sizeof(unsigned), st));
    rc = s->net.forward_backward(static_cast<const __nv_bfloat16*>(x0), target, dom, s->scr, st);
    if (!rc && lr > 0.f) rc = s->net.adam_step(lr, st);
    if (rc) return rc;
    double h = 0.0;
    GBP_CUDA(cudaMemcpyAsync(&h, s->scr, sizeof(double), cudaMemcpyDeviceToHost, st));
    rc = finish_sync(s->net.err_word(), st);
    if (loss) *loss = h;
    return rc;
}

int gbp_surrogate_predict(gbp_surrogate* s, const int dims[3], const void* x0, void* hout, void* stream)
{
    if (!s || !dims || !x0) {
        set_error("gbp_surrogate_predict: bad arguments");
        return GBP_BAD_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = s->net.workspace(dims, false);
    if (rc) return rc;
    GBP_CUDA(cudaMemsetAsync(s->net.err_word(), 0, sizeof(unsigned), st));
    rc = s->net.forward(static_cast<const __nv_bfloat16*>(x0), st);
    if (rc) return rc;
    if (hout) {
        const nn::Grid3& g = s->net.grid0();
        GBP_CUDA(cudaMemcpyAsync(hout, s->net.hout(), (size_t)g.R * nn::kHeadC * sizeof(__nv_bfloat16),
                                 cudaMemcpyDeviceToDevice, st));
    }
    return finish_sync(s->net.err_word(), st);
}

int gbp_surrogate_train_step(gbp_surrogate* s, gbp_plan* plan, const gbp_array4* phi_prev, float lr, double* loss)
{
    if (!s || !plan || !plan->nodal || !(lr >= 0.f)) {
        set_error("gbp_surrogate_train_step: needs a surrogate, a nodal plan after a projection and lr >= 0");
        return GBP_BAD_ARG;
    }
    NodalSolver& ns = *plan->nodal;
    cudaStream_t st = ns.stream();
    int dims[3];
    nn::net_dims(ns.geom0(), dims);
    const nn::Grid3 g0 = nn::make_grid3(dims[0], dims[1], dims[2]);
    if (g0.R > s->stream_rows) {
        if (s->stream_pair.x0) cudaFree(s->stream_pair.x0);
        if (s->stream_pair.target) cudaFree(s->stream_pair.target);
        s->stream_pair = SurrogateSample{};
        s->stream_rows = 0;
        GBP_CUDA(cudaMalloc(&s->stream_pair.x0, (size_t)g0.R * nn::kInC * sizeof(__nv_bfloat16)));
        GBP_CUDA(cudaMalloc(&s->stream_pair.target, (size_t)g0.R * sizeof(float)));
        s->stream_rows = g0.R;
    }
    int rc = make_pair(s, plan, phi_prev, s->stream_pair, dims);
    if (rc) return rc;
    const int dom[3] = {ns.geom0().nu[0], ns.geom0().nu[1], ns.geom0().nu[2]};
    rc = s->net.workspace(dims, true);
    if (rc) return rc;
    GBP_CUDA(cudaMemsetAsync(s->scr + 8, 0, sizeof(double), st));
    GBP_CUDA(cudaMemsetAsync(s->net.err_word(), 0, sizeof(unsigned), st));
    rc = s->net.forward_backward(s->stream_pair.x0, s->stream_pair.target, dom, s->scr + 8, st);
    if (!rc && lr > 0.f) rc = s->net.adam_step(lr, st);
    if (rc) return rc;
    double h = 0.0;
    GBP_CUDA(cudaMemcpyAsync(&h, s->scr + 8, sizeof(double), cudaMemcpyDeviceToHost, st));
    rc = finish_sync(s->net.err_word(), st);
    if (loss) *loss = h;
    return rc;
}

int gbp_surrogate_add_sample(gbp_surrogate* s, gbp_plan* plan, const gbp_array4* phi_prev)
{
    if (!s || !plan || !plan->nodal) {
        set_error("gbp_surrogate_add_sample: needs a surrogate and a nodal plan after a projection");
        return GBP_BAD_ARG;
    }
    NodalSolver& ns = *plan->nodal;
    const NodalGeom& g = ns.geom0();
    cudaStream_t st = ns.stream();
    int dims[3];
    nn::net_dims(g, dims);
    if (!s->samples.empty() && (dims[0] != s->dims[0] || dims[1] != s->dims[1] || dims[2] != s->dims[2])) {
        set_error("gbp_surrogate_add_sample: all samples must come from plans of the same size");
        return GBP_BAD_ARG;
    }
    const nn::Grid3 g0 = nn::make_grid3(dims[0], dims[1], dims[2]);
    SurrogateSample q;
    GBP_CUDA(cudaMalloc(&q.x0, (size_t)g0.R * nn::kInC * sizeof(__nv_bfloat16)));
    if (cudaMalloc(&q.target, (size_t)g0.R * sizeof(float)) != cudaSuccess) {
        cudaFree(q.x0);
        return cuda_fail(cudaGetLastError(), "cudaMalloc(sample)");
    }
    int rc = make_pair(s, plan, phi_prev, q, dims);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "add_sample");
    }
    if (rc) {
        cudaFree(q.x0);
        cudaFree(q.target);
        return rc;
    }
    for (int d = 0; d < 3; ++d) {
        s->dims[d] = dims[d];
        s->dom[d] = g.nu[d];
    }
    s->samples.push_back(q);
    return GBP_OK;
}

int gbp_surrogate_num_samples(const gbp_surrogate* s) { return s ? (int)s->samples.size() : 0; }

int gbp_surrogate_clear_samples(gbp_surrogate* s)
{
    if (!s) return GBP_BAD_ARG;
    cudaDeviceSynchronize();
    for (auto& q : s->samples) {
        cudaFree(q.x0);
        cudaFree(q.target);
    }
    s->samples.clear();
    return GBP_OK;
}

int gbp_surrogate_train(gbp_surrogate* s, int steps, float lr, unsigned long long seed, float* losses, void* stream)
{
    if (!s || steps < 0 || s->samples.empty() || steps > 60) {
        if (!s || s->samples.empty()) set_error("gbp_surrogate_train: no samples");
        else set_error("gbp_surrogate_train: steps must be 0..60 per call (losses are kept on the device)");
        return GBP_BAD_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = s->net.workspace(s->dims, true);
    if (rc) return rc;
    GBP_CUDA(cudaMemsetAsync(s->scr, 0, 64 * sizeof(double), st));
    GBP_CUDA(cudaMemsetAsync(s->net.err_word(), 0, sizeof(unsigned), st));
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + 1;
    for (int k = 0; k < steps; ++k) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        const SurrogateSample& q = s->samples[x % s->samples.size()];
        rc = s->net.forward_backward(q.x0, q.target, s->dom, s->scr + k, st);
        if (!rc) rc = s->net.adam_step(lr, st);
        if (rc) return rc;
    }
    double h[64];
    GBP_CUDA(cudaMemcpyAsync(h, s->scr, 64 * sizeof(double), cudaMemcpyDeviceToHost, st));
    rc = finish_sync(s->net.err_word(), st);
    if (losses)
        for (int k = 0; k < steps; ++k) losses[k] = (float)h[k];
    return rc;
}

int gbp_plan_set_surrogate(gbp_plan* plan, gbp_surrogate* s, int level, int mode)
{
    if (!plan || !plan->nodal) {
        set_error("gbp_plan_set_surrogate: needs a nodal plan");
        return GBP_BAD_ARG;
    }
    return plan->nodal->set_surrogate(s ? &s->net : nullptr, level, mode);
}

}  // extern "C"
