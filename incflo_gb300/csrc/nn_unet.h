// Warm-start U-Net: four levels (base, 2 base, 4 base, 8 base channels), two 3x3x3 convolutions
// + GELU per level on the way down (2x2x2 average pooling between levels) and on the way up
// (nearest-neighbour upsampling, concatenation with the skip tensor of the same level), and a 1x1x1
// head whose channel 0 is the prediction. Inputs (3 channels in a 16-channel tensor): the nodal
// right-hand side / rms, the node-averaged sigma / mean, the previous phi / rms. Output: the shape
// of phi; its amplitude is fitted by the solver (Galerkin scaling). BF16 activations and weights,
// FP32 accumulation, FP32 master weights with Adam.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <stdint.h>

#include <vector>

#include "gbp_internal.cuh"
#include "nn.h"

namespace gbp {
namespace nn {

constexpr int kLevels = 4;
constexpr int kInC = 16;   // input tensor channels (3 used)
constexpr int kHeadC = 16; // head output channels (1 used)

struct Layer {
    int nin, cin[2], cin_tot, cout, ntaps;
    size_t w_off, b_off;   // FP32 parameter offsets
    size_t wk_off, wt_off; // BF16 weight offsets (forward [tap][cout][cin], transposed [tap][cin][cout])
};

struct Workspace {
    int dims[3] = {0, 0, 0};
    bool train = false;
    Grid3 g[kLevels];
    __nv_bfloat16 *ea_pre[kLevels] = {}, *ea[kLevels] = {}, *eb_pre[kLevels] = {}, *eb[kLevels] = {};
    __nv_bfloat16* pin[kLevels] = {};  // pooled input of level l >= 1 ([R_l][C_{l-1}])
    __nv_bfloat16 *up[kLevels] = {}, *da_pre[kLevels] = {}, *da[kLevels] = {}, *db_pre[kLevels] = {}, *db[kLevels] = {};
    __nv_bfloat16* hout = nullptr;  // [R_0][16]
    // gradients (training only)
    __nv_bfloat16 *gA[kLevels] = {}, *gB[kLevels] = {}, *gskip[kLevels] = {}, *gup[kLevels] = {}, *gpin[kLevels] = {};
    __nv_bfloat16* gout = nullptr;
    char* base = nullptr;
    size_t bytes = 0;
};

class UNet {
public:
    int create(int base_channels, uint64_t seed);
    void destroy();
    ~UNet() { destroy(); }

    size_t num_params() const { return nparam; }
    int set_params(const float* host, size_t n);
    int get_params(float* host, size_t n) const;
    int get_grads(float* host, size_t n) const;
    int save(const char* path) const;
    int load(const char* path);
    int base() const { return base_c; }

    // dims: the network grid (each a multiple of 8); buffers are (re)allocated when dims change
    int workspace(const int dims[3], bool train);
    // forward pass on x0 ([R_0][16] BF16, zero halo); the prediction is channel 0 of hout()
    int forward(const __nv_bfloat16* x0, cudaStream_t st);
    // zero grads, forward, MSE loss against target ([R_0] FP32; only voxels with x < dom[0], y < dom[1],
    // z < dom[2] count), backward; *loss_dev receives the loss (device double)
    int forward_backward(const __nv_bfloat16* x0, const float* target, const int dom[3], double* loss_dev,
                         cudaStream_t st);
    int adam_step(float lr, cudaStream_t st);
    const __nv_bfloat16* hout() const { return ws.hout; }
    const Grid3& grid0() const { return ws.g[0]; }
    unsigned* err_word() const { return err; }
    long long launches() const { return nlaunch; }

private:
    int conv(const Layer& L, int level, const __nv_bfloat16* in0, const __nv_bfloat16* in1, __nv_bfloat16* out,
             __nv_bfloat16* pre, cudaStream_t st, bool gelu);
    int conv_bwd(const Layer& L, int level, const __nv_bfloat16* g, __nv_bfloat16* dx0, __nv_bfloat16* dx1,
                 const __nv_bfloat16* pre0, const __nv_bfloat16* pre1, cudaStream_t st);
    int wgrad(const Layer& L, int level, const __nv_bfloat16* in0, const __nv_bfloat16* in1, const __nv_bfloat16* g,
              cudaStream_t st);
    int refresh_bf16(cudaStream_t st);

    int base_c = 16;
    std::vector<Layer> layers;
    size_t nparam = 0, nw = 0;
    float *param = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *wk = nullptr, *wt = nullptr;
    bool bf16_stale = true;
    int step = 0;
    unsigned* err = nullptr;
    Workspace ws;
    long long nlaunch = 0;
};

// Input tensor of the network from one nodal level: rhs (weak form) and sigma of that level,
// optional phi_prev (FP64 nodal, may be null). stats: 4 device doubles of scratch.
template <typename T>
int build_input(const NodalGeom& g, const T* rhs, const T* sigma, const double* phi_prev, const Grid3& g0,
                __nv_bfloat16* x0, double* stats, cudaStream_t st);
// Target tensor of the network from a nodal solution, on the unique nodes:
// target = (phi - phi_prev) / rms (phi_prev == nullptr: phi / rms): the increment the network predicts on
// top of the previous solution, or the solution itself from a zero start
int build_target(const NodalGeom& g, const double* phi, const double* phi_prev, const Grid3& g0, float* target,
                 double* stats,
                 cudaStream_t st);
// Prediction (channel 0 of hout) onto the unique nodes of a nodal level, with periodic aliases.
int extract_output(const Grid3& g0, const __nv_bfloat16* hout, const NodalGeom& g, float* out, cudaStream_t st);
// network grid of a nodal level: unique nodes rounded up to multiples of 8
void net_dims(const NodalGeom& g, int dims[3]);
// out[0] = sum x.b, out[1] = sum x.r over the unique, non-Dirichlet nodes (FP64 sums, device)
int node_dot2(const NodalGeom& g, const float* x, const float* b, const float* r, double* out, cudaStream_t st);
// out[i] = alpha * x[i] over a whole padded level array
int scale_to64(long long count, const float* x, double alpha, double* out, cudaStream_t st);
// x *= a over count padded positions
int scale32(long long count, float* x, float a, cudaStream_t st);
// out = base + alpha x over count padded positions (the previous solution plus the scaled increment)
int axpy_to64(long long count, const double* base, const float* x, double alpha, double* out, cudaStream_t st);
// dst = src at every unique node of the coarse level gc (the fine level's node (f i, f j, f k), f = 2^levels
// apart, periodic aliases written): the previous solution injected onto the network's level
int inject_nodes(const NodalGeom& gf, const NodalGeom& gc, int f, const double* src, double* dst, cudaStream_t st);

}  // namespace nn
}  // namespace gbp
