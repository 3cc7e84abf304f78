// Learned warm start: BF16 3-D U-Net building blocks on the 5th-generation tensor cores.
//
// Activation layout: channels-last BF16 on a grid with a one-voxel zero halo. A level with
// interior X x Y x Z voxels and C channels is the row-major matrix [R][C], R = (X+2)(Y+2)(Z+2),
// row p = (z+1)*PXY + (y+1)*PX + (x+1) with PX = X+2, PXY = PX*(Y+2). Halo rows are always zero,
// so a 3x3x3 "same" convolution at row p reads rows p + off(tap) with no bounds logic, and the
// implicit GEMM tile of 128 consecutive output rows is, for each tap, one 2-D TMA box.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gbp {
namespace nn {

struct Grid3 {
    int X, Y, Z;
    long long PX, PXY, R;
};

inline Grid3 make_grid3(int X, int Y, int Z)
{
    Grid3 g{X, Y, Z, X + 2, (long long)(X + 2) * (Y + 2), 0};
    g.R = g.PXY * (Z + 2);
    return g;
}

#ifdef __CUDACC__
// GELU, tanh form (Hendrycks & Gimpel 2016), and its derivative
__device__ __forceinline__ float gelu_f(float x)
{
    const float u = 0.7978845608f * (x + 0.044715f * x * x * x);
    return 0.5f * x * (1.f + tanhf(u));
}

__device__ __forceinline__ float dgelu_f(float x)
{
    const float u = 0.7978845608f * (x + 0.044715f * x * x * x);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * 0.7978845608f * (1.f + 3.f * 0.044715f * x * x);
}
#endif

// epilogue flags
constexpr int kGelu = 1;     // forward: out = gelu(acc + bias), aux (if set) = acc + bias
constexpr int kAccum = 2;    // backward: acc += out (existing gradient)
constexpr int kDGelu = 4;    // backward: acc *= gelu'(aux)

// One convolution launch: out[p][c] = epilogue(sum_i sum_tap sum_ci in_i[p + off(tap)][ci] w[tap][c][ci0_i + ci])
// w is [ntaps][N][cin_tot] BF16 (cin_tot = sum of the inputs' channels, input i at ci0_i).
// flip = 1 negates every tap offset (the data-gradient of a convolution). The output columns are
// split into nseg segments (channel ranges of separate tensors, each [R][seg width]).
struct ConvLaunch {
    Grid3 g;
    int nin;
    const __nv_bfloat16* in[2];
    int cin[2];
    const __nv_bfloat16* w;
    int ntaps, flip, N;
    const float* bias;
    int nseg;
    __nv_bfloat16* out[2];
    __nv_bfloat16* aux[2];
    int seg_c[2];  // channel count of each segment; sum = N
    int flags;
    unsigned* err;
};

int conv3d(const ConvLaunch& L, cudaStream_t st);

// Weight gradient: dw[tap][co][ci] (+)= sum_p gout[p][co] * in[p + off(tap)][ci] for one input tensor
// (channels cin, written at channel offset ci0 of a dw with cin_tot columns), FP32 accumulation
// into dw (which the caller zeroes once per step).
struct WgradLaunch {
    Grid3 g;
    const __nv_bfloat16* in;
    int cin, ci0, cin_tot;
    const __nv_bfloat16* gout;
    int cout, ntaps;
    float* dw;
    unsigned* err;
};

int conv3d_wgrad(const WgradLaunch& L, cudaStream_t st);

}  // namespace nn
}  // namespace gbp
