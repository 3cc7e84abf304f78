// Warm-start U-Net: parameters, workspace, forward / backward schedule on the tensor-core
// convolutions, and the elementwise kernels around them (pooling, upsampling and their gradients,
// bias gradients, loss, Adam, BF16 weight copies, input / target / output conversion).
#include <cuda_bf16.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "gbp_internal.cuh"
#include "nn.h"
#include "nn_unet.h"

namespace gbp {
namespace nn {

namespace {

constexpr int kT = 256;

inline unsigned nblocks(long long n, int t = kT) { return (unsigned)((n + t - 1) / t); }

__device__ __forceinline__ long long row_of(const Grid3& g, int x, int y, int z)
{
    return (long long)(z + 1) * g.PXY + (long long)(y + 1) * g.PX + (x + 1);
}

__device__ __forceinline__ void ld8(const __nv_bfloat16* p, float (&v)[8])
{
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float2 f = __bfloat1622float2(h[q]);
        v[2 * q] = f.x;
        v[2 * q + 1] = f.y;
    }
}

__device__ __forceinline__ void st8(__nv_bfloat16* p, const float (&v)[8])
{
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
    *reinterpret_cast<uint4*>(p) = u;
}

// decompose a thread index over (interior voxels of g) x (C/8 channel groups)
__device__ __forceinline__ bool voxel_group(const Grid3& g, int G, int& x, int& y, int& z, int& cg)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.X * g.Y * g.Z * G) return false;
    cg = (int)(t % G);
    long long v = t / G;
    x = (int)(v % g.X);
    v /= g.X;
    y = (int)(v % g.Y);
    z = (int)(v / g.Y);
    return true;
}

__global__ void k_pool(const __nv_bfloat16* __restrict__ f, Grid3 gf, __nv_bfloat16* __restrict__ c, Grid3 gc, int C)
{
    int x, y, z, cg;
    if (!voxel_group(gc, C / 8, x, y, z, cg)) return;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                float v[8];
                ld8(f + row_of(gf, 2 * x + dx, 2 * y + dy, 2 * z + dz) * C + cg * 8, v);
#pragma unroll
                for (int e = 0; e < 8; ++e) acc[e] += v[e];
            }
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] *= 0.125f;
    st8(c + row_of(gc, x, y, z) * C + cg * 8, acc);
}

__global__ void k_upsample(const __nv_bfloat16* __restrict__ c, Grid3 gc, __nv_bfloat16* __restrict__ f, Grid3 gf, int C)
{
    int x, y, z, cg;
    if (!voxel_group(gf, C / 8, x, y, z, cg)) return;
    const uint4 u = *reinterpret_cast<const uint4*>(c + row_of(gc, x >> 1, y >> 1, z >> 1) * C + cg * 8);
    *reinterpret_cast<uint4*>(f + row_of(gf, x, y, z) * C + cg * 8) = u;
}

// gradient of the upsampling, times gelu'(pre) of the coarse tensor
__global__ void k_upsample_bwd(const __nv_bfloat16* __restrict__ gup, Grid3 gf, const __nv_bfloat16* __restrict__ pre,
                               Grid3 gc, __nv_bfloat16* __restrict__ out, int C)
{
    int x, y, z, cg;
    if (!voxel_group(gc, C / 8, x, y, z, cg)) return;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                float v[8];
                ld8(gup + row_of(gf, 2 * x + dx, 2 * y + dy, 2 * z + dz) * C + cg * 8, v);
#pragma unroll
                for (int e = 0; e < 8; ++e) acc[e] += v[e];
            }
    const long long p = row_of(gc, x, y, z) * C + cg * 8;
    float a[8];
    ld8(pre + p, a);
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] *= dgelu_f(a[e]);
    st8(out + p, acc);
}

// gradient of the skip tensor: (concat part + pooling part / 8) * gelu'(pre)
__global__ void k_pool_bwd(const __nv_bfloat16* __restrict__ gpin, Grid3 gc, const __nv_bfloat16* __restrict__ gskip,
                           const __nv_bfloat16* __restrict__ pre, Grid3 gf, __nv_bfloat16* __restrict__ out, int C)
{
    int x, y, z, cg;
    if (!voxel_group(gf, C / 8, x, y, z, cg)) return;
    const long long p = row_of(gf, x, y, z) * C + cg * 8;
    float s[8], q[8], a[8];
    ld8(gskip + p, s);
    ld8(gpin + row_of(gc, x >> 1, y >> 1, z >> 1) * C + cg * 8, q);
    ld8(pre + p, a);
#pragma unroll
    for (int e = 0; e < 8; ++e) s[e] = (s[e] + 0.125f * q[e]) * dgelu_f(a[e]);
    st8(out + p, s);
}

// db[c] += sum over rows of G[row][c] (halo rows are zero)
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ Gm, long long R, int C, float* __restrict__ db)
{
    __shared__ float s[128];
    const int G = C / 8;
    const int rows_per = blockDim.x / G;
    for (int i = threadIdx.x; i < C; i += blockDim.x) s[i] = 0.f;
    __syncthreads();
    const int cg = threadIdx.x % G;
    const int r0 = threadIdx.x / G;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (r0 < rows_per)
        for (long long r = (long long)blockIdx.x * rows_per + r0; r < R; r += (long long)gridDim.x * rows_per) {
            float v[8];
            ld8(Gm + r * C + cg * 8, v);
#pragma unroll
            for (int e = 0; e < 8; ++e) acc[e] += v[e];
        }
#pragma unroll
    for (int e = 0; e < 8; ++e) atomicAdd(&s[cg * 8 + e], acc[e]);
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) atomicAdd(db + i, s[i]);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float bc1, float bc2)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void k_cvt_weights(const float* __restrict__ w, __nv_bfloat16* __restrict__ wk, __nv_bfloat16* __restrict__ wt,
                              int taps, int cout, int cin)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)taps * cout * cin) return;
    const int ci = (int)(i % cin);
    const long long r = i / cin;
    const int co = (int)(r % cout);
    const int t = (int)(r / cout);
    const __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
    wk[i] = b;
    wt[((long long)t * cin + ci) * cout + co] = b;
}

__device__ __forceinline__ double block_sum_d(double v)
{
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// MSE over the domain voxels; gradient into channel 0 of gout
__global__ void k_loss(const __nv_bfloat16* __restrict__ hout, const float* __restrict__ target, Grid3 g, int d0, int d1,
                       int d2, float inv_n, __nv_bfloat16* __restrict__ gout, double* __restrict__ loss)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0;
    if (t < (long long)g.X * g.Y * g.Z) {
        const int x = (int)(t % g.X);
        const int y = (int)((t / g.X) % g.Y);
        const int z = (int)(t / ((long long)g.X * g.Y));
        const long long p = row_of(g, x, y, z);
        float d = 0.f;
        if (x < d0 && y < d1 && z < d2) {
            d = __bfloat162float(hout[p * kHeadC]) - target[p];
            sq = (double)d * d;
        }
        gout[p * kHeadC] = __float2bfloat16_rn(2.f * d * inv_n);
    }
    sq = block_sum_d(sq);
    if (threadIdx.x == 0) atomicAdd(loss, sq * inv_n);
}

template <typename T>
__device__ __forceinline__ float sigma_node(const NodalGeom& g, const T* s, int i, int j, int k)
{
    float a = 0.f;
    for (int c = -1; c <= 0; ++c)
        for (int b = -1; b <= 0; ++b)
            for (int q = -1; q <= 0; ++q) a += (float)s[pidx(g.sy, g.sz, i + q, j + b, k + c)];
    return 0.125f * a;
}

// stats[0] += sum rhs^2, [1] += sum sigma_node, [2] += sum phi_prev^2, [3] += count (unique nodes)
template <typename T>
__global__ void k_input_stats(NodalGeom g, const T* __restrict__ rhs, const T* __restrict__ s,
                              const double* __restrict__ phip, double* __restrict__ stats)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, b = 0.0, c = 0.0, n = 0.0;
    if (t < (long long)g.nu[0] * g.nu[1] * g.nu[2]) {
        const int i = (int)(t % g.nu[0]);
        const int j = (int)((t / g.nu[0]) % g.nu[1]);
        const int k = (int)(t / ((long long)g.nu[0] * g.nu[1]));
        const long long p = pidx(g.sy, g.sz, i, j, k);
        const double r = (double)rhs[p];
        a = r * r;
        b = sigma_node(g, s, i, j, k);
        if (phip) c = phip[p] * phip[p];
        n = 1.0;
    }
    a = block_sum_d(a);
    b = block_sum_d(b);
    c = block_sum_d(c);
    n = block_sum_d(n);
    if (threadIdx.x == 0) {
        atomicAdd(stats + 0, a);
        atomicAdd(stats + 1, b);
        atomicAdd(stats + 2, c);
        atomicAdd(stats + 3, n);
    }
}

template <typename T>
__global__ void k_input_write(NodalGeom g, const T* __restrict__ rhs, const T* __restrict__ s,
                              const double* __restrict__ phip, Grid3 g0, __nv_bfloat16* __restrict__ x0,
                              const double* __restrict__ stats)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g0.X * g0.Y * g0.Z) return;
    const int x = (int)(t % g0.X);
    const int y = (int)((t / g0.X) % g0.Y);
    const int z = (int)(t / ((long long)g0.X * g0.Y));
    float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (x < g.nu[0] && y < g.nu[1] && z < g.nu[2]) {
        const double n = fmax(stats[3], 1.0);
        const double rr = stats[0] / n, sm = stats[1] / n, pp = stats[2] / n;
        const long long p = pidx(g.sy, g.sz, x, y, z);
        v[0] = rr > 0.0 ? (float)((double)rhs[p] / sqrt(rr)) : 0.f;
        v[1] = sm > 0.0 ? (float)(sigma_node(g, s, x, y, z) / sm) - 1.f : 0.f;
        v[2] = (phip && pp > 0.0) ? (float)(phip[p] / sqrt(pp)) : 0.f;
    }
    __nv_bfloat16* o = x0 + row_of(g0, x, y, z) * kInC;
    st8(o, v);
    const float zz[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    st8(o + 8, zz);
}

__global__ void k_target_stats(NodalGeom g, const double* __restrict__ phi, const double* __restrict__ prev,
                               double* __restrict__ stats)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, n = 0.0;
    if (t < (long long)g.nu[0] * g.nu[1] * g.nu[2]) {
        const int i = (int)(t % g.nu[0]);
        const int j = (int)((t / g.nu[0]) % g.nu[1]);
        const int k = (int)(t / ((long long)g.nu[0] * g.nu[1]));
        const long long p = pidx(g.sy, g.sz, i, j, k);
        const double v = phi[p] - (prev ? prev[p] : 0.0);
        a = v * v;
        n = 1.0;
    }
    a = block_sum_d(a);
    n = block_sum_d(n);
    if (threadIdx.x == 0) {
        atomicAdd(stats + 0, a);
        atomicAdd(stats + 1, n);
    }
}

__global__ void k_target_write(NodalGeom g, const double* __restrict__ phi, const double* __restrict__ prev, Grid3 g0,
                               float* __restrict__ target, const double* __restrict__ stats)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g0.X * g0.Y * g0.Z) return;
    const int x = (int)(t % g0.X);
    const int y = (int)((t / g0.X) % g0.Y);
    const int z = (int)(t / ((long long)g0.X * g0.Y));
    float v = 0.f;
    if (x < g.nu[0] && y < g.nu[1] && z < g.nu[2]) {
        const double ms = stats[0] / fmax(stats[1], 1.0);
        const long long p = pidx(g.sy, g.sz, x, y, z);
        v = ms > 0.0 ? (float)((phi[p] - (prev ? prev[p] : 0.0)) / sqrt(ms)) : 0.f;
    }
    target[row_of(g0, x, y, z)] = v;
}

__global__ void k_extract(Grid3 g0, const __nv_bfloat16* __restrict__ hout, NodalGeom g, float* __restrict__ out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.nu[0] * g.nu[1] * g.nu[2]) return;
    const int i = (int)(t % g.nu[0]);
    const int j = (int)((t / g.nu[0]) % g.nu[1]);
    const int k = (int)(t / ((long long)g.nu[0] * g.nu[1]));
    const float v = node_is_dirichlet(g, i, j, k) ? 0.f : __bfloat162float(hout[row_of(g0, i, j, k) * kHeadC]);
    store_node(out, g, i, j, k, v);
}

__global__ void k_dot2(NodalGeom g, const float* __restrict__ x, const float* __restrict__ b,
                       const float* __restrict__ r, double* __restrict__ out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0, c = 0.0;
    if (t < (long long)g.nu[0] * g.nu[1] * g.nu[2]) {
        const int i = (int)(t % g.nu[0]);
        const int j = (int)((t / g.nu[0]) % g.nu[1]);
        const int k = (int)(t / ((long long)g.nu[0] * g.nu[1]));
        if (!node_is_dirichlet(g, i, j, k)) {
            const long long p = pidx(g.sy, g.sz, i, j, k);
            a = (double)x[p] * b[p];
            c = (double)x[p] * r[p];
        }
    }
    a = block_sum_d(a);
    c = block_sum_d(c);
    if (threadIdx.x == 0) {
        atomicAdd(out, a);
        atomicAdd(out + 1, c);
    }
}

__global__ void k_scale_to64(long long n, const float* __restrict__ x, double alpha, double* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = alpha * (double)x[i];
}

__global__ void k_scale32(long long n, float* __restrict__ x, float a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= a;
}

__global__ void k_axpy_to64(long long n, const double* __restrict__ base, const float* __restrict__ x, double alpha,
                            double* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fma(alpha, (double)x[i], base[i]);
}

__global__ void k_inject_nodes(NodalGeom gf, NodalGeom gc, int f, const double* __restrict__ src, double* __restrict__ dst)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)gc.nu[0] * gc.nu[1] * gc.nu[2]) return;
    const int i = (int)(t % gc.nu[0]);
    const int j = (int)((t / gc.nu[0]) % gc.nu[1]);
    const int k = (int)(t / ((long long)gc.nu[0] * gc.nu[1]));
    store_node(dst, gc, i, j, k, src[pidx(gf.sy, gf.sz, f * i, f * j, f * k)]);
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double gauss(uint64_t& s)
{
    // Box-Muller on two uniforms in (0, 1)
    const double u1 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = ((splitmix(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

constexpr uint32_t kFileMagic = 0x474E4E55u;  // "UNNG"

}  // namespace

void net_dims(const NodalGeom& g, int dims[3])
{
    for (int d = 0; d < 3; ++d) dims[d] = (g.nu[d] + 7) / 8 * 8;
}

// ------------------------------------------------------------------ UNet
int UNet::create(int base_channels, uint64_t seed)
{
    destroy();
    if (base_channels != 16) {
        set_error("surrogate: base_channels must be 16 (channel counts 16/32/64/128)");
        return GBP_BAD_ARG;
    }
    base_c = base_channels;
    auto C = [&](int l) { return base_c << l; };
    auto add = [&](int nin, int c0, int c1, int cout, int taps) {
        Layer L{};
        L.nin = nin;
        L.cin[0] = c0;
        L.cin[1] = c1;
        L.cin_tot = c0 + (nin > 1 ? c1 : 0);
        L.cout = cout;
        L.ntaps = taps;
        L.w_off = nparam;
        nparam += (size_t)taps * cout * L.cin_tot;
        L.b_off = nparam;
        nparam += cout;
        L.wk_off = nw;
        nw += (size_t)taps * cout * L.cin_tot;
        L.wt_off = nw;
        nw += (size_t)taps * cout * L.cin_tot;
        layers.push_back(L);
    };
    nparam = nw = 0;
    for (int l = 0; l < kLevels; ++l) {
        add(1, l == 0 ? kInC : C(l - 1), 0, C(l), 27);
        add(1, C(l), 0, C(l), 27);
    }
    for (int l = kLevels - 2; l >= 0; --l) {
        add(2, C(l + 1), C(l), C(l), 27);
        add(1, C(l), 0, C(l), 27);
    }
    add(1, C(0), 0, kHeadC, 1);
    GBP_CUDA(cudaMalloc(&param, 4 * nparam * sizeof(float)));
    grad = param + nparam;
    m1 = grad + nparam;
    m2 = m1 + nparam;
    GBP_CUDA(cudaMemset(grad, 0, 3 * nparam * sizeof(float)));
    GBP_CUDA(cudaMalloc(&wk, 2 * nw * sizeof(__nv_bfloat16)));
    wt = wk + nw;
    GBP_CUDA(cudaMalloc(&err, sizeof(unsigned)));
    GBP_CUDA(cudaMemset(err, 0, sizeof(unsigned)));
    // He-normal weights (GELU layers), small head, zero biases
    std::vector<float> h(nparam, 0.f);
    uint64_t s = seed;
    for (size_t li = 0; li < layers.size(); ++li) {
        const Layer& L = layers[li];
        const bool head = li + 1 == layers.size();
        const double sd = head ? 0.1 / sqrt((double)L.cin_tot) : sqrt(2.0 / (L.ntaps * (double)L.cin_tot));
        for (int t = 0; t < L.ntaps; ++t)
            for (int co = 0; co < L.cout; ++co)
                for (int ci = 0; ci < L.cin_tot; ++ci) {
                    const double v = gauss(s) * sd;
                    if (!head || co == 0) h[L.w_off + ((size_t)t * L.cout + co) * L.cin_tot + ci] = (float)v;
                }
    }
    GBP_CUDA(cudaMemcpy(param, h.data(), nparam * sizeof(float), cudaMemcpyHostToDevice));
    bf16_stale = true;
    step = 0;
    return GBP_OK;
}

void UNet::destroy()
{
    if (param) cudaFree(param);
    if (wk) cudaFree(wk);
    if (err) cudaFree(err);
    if (ws.base) cudaFree(ws.base);
    param = grad = m1 = m2 = nullptr;
    wk = wt = nullptr;
    err = nullptr;
    ws = Workspace{};
    layers.clear();
    nparam = nw = 0;
}

int UNet::set_params(const float* host, size_t n)
{
    if (n != nparam) {
        set_error("surrogate: parameter count mismatch");
        return GBP_BAD_ARG;
    }
    GBP_CUDA(cudaMemcpy(param, host, n * sizeof(float), cudaMemcpyHostToDevice));
    GBP_CUDA(cudaMemset(m1, 0, 2 * nparam * sizeof(float)));
    step = 0;
    bf16_stale = true;
    return GBP_OK;
}

int UNet::get_params(float* host, size_t n) const
{
    if (n != nparam) {
        set_error("surrogate: parameter count mismatch");
        return GBP_BAD_ARG;
    }
    GBP_CUDA(cudaMemcpy(host, param, n * sizeof(float), cudaMemcpyDeviceToHost));
    return GBP_OK;
}

int UNet::get_grads(float* host, size_t n) const
{
    if (n != nparam) {
        set_error("surrogate: parameter count mismatch");
        return GBP_BAD_ARG;
    }
    GBP_CUDA(cudaMemcpy(host, grad, n * sizeof(float), cudaMemcpyDeviceToHost));
    return GBP_OK;
}

int UNet::save(const char* path) const
{
    std::vector<float> h(nparam);
    int rc = get_params(h.data(), nparam);
    if (rc) return rc;
    FILE* f = fopen(path, "wb");
    if (!f) {
        set_error(std::string("surrogate: cannot write ") + path);
        return GBP_BAD_ARG;
    }
    const uint32_t hdr[4] = {kFileMagic, 1u, (uint32_t)base_c, (uint32_t)nparam};
    bool ok = fwrite(hdr, sizeof(hdr), 1, f) == 1 && fwrite(h.data(), sizeof(float), nparam, f) == nparam;
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("surrogate: short write to ") + path);
        return GBP_BAD_ARG;
    }
    return GBP_OK;
}

int UNet::load(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("surrogate: cannot read ") + path);
        return GBP_BAD_ARG;
    }
    uint32_t hdr[4] = {0, 0, 0, 0};
    std::vector<float> h(nparam);
    const bool ok = fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == kFileMagic && hdr[1] == 1u &&
                    hdr[2] == (uint32_t)base_c && hdr[3] == (uint32_t)nparam &&
                    fread(h.data(), sizeof(float), nparam, f) == nparam;
    fclose(f);
    if (!ok) {
        set_error(std::string("surrogate: ") + path + " is not a weight file of this network");
        return GBP_BAD_ARG;
    }
    return set_params(h.data(), nparam);
}

int UNet::workspace(const int dims[3], bool train)
{
    for (int d = 0; d < 3; ++d)
        if (dims[d] < 8 || dims[d] % 8) {
            set_error("surrogate: network grid dims must be positive multiples of 8");
            return GBP_BAD_ARG;
        }
    if (ws.base && ws.dims[0] == dims[0] && ws.dims[1] == dims[1] && ws.dims[2] == dims[2] && (ws.train || !train))
        return GBP_OK;
    if (ws.base) cudaFree(ws.base);
    Workspace w{};
    for (int d = 0; d < 3; ++d) w.dims[d] = dims[d];
    w.train = train;
    for (int l = 0; l < kLevels; ++l) w.g[l] = make_grid3(dims[0] >> l, dims[1] >> l, dims[2] >> l);
    // two passes: size, then carve
    size_t off = 0;
    char* base = nullptr;
    auto take = [&](long long rows, int c) {
        const size_t b = ((size_t)rows * c * sizeof(__nv_bfloat16) + 255) & ~size_t(255);
        __nv_bfloat16* p = base ? reinterpret_cast<__nv_bfloat16*>(base + off) : nullptr;
        off += b;
        return p;
    };
    auto C = [&](int l) { return base_c << l; };
    for (int pass = 0; pass < 2; ++pass) {
        off = 0;
        for (int l = 0; l < kLevels; ++l) {
            const long long R = w.g[l].R;
            w.ea[l] = take(R, C(l));
            w.eb[l] = take(R, C(l));
            if (train) {
                w.ea_pre[l] = take(R, C(l));
                w.eb_pre[l] = take(R, C(l));
            }
            if (l >= 1) w.pin[l] = take(R, C(l - 1));
            if (l <= kLevels - 2) {
                w.up[l] = take(R, C(l + 1));
                w.da[l] = take(R, C(l));
                w.db[l] = take(R, C(l));
                if (train) {
                    w.da_pre[l] = take(R, C(l));
                    w.db_pre[l] = take(R, C(l));
                }
            }
            if (train) {
                w.gA[l] = take(R, C(l));
                w.gB[l] = take(R, C(l));
                w.gskip[l] = take(R, C(l));
                if (l <= kLevels - 2) w.gup[l] = take(R, C(l + 1));
                if (l >= 1) w.gpin[l] = take(R, C(l - 1));
            }
        }
        w.hout = take(w.g[0].R, kHeadC);
        if (train) w.gout = take(w.g[0].R, kHeadC);
        if (pass == 0) {
            GBP_CUDA(cudaMalloc(&base, off));
            GBP_CUDA(cudaMemset(base, 0, off));
        }
    }
    w.base = base;
    w.bytes = off;
    ws = w;
    return GBP_OK;
}

int UNet::refresh_bf16(cudaStream_t st)
{
    if (!bf16_stale) return GBP_OK;
    for (const Layer& L : layers) {
        const long long n = (long long)L.ntaps * L.cout * L.cin_tot;
        k_cvt_weights<<<nblocks(n), kT, 0, st>>>(param + L.w_off, wk + L.wk_off, wt + L.wt_off, L.ntaps, L.cout,
                                                  L.cin_tot);
        ++nlaunch;
    }
    GBP_CUDA(cudaGetLastError());
    bf16_stale = false;
    return GBP_OK;
}

int UNet::conv(const Layer& L, int level, const __nv_bfloat16* in0, const __nv_bfloat16* in1, __nv_bfloat16* out,
               __nv_bfloat16* pre, cudaStream_t st, bool gelu)
{
    ConvLaunch c{};
    c.g = ws.g[level];
    c.nin = L.nin;
    c.in[0] = in0;
    c.in[1] = in1;
    c.cin[0] = L.cin[0];
    c.cin[1] = L.cin[1];
    c.w = wk + L.wk_off;
    c.ntaps = L.ntaps;
    c.flip = 0;
    c.N = L.cout;
    c.bias = param + L.b_off;
    c.nseg = 1;
    c.out[0] = out;
    c.aux[0] = pre;
    c.seg_c[0] = L.cout;
    c.flags = gelu ? kGelu : 0;
    c.err = err;
    ++nlaunch;
    return conv3d(c, st);
}

int UNet::conv_bwd(const Layer& L, int level, const __nv_bfloat16* g, __nv_bfloat16* dx0, __nv_bfloat16* dx1,
                   const __nv_bfloat16* pre0, const __nv_bfloat16* pre1, cudaStream_t st)
{
    ConvLaunch c{};
    c.g = ws.g[level];
    c.nin = 1;
    c.in[0] = g;
    c.cin[0] = L.cout;
    c.w = wt + L.wt_off;
    c.ntaps = L.ntaps;
    c.flip = 1;
    c.N = L.cin_tot;
    c.bias = nullptr;
    c.nseg = L.nin;
    c.out[0] = dx0;
    c.out[1] = dx1;
    c.aux[0] = const_cast<__nv_bfloat16*>(pre0);
    c.aux[1] = const_cast<__nv_bfloat16*>(pre1);
    c.seg_c[0] = L.cin[0];
    c.seg_c[1] = L.cin[1];
    c.flags = pre0 ? kDGelu : 0;
    c.err = err;
    ++nlaunch;
    return conv3d(c, st);
}

int UNet::wgrad(const Layer& L, int level, const __nv_bfloat16* in0, const __nv_bfloat16* in1, const __nv_bfloat16* g,
                cudaStream_t st)
{
    for (int i = 0; i < L.nin; ++i) {
        WgradLaunch w{};
        w.g = ws.g[level];
        w.in = i == 0 ? in0 : in1;
        w.cin = L.cin[i];
        w.ci0 = i == 0 ? 0 : L.cin[0];
        w.cin_tot = L.cin_tot;
        w.gout = g;
        w.cout = L.cout;
        w.ntaps = L.ntaps;
        w.dw = grad + L.w_off;
        w.err = err;
        int rc = conv3d_wgrad(w, st);
        if (rc) return rc;
        ++nlaunch;
    }
    const long long R = ws.g[level].R;
    const int rows_per = kT / (L.cout / 8);
    const unsigned nb = (unsigned)std::min<long long>(1024, (R + rows_per - 1) / rows_per);
    k_bias_grad<<<nb, kT, 0, st>>>(g, R, L.cout, grad + L.b_off);
    ++nlaunch;
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int UNet::forward(const __nv_bfloat16* x0, cudaStream_t st)
{
    if (!ws.base) {
        set_error("surrogate: no workspace");
        return GBP_BAD_ARG;
    }
    int rc = refresh_bf16(st);
    if (rc) return rc;
    auto C = [&](int l) { return base_c << l; };
    const bool tr = ws.train;
    for (int l = 0; l < kLevels; ++l) {
        const __nv_bfloat16* in = x0;
        if (l >= 1) {
            const Grid3& gc = ws.g[l];
            k_pool<<<nblocks((long long)gc.X * gc.Y * gc.Z * (C(l - 1) / 8)), kT, 0, st>>>(ws.eb[l - 1], ws.g[l - 1],
                                                                                           ws.pin[l], gc, C(l - 1));
            ++nlaunch;
            in = ws.pin[l];
        }
        if ((rc = conv(layers[2 * l], l, in, nullptr, ws.ea[l], tr ? ws.ea_pre[l] : nullptr, st, true))) return rc;
        if ((rc = conv(layers[2 * l + 1], l, ws.ea[l], nullptr, ws.eb[l], tr ? ws.eb_pre[l] : nullptr, st, true)))
            return rc;
    }
    for (int l = kLevels - 2; l >= 0; --l) {
        const int li = 2 * kLevels + 2 * (kLevels - 2 - l);
        const __nv_bfloat16* src = l == kLevels - 2 ? ws.eb[l + 1] : ws.db[l + 1];
        const Grid3& gf = ws.g[l];
        k_upsample<<<nblocks((long long)gf.X * gf.Y * gf.Z * (C(l + 1) / 8)), kT, 0, st>>>(src, ws.g[l + 1], ws.up[l],
                                                                                           gf, C(l + 1));
        ++nlaunch;
        if ((rc = conv(layers[li], l, ws.up[l], ws.eb[l], ws.da[l], tr ? ws.da_pre[l] : nullptr, st, true))) return rc;
        if ((rc = conv(layers[li + 1], l, ws.da[l], nullptr, ws.db[l], tr ? ws.db_pre[l] : nullptr, st, true)))
            return rc;
    }
    rc = conv(layers.back(), 0, ws.db[0], nullptr, ws.hout, nullptr, st, false);
    GBP_CUDA(cudaGetLastError());
    return rc;
}

int UNet::forward_backward(const __nv_bfloat16* x0, const float* target, const int dom[3], double* loss_dev,
                           cudaStream_t st)
{
    if (!ws.train) {
        set_error("surrogate: the workspace was not made for training");
        return GBP_BAD_ARG;
    }
    GBP_CUDA(cudaMemsetAsync(grad, 0, nparam * sizeof(float), st));
    int rc = forward(x0, st);
    if (rc) return rc;
    auto C = [&](int l) { return base_c << l; };
    const Grid3& g0 = ws.g[0];
    long long ndom = (long long)std::min(dom[0], g0.X) * std::min(dom[1], g0.Y) * std::min(dom[2], g0.Z);
    k_loss<<<nblocks((long long)g0.X * g0.Y * g0.Z), kT, 0, st>>>(ws.hout, target, g0, dom[0], dom[1], dom[2],
                                                                  1.f / (float)std::max(1ll, ndom), ws.gout, loss_dev);
    ++nlaunch;
    // head (1x1x1, no activation)
    const Layer& H = layers.back();
    if ((rc = wgrad(H, 0, ws.db[0], nullptr, ws.gout, st))) return rc;
    if ((rc = conv_bwd(H, 0, ws.gout, ws.gA[0], nullptr, ws.db_pre[0], nullptr, st))) return rc;
    // decoder, finest first; G of d_b(l) arrives in gA[l]
    for (int l = 0; l <= kLevels - 2; ++l) {
        const int li = 2 * kLevels + 2 * (kLevels - 2 - l);
        const Layer& A = layers[li];
        const Layer& B = layers[li + 1];
        if ((rc = wgrad(B, l, ws.da[l], nullptr, ws.gA[l], st))) return rc;
        if ((rc = conv_bwd(B, l, ws.gA[l], ws.gB[l], nullptr, ws.da_pre[l], nullptr, st))) return rc;
        if ((rc = wgrad(A, l, ws.up[l], ws.eb[l], ws.gB[l], st))) return rc;
        if ((rc = conv_bwd(A, l, ws.gB[l], ws.gup[l], ws.gskip[l], nullptr, nullptr, st))) return rc;
        const Grid3& gc = ws.g[l + 1];
        const __nv_bfloat16* pre_c = l == kLevels - 2 ? ws.eb_pre[l + 1] : ws.db_pre[l + 1];
        k_upsample_bwd<<<nblocks((long long)gc.X * gc.Y * gc.Z * (C(l + 1) / 8)), kT, 0, st>>>(
            ws.gup[l], ws.g[l], pre_c, gc, ws.gA[l + 1], C(l + 1));
        ++nlaunch;
    }
    // encoder, coarsest first; G of e_b(l) arrives in gA[l]
    for (int l = kLevels - 1; l >= 0; --l) {
        const Layer& A = layers[2 * l];
        const Layer& B = layers[2 * l + 1];
        if ((rc = wgrad(B, l, ws.ea[l], nullptr, ws.gA[l], st))) return rc;
        if ((rc = conv_bwd(B, l, ws.gA[l], ws.gB[l], nullptr, ws.ea_pre[l], nullptr, st))) return rc;
        const __nv_bfloat16* in = l == 0 ? x0 : ws.pin[l];
        if ((rc = wgrad(A, l, in, nullptr, ws.gB[l], st))) return rc;
        if (l == 0) break;
        if ((rc = conv_bwd(A, l, ws.gB[l], ws.gpin[l], nullptr, nullptr, nullptr, st))) return rc;
        const Grid3& gf = ws.g[l - 1];
        k_pool_bwd<<<nblocks((long long)gf.X * gf.Y * gf.Z * (C(l - 1) / 8)), kT, 0, st>>>(
            ws.gpin[l], ws.g[l], ws.gskip[l - 1], ws.eb_pre[l - 1], gf, ws.gA[l - 1], C(l - 1));
        ++nlaunch;
    }
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int UNet::adam_step(float lr, cudaStream_t st)
{
    ++step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
    k_adam<<<nblocks((long long)nparam), kT, 0, st>>>(param, grad, m1, m2, (long long)nparam, lr, b1, b2, 1e-8f, bc1,
                                                       bc2);
    ++nlaunch;
    bf16_stale = true;
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

// ------------------------------------------------------------------ conversions
template <typename T>
int build_input(const NodalGeom& g, const T* rhs, const T* sigma, const double* phi_prev, const Grid3& g0,
                __nv_bfloat16* x0, double* stats, cudaStream_t st)
{
    GBP_CUDA(cudaMemsetAsync(stats, 0, 4 * sizeof(double), st));
    const long long nu = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    k_input_stats<T><<<nblocks(nu), kT, 0, st>>>(g, rhs, sigma, phi_prev, stats);
    k_input_write<T><<<nblocks((long long)g0.X * g0.Y * g0.Z), kT, 0, st>>>(g, rhs, sigma, phi_prev, g0, x0, stats);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

template int build_input<float>(const NodalGeom&, const float*, const float*, const double*, const Grid3&,
                                __nv_bfloat16*, double*, cudaStream_t);
template int build_input<double>(const NodalGeom&, const double*, const double*, const double*, const Grid3&,
                                 __nv_bfloat16*, double*, cudaStream_t);

int build_target(const NodalGeom& g, const double* phi, const double* phi_prev, const Grid3& g0, float* target,
                 double* stats, cudaStream_t st)
{
    GBP_CUDA(cudaMemsetAsync(stats, 0, 2 * sizeof(double), st));
    const long long nu = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    k_target_stats<<<nblocks(nu), kT, 0, st>>>(g, phi, phi_prev, stats);
    k_target_write<<<nblocks((long long)g0.X * g0.Y * g0.Z), kT, 0, st>>>(g, phi, phi_prev, g0, target, stats);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int node_dot2(const NodalGeom& g, const float* x, const float* b, const float* r, double* out, cudaStream_t st)
{
    GBP_CUDA(cudaMemsetAsync(out, 0, 2 * sizeof(double), st));
    const long long nu = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    k_dot2<<<nblocks(nu), kT, 0, st>>>(g, x, b, r, out);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int scale_to64(long long count, const float* x, double alpha, double* out, cudaStream_t st)
{
    k_scale_to64<<<nblocks(count), kT, 0, st>>>(count, x, alpha, out);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int scale32(long long count, float* x, float a, cudaStream_t st)
{
    k_scale32<<<nblocks(count), kT, 0, st>>>(count, x, a);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int axpy_to64(long long count, const double* base, const float* x, double alpha, double* out, cudaStream_t st)
{
    k_axpy_to64<<<nblocks(count), kT, 0, st>>>(count, base, x, alpha, out);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int inject_nodes(const NodalGeom& gf, const NodalGeom& gc, int f, const double* src, double* dst, cudaStream_t st)
{
    const long long nu = (long long)gc.nu[0] * gc.nu[1] * gc.nu[2];
    k_inject_nodes<<<nblocks(nu), kT, 0, st>>>(gf, gc, f, src, dst);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int extract_output(const Grid3& g0, const __nv_bfloat16* hout, const NodalGeom& g, float* out, cudaStream_t st)
{
    const long long nu = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    k_extract<<<nblocks(nu), kT, 0, st>>>(g0, hout, g, out);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

}  // namespace nn
}  // namespace gbp
