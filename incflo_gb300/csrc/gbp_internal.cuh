// Internal declarations shared by the projection kernels and the host driver.
//
// Device layout of every multigrid level (nodal and cell-centred alike): one padded box
// that covers indices -1..n+1 in each direction, x fastest, with the x extent rounded up to
// a multiple of 8 elements so that every row starts on a 64-byte boundary. Entry (i,j,k) of
// a level sits at (i+1) + sy*(j+1) + sz*(k+1). A cell (i,j,k) and the node (i,j,k) at its low
// corner share that offset, so nodal stencils address their 8 surrounding cells with the same
// arithmetic as their 27 neighbouring nodes.
//
// Boundaries live in the padding, never in branches of the stencil:
//   periodic     every kernel that writes a value also writes its periodic aliases
//                (node 0 -> n, node 1 -> n+1, node n-1 -> -1; cell 0 -> n, cell n-1 -> -1);
//   non-periodic the padding holds 0: cell coefficients outside the domain are 0, so a node
//                on a Neumann/inflow face sees only its interior cells (the natural boundary
//                condition of the weak form) and a MAC Dirichlet face uses a zero ghost with
//                a doubled face coefficient.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/incflo_gb300.h"

namespace gbp {

constexpr int kMaxLevels = 24;

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Geometry of one nodal level, passed to kernels by value.
struct NodalGeom {
    int n[3];      // cells
    int nu[3];     // unique nodes: n (periodic) or n+1
    int per[3];
    int dlo[3];    // Dirichlet face on the low side
    int dhi[3];
    long long sy, sz, count;
    double K[8];   // element stiffness integral(grad N_a . grad N_b) by differing-direction mask
    double vol;    // cell volume
    double ivol;   // 1 / vol
    double h[3];
    int iso;       // hx == hy == hz: K[1] = K[2] = K[4] = 0 and K[3..7] equal
    const unsigned char* mask;  // overset mask over the padded nodes (0 = phi held at 0), or null
};

// Geometry of one cell-centred (MAC) level.
struct CellGeom {
    int n[3];
    int per[3];
    int dlo[3];
    int dhi[3];
    long long sy, sz, count;
    double w[3];   // V / h_d^2: face weight per unit beta
    double vol;
    double h[3];
    double ih[3];  // 1 / h_d (kernels multiply: an FP64 division is a dozen FP64 instructions)
    // diagonal term alpha a V per cell (the ABecLaplacian's alpha a), or null (the Poisson operator)
    const double* a64;
    const float* a32;
};

// x position of index 0 in a padded row: 4 elements, so that node/cell 0 starts a 16-byte (FP32) /
// 32-byte (FP64) boundary and even-indexed pairs can be stored as one vector; index -1 (the ghost)
// sits at position 3. Rows hold positions 0 .. n+6 (one spare past the last ghost, so a pair read
// starting at the last node stays inside its row) rounded up to a multiple of 8 elements.
constexpr int kOX = 4;
inline int padded_row(int n) { return round_up(n + kOX + 3, 8); }

__host__ __device__ inline long long pidx(long long sy, long long sz, int i, int j, int k)
{
    return (long long)(i + kOX) + sy * (long long)(j + 1) + sz * (long long)(k + 1);
}

// Positions in the padded box that alias unique node i of a direction with n cells.
__device__ __forceinline__ int node_aliases(int i, int n, int per, int out[3])
{
    out[0] = i;
    int m = 1;
    if (per) {
        if (i == 0) out[m++] = n;
        if (i == 1) out[m++] = n + 1;
        if (i == n - 1) out[m++] = -1;
    }
    return m;
}

__device__ __forceinline__ int cell_aliases(int i, int n, int per, int out[3])
{
    out[0] = i;
    int m = 1;
    if (per) {
        if (i == 0) out[m++] = n;
        if (i == n - 1) out[m++] = -1;
    }
    return m;
}

// candidate c (0..3) of the padded positions aliasing unique node i, or kNoAlias
constexpr int kNoAlias = -1000;
__device__ __forceinline__ int node_alias_cand(int i, int n, int per, int c)
{
    if (c == 0) return i;
    if (!per) return kNoAlias;
    if (c == 1) return i == 0 ? n : kNoAlias;
    if (c == 2) return i == 1 ? n + 1 : kNoAlias;
    return i == n - 1 ? -1 : kNoAlias;
}

template <typename T>
__device__ __forceinline__ void store_node(T* a, const NodalGeom& g, int i, int j, int k, T v)
{
    // nodes away from a periodic seam (all but a few planes) have no alias: one store
    const bool ax = g.per[0] && (i <= 1 || i >= g.n[0] - 1);
    const bool ay = g.per[1] && (j <= 1 || j >= g.n[1] - 1);
    const bool az = g.per[2] && (k <= 1 || k >= g.n[2] - 1);
    if (!(ax || ay || az)) {
        a[pidx(g.sy, g.sz, i, j, k)] = v;
        return;
    }
    // a node on a periodic seam: every combination of its per-direction aliases (kept as rolled
    // loops: this path is rare, and inlining it unrolled bloats every kernel that stores nodes)
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        const int kk = node_alias_cand(k, g.n[2], g.per[2], c);
        if (kk == kNoAlias) continue;
#pragma unroll 1
        for (int b = 0; b < 4; ++b) {
            const int jj = node_alias_cand(j, g.n[1], g.per[1], b);
            if (jj == kNoAlias) continue;
#pragma unroll 1
            for (int q = 0; q < 4; ++q) {
                const int ii = node_alias_cand(i, g.n[0], g.per[0], q);
                if (ii == kNoAlias) continue;
                a[pidx(g.sy, g.sz, ii, jj, kk)] = v;
            }
        }
    }
}

// store_node with the alias lists unrolled (at most 3 positions per direction, on levels of 2 cells): for kernels
// where most nodes lie on a periodic seam (the smallest levels), the rolled candidate loops cost more
// than the stencil
template <typename T>
__device__ __forceinline__ void store_node_unrolled(T* a, const NodalGeom& g, int i, int j, int k, T v)
{
    int xs[3], ys[3], zs[3];
    const int nx = node_aliases(i, g.n[0], g.per[0], xs);
    const int ny = node_aliases(j, g.n[1], g.per[1], ys);
    const int nz = node_aliases(k, g.n[2], g.per[2], zs);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c >= nz) break;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            if (b >= ny) break;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q >= nx) break;
                a[pidx(g.sy, g.sz, xs[q], ys[b], zs[c])] = v;
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void store_cell(T* a, const CellGeom& g, int i, int j, int k, T v)
{
    int xs[2], ys[2], zs[2];
    int nx = cell_aliases(i, g.n[0], g.per[0], xs);
    int ny = cell_aliases(j, g.n[1], g.per[1], ys);
    int nz = cell_aliases(k, g.n[2], g.per[2], zs);
    for (int c = 0; c < nz; ++c)
        for (int b = 0; b < ny; ++b)
            for (int q = 0; q < nx; ++q) a[pidx(g.sy, g.sz, xs[q], ys[b], zs[c])] = v;
}

// Sigma of the 8 cells around a node, used with periodic aliases of cells.
template <typename T>
__device__ __forceinline__ void store_sigma_cell(T* a, const NodalGeom& g, int i, int j, int k, T v)
{
    int xs[2], ys[2], zs[2];
    int nx = cell_aliases(i, g.n[0], g.per[0], xs);
    int ny = cell_aliases(j, g.n[1], g.per[1], ys);
    int nz = cell_aliases(k, g.n[2], g.per[2], zs);
    for (int c = 0; c < nz; ++c)
        for (int b = 0; b < ny; ++b)
            for (int q = 0; q < nx; ++q) a[pidx(g.sy, g.sz, xs[q], ys[b], zs[c])] = v;
}

__device__ __forceinline__ bool node_is_dirichlet(const NodalGeom& g, int i, int j, int k)
{
    return (g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) ||
           (g.dhi[1] && j == g.n[1]) || (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]) ||
           (g.mask && !g.mask[pidx(g.sy, g.sz, i, j, k)]);
}

// (i, j, k) of the linear index t < total = n0 n1 n2 (x fastest): 32-bit unsigned divisions when the range
// allows (a 64-bit integer division is emulated in far more instructions)
__device__ __forceinline__ void split3(long long t, int n0, int n1, long long total, int& i, int& j, int& k)
{
    if (total <= 0xffffffffll) {
        const unsigned u = (unsigned)t, a = (unsigned)n0, ab = (unsigned)n0 * (unsigned)n1;
        const unsigned kk = u / ab, r = u - kk * ab, jj = r / a;
        k = (int)kk;
        j = (int)jj;
        i = (int)(r - jj * a);
    } else {
        const long long ab = (long long)n0 * n1;
        k = (int)(t / ab);
        const long long r = t - (long long)k * ab;
        j = (int)(r / n0);
        i = (int)(r - (long long)j * n0);
    }
}

// Control volume of a node: h per direction, h/2 on a non-periodic boundary.
__device__ __forceinline__ double node_volume(const NodalGeom& g, int i, int j, int k)
{
    double v = g.vol;
    if (!g.per[0] && (i == 0 || i == g.n[0])) v *= 0.5;
    if (!g.per[1] && (j == 0 || j == g.n[1])) v *= 0.5;
    if (!g.per[2] && (k == 0 || k == g.n[2])) v *= 0.5;
    return v;
}

// max that propagates NaN (fmax would drop it): a NaN residual must surface as a NaN norm
__device__ __forceinline__ double nanmax(double a, double b) { return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000ll) : fmax(a, b); }

// Order-preserving atomic max of a non-negative double (NaN propagates as the largest).
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* dst, double v)
{
    unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    if (v != v) bits = 0x7ff8000000000000ull;
    atomicMax(dst, bits);
}

__device__ __forceinline__ void cluster_barrier()
{
    // every thread of every CTA of the cluster arrives; release / acquire order the global stores of
    // one phase before the loads of the next at cluster scope
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ unsigned cluster_nctas()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// |v| as an order-preserving integer key: for non-negative doubles the IEEE bit pattern orders like
// the value and every NaN pattern (sign cleared) lies above +inf, so an integer max over keys is a
// NaN-propagating max of |v| that costs no FP64 instruction.
__device__ __forceinline__ unsigned long long abs_key(double v)
{
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ double key_value(unsigned long long k)
{
    return k > 0x7ff0000000000000ull ? __longlong_as_double(0x7ff8000000000000ll) : __longlong_as_double((long long)k);
}

// Warp reductions over the lanes that exist: a block whose size is not a multiple of 32 has a
// partial last warp, whose missing lanes must neither be named in the shuffle mask nor read.
// Results are valid in lane 0; the order of the additions is fixed (deterministic).
__device__ __forceinline__ unsigned lanes_mask(int nl) { return nl >= 32 ? 0xffffffffu : ((1u << nl) - 1u); }
__device__ __forceinline__ double warp_sum0(double v, int lane, int nl)
{
    const unsigned m = lanes_mask(nl);
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_down_sync(m, v, o);
        if (lane + o < nl) v += w;
    }
    return v;
}
__device__ __forceinline__ double warp_max0(double v, int lane, int nl)
{
    const unsigned m = lanes_mask(nl);
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_down_sync(m, v, o);
        if (lane + o < nl) v = nanmax(v, w);
    }
    return v;
}

__device__ __forceinline__ double block_max(double v)
{
    __shared__ double red[32];
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    const int nw = (nt + 31) >> 5;
    const int lin = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = lin & 31, wid = lin >> 5;
    v = warp_max0(v, lane, min(32, nt - (wid << 5)));
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? red[lane] : 0.0;
        v = warp_max0(v, lane, min(32, nt));
    }
    return v;  // valid in thread 0
}

// block max of integer keys (valid in thread 0), partial warps allowed
__device__ __forceinline__ unsigned long long block_max_key(unsigned long long v)
{
    __shared__ unsigned long long redk[32];
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    const int nw = (nt + 31) >> 5;
    const int lin = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = lin & 31, wid = lin >> 5;
    int nl = min(32, nt - (wid << 5));
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(lanes_mask(nl), v, o);
        if (lane + o < nl && w > v) v = w;
    }
    __syncthreads();
    if (lane == 0) redk[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? redk[lane] : 0ull;
        nl = min(32, nt);
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_down_sync(lanes_mask(nl), v, o);
            if (lane + o < nl && w > v) v = w;
        }
    }
    return v;
}

// Deterministic block sum (fixed reduction tree), the result valid in every thread.
__device__ __forceinline__ double block_sum_all(double v)
{
    __shared__ double red[33];
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    const int nw = (nt + 31) >> 5;
    const int lin = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = lin & 31, wid = lin >> 5;
    v = warp_sum0(v, lane, min(32, nt - (wid << 5)));
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = lane < nw ? red[lane] : 0.0;
        t = warp_sum0(t, lane, min(32, nt));
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

// inverse control volume of a node (1/V_i): 1/h^3 doubled per non-periodic boundary face
__device__ __forceinline__ double node_inv_volume(const NodalGeom& g, int i, int j, int k)
{
    double f = 1.0;
    if (!g.per[0] && (i == 0 || i == g.n[0])) f *= 2.0;
    if (!g.per[1] && (j == 0 || j == g.n[1])) f *= 2.0;
    if (!g.per[2] && (k == 0 || k == g.n[2])) f *= 2.0;
    return f * g.ivol;
}

// ---------------------------------------------------------------------------------------
// error reporting
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define GBP_CUDA(call)                                   \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

}  // namespace gbp
