// Level sweeps of the nodal operator staged through shared memory by TMA.
//
// A CTA owns a column of nodes in (x, y) and marches up a chunk of z planes. Per plane it needs x on
// plane k+1 with a one-node halo, sigma on cell plane k with a one-cell halo and b on plane k; one
// elected thread brings these in with three cp.async.bulk.tensor loads that complete on one
// mbarrier per pipeline slot (NS slots, prefetch distance NS). Planes k-1 and k of each thread's
// neighbourhood window and cell plane k-1 stay in registers, so every array is read from HBM once
// per sweep (halos come from L2) and each node reads only plane k+1 from shared memory.
//
// This file holds the FP64 sweep (FP64-issue-bound on GB300: one node per thread, 32 x 8 nodes per
// CTA, 3 slots), the FP32 sweep of the same design, the tensor-map cache and the launch helpers.
//
// Padded layout (gbp_internal.cuh): node / cell q of a row sits at position q + 4. Every x box
// starts at position x0 (node x0 - 4), a multiple of 32 elements, so it is 16-byte aligned; a box
// may start at the ghost row / plane -1 and run past the padded end (zero fill).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "gbp_internal.cuh"
#include "nodal_sweep.h"
#include "tma.cuh"

namespace gbp {

constexpr int round16(int bytes) { return (bytes + 15) / 16 * 16; }
constexpr int round128(int bytes) { return (bytes + 127) / 128 * 128; }

// Tile shapes. NX = nodes per CTA row, TY = rows, NPT = nodes per thread (x-adjacent).
template <typename T>
struct SweepCfg;
template <>
struct SweepCfg<float> {
    static constexpr int NX = 32, TY = 8, NS = 3, NPT = 1;
};
template <>
struct SweepCfg<double> {
    static constexpr int NX = 32, TY = 8, NS = 3, NPT = 1;
};

template <typename T>
struct SweepShape {
    using C = SweepCfg<T>;
    static constexpr int NX = C::NX, TY = C::TY, NS = C::NS, NPT = C::NPT;
    static constexpr int THREADS = (NX / NPT) * TY;
    static constexpr int ES = (int)sizeof(T);
    // x box: nodes x0-4 .. x0+NX (smem column of node q: q - x0 + 4)
    static constexpr int BXX = round16((NX + 5) * ES) / ES;
    // sigma box: cells x0-4 .. x0+NX-1 (column of cell c: c - x0 + 4)
    static constexpr int BXS = round16((NX + 4) * ES) / ES;
    // b box: nodes x0 .. x0+NX-1 (column of node q: q - x0)
    static constexpr int BXB = NX;
    static constexpr int XB = (TY + 2) * BXX * ES;
    static constexpr int SB = (TY + 1) * BXS * ES;
    static constexpr int BB = TY * BXB * ES;
    static constexpr int XO = 0;
    static constexpr int SO = round128(XB);
    static constexpr int BO = SO + round128(SB);
    static constexpr int STAGE = BO + round128(BB);
    static constexpr int SMEM = NS * STAGE;
    static constexpr uint32_t TX_BYTES = (uint32_t)(XB + SB + BB);
};

__device__ __forceinline__ bool alias_k(const NodalGeom& g, int k) { return g.per[2] && (k <= 1 || k == g.n[2] - 1); }
__device__ __forceinline__ bool alias_xy(const NodalGeom& g, int i, int j)
{
    return (g.per[0] && (i <= 1 || i == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1));
}
__device__ __forceinline__ bool dir_xy(const NodalGeom& g, int i, int j)
{
    return (g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]);
}
__device__ __forceinline__ bool dir_k(const NodalGeom& g, int k) { return (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]); }

template <typename T>
__device__ __forceinline__ void store_with_aliases(T* out, const NodalGeom& g, int i, int j, int k, T v, bool alias)
{
    if (alias)
        store_node(out, g, i, j, k, v);
    else
        out[pidx(g.sy, g.sz, i, j, k)] = v;
}

// (A x) at the node in window column c (FP32). P0/P1/P2: planes k-1, k, k+1 of the window (3 rows x
// W columns, column q = node i0-1+q); Sb/Sa: sigma of the cell layers below / above (2 rows x W-1,
// column q = cell i0-1+q). Isotropic form: couplings summed per neighbour with the sigma of every
// cell that contains both nodes (edge-diagonal pairs, corners single), differences to the centre.
// ------------------------------------------------------------------------------------ FP64
// One cell layer of (A x)_i from the register planes: Pn = plane k, Pd = the layer's far plane
// (k-1 or k+1), sg = sigma of the layer's 2x2 cells; accumulates into acc and the sigma sum.
template <bool ISO>
__device__ __forceinline__ void layer64(const double (&Pn)[3][3], const double (&Pd)[3][3], const double (&sg)[2][2],
                                        const NodalGeom& g, double& acc, double& ssum)
{
    const double xc = Pn[1][1];
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
        for (int cx = 0; cx < 2; ++cx) {
            const int ox = cx ? 2 : 0, oy = cy ? 2 : 0;
            const double s = sg[cy][cx];
            ssum += s;
            if (ISO) {
                const double S = (Pn[oy][ox] + Pd[1][ox]) + (Pd[oy][1] + Pd[oy][ox]);
                acc = fma(s, S, acc);
            } else {
                const double t = g.K[1] * (Pn[1][ox] - xc) + g.K[2] * (Pn[oy][1] - xc) + g.K[4] * (Pd[1][1] - xc) +
                                 g.K[3] * (Pn[oy][ox] - xc) + g.K[5] * (Pd[1][ox] - xc) +
                                 g.K[6] * (Pd[oy][1] - xc) + g.K[7] * (Pd[oy][ox] - xc);
                acc = fma(s, t, acc);
            }
        }
}

// FP32 counterpart of layer64 for the isotropic operator: differences to the centre, so rounding
// scales with the local variation of x rather than with x
__device__ __forceinline__ void layer32(const float (&Pn)[3][3], const float (&Pd)[3][3], const float (&sg)[2][2],
                                        float& acc, float& ssum)
{
    const float xc = Pn[1][1];
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
        for (int cx = 0; cx < 2; ++cx) {
            const int ox = cx ? 2 : 0, oy = cy ? 2 : 0;
            const float s = sg[cy][cx];
            ssum += s;
            const float S = ((Pn[oy][ox] - xc) + (Pd[1][ox] - xc)) + ((Pd[oy][1] - xc) + (Pd[oy][ox] - xc));
            acc = fmaf(s, S, acc);
        }
}

// FP32 sweep of the same design as the FP64 one below (isotropic spacing only): one node per
// thread, 32 x 8 nodes per CTA, 3-slot TMA ring, one block barrier per plane, float constants
// passed in (no FP64 conversions in the loop). Several CTAs per SM keep enough warps in flight.
template <int MODE>
__global__ void __launch_bounds__(SweepShape<float>::THREADS)
    k_sweep32t(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap ms,
               const __grid_constant__ CUtensorMap mb, NodalGeom g, float* __restrict__ out, float k0, float k3,
               float omega, int kchunk, unsigned* err, unsigned long long* norm)
{
    using S = SweepShape<float>;
    constexpr int NS = S::NS;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar[NS];
    __shared__ int abort_flag;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + 32 * ty;
    const int x0 = blockIdx.x * S::NX, y0 = blockIdx.y * S::TY;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    const int nsteps = kend - kbeg + 2;
    const int i = x0 + tx, j = y0 + ty;
    const bool active = i < g.nu[0] && j < g.nu[1];
    const bool dxy = dir_xy(g, i, j), axy = alias_xy(g, i, j);
    float* op = out + pidx(g.sy, g.sz, i, j, kbeg);

    auto issue = [&](int s) {
        const int slot = s % NS;
        unsigned char* base = smem + slot * S::STAGE;
        const int k = kbeg - 2 + s;
        mbar_arrive_expect_tx(&bar[slot], S::TX_BYTES);
        tma_load_3d(base + S::XO, &mx, &bar[slot], x0, y0, k + 2);
        tma_load_3d(base + S::SO, &ms, &bar[slot], x0, y0, k + 1);
        tma_load_3d(base + S::BO, &mb, &bar[slot], x0 + kOX, y0 + 1, k + 1);
    };
    if (tid == 0) {
        for (int q = 0; q < NS; ++q) mbar_init(&bar[q], 1);
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NS && s < nsteps; ++s) issue(s);

    float P0[3][3], P1[3][3], P2[3][3], S0[2][2], S1[2][2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) P0[a][b] = P1[a][b] = 0.f;
    S0[0][0] = S0[0][1] = S0[1][0] = S0[1][1] = 0.f;
    float nmax = 0.f;

    for (int s = 0; s < nsteps; ++s) {
        const int slot = s % NS;
        const unsigned char* base = smem + slot * S::STAGE;
        if (!mbar_wait_bounded(&bar[slot], (uint32_t)((s / NS) & 1), err)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        const float* sx = reinterpret_cast<const float*>(base + S::XO) + tx + 3;
        const float* ss = reinterpret_cast<const float*>(base + S::SO) + tx + 3;
        const float* sb = reinterpret_cast<const float*>(base + S::BO) + tx;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) P2[a][b] = sx[(ty + a) * S::BXX + b];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) S1[a][b] = ss[(ty + a) * S::BXS + b];
        const float bv = sb[ty * S::BXB];
        const int k = kbeg - 2 + s;
        if (s >= 2 && active) {
            float v = 0.f;
            if (!(dxy || dir_k(g, k))) {
                float acc = 0.f, ssum = 0.f;
                layer32(P1, P0, S0, acc, ssum);
                layer32(P1, P2, S1, acc, ssum);
                const float ax = k3 * acc;
                if (MODE == 0) {
                    v = fmaf(omega * (bv - ax), __frcp_rn(k0 * ssum), P1[1][1]);
                } else {
                    v = bv - ax;
                    if (norm)
                        nmax = (v != v || nmax != nmax) ? __int_as_float(0x7fc00000)
                                                        : fmaxf(nmax, fabsf(v) * (float)node_inv_volume(g, i, j, k));
                }
            }
            if (axy || alias_k(g, k))
                store_node(out, g, i, j, k, v);
            else
                *op = v;
            op += g.sz;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                P0[a][b] = P1[a][b];
                P1[a][b] = P2[a][b];
            }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) S0[a][b] = S1[a][b];
        __syncthreads();
        if (tid == 0 && s + NS < nsteps) {
            fence_proxy_async();
            issue(s + NS);
        }
    }
    if (abort_flag && tid == 0)
        for (int q = 0; q < NS; ++q) (void)mbar_wait_bounded(&bar[q], 0, nullptr);
    if (MODE == 1 && norm) {
        const double m = block_max((double)nmax);
        if (tid == 0) atomic_max_nonneg(norm, m);
    }
}

template <int MODE, bool ISO>
__global__ void __launch_bounds__(SweepShape<double>::THREADS)
    k_sweep64(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap ms,
              const __grid_constant__ CUtensorMap mb, NodalGeom g, double* __restrict__ out, double omega, int kchunk,
              unsigned* err, unsigned long long* norm)
{
    using S = SweepShape<double>;
    constexpr int NS = S::NS;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar[NS];
    __shared__ int abort_flag;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + 32 * ty;
    const int x0 = blockIdx.x * S::NX, y0 = blockIdx.y * S::TY;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    const int nsteps = kend - kbeg + 2;
    const int i = x0 + tx, j = y0 + ty;
    const bool active = i < g.nu[0] && j < g.nu[1];
    const bool dxy = dir_xy(g, i, j), axy = alias_xy(g, i, j);

    auto issue = [&](int s) {
        const int slot = s % NS;
        unsigned char* base = smem + slot * S::STAGE;
        const int k = kbeg - 2 + s;
        mbar_arrive_expect_tx(&bar[slot], S::TX_BYTES);
        tma_load_3d(base + S::XO, &mx, &bar[slot], x0, y0, k + 2);
        tma_load_3d(base + S::SO, &ms, &bar[slot], x0, y0, k + 1);
        tma_load_3d(base + S::BO, &mb, &bar[slot], x0 + kOX, y0 + 1, k + 1);
    };
    if (tid == 0) {
        for (int q = 0; q < NS; ++q) mbar_init(&bar[q], 1);
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NS && s < nsteps; ++s) issue(s);

    double P0[3][3], P1[3][3], P2[3][3], S0[2][2], S1[2][2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) P0[a][b] = P1[a][b] = 0.0;
    S0[0][0] = S0[0][1] = S0[1][0] = S0[1][1] = 0.0;
    double nmax = 0.0;

    for (int s = 0; s < nsteps; ++s) {
        const int slot = s % NS;
        const unsigned char* base = smem + slot * S::STAGE;
        if (!mbar_wait_bounded(&bar[slot], (uint32_t)((s / NS) & 1), err)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        const double* sx = reinterpret_cast<const double*>(base + S::XO) + tx + 3;
        const double* ss = reinterpret_cast<const double*>(base + S::SO) + tx + 3;
        const double* sb = reinterpret_cast<const double*>(base + S::BO) + tx;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) P2[a][b] = sx[(ty + a) * S::BXX + b];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) S1[a][b] = ss[(ty + a) * S::BXS + b];
        const double bv = sb[ty * S::BXB];
        const int k = kbeg - 2 + s;
        if (s >= 2 && active) {
            double v = 0.0;
            if (!(dxy || dir_k(g, k))) {
                double acc = 0.0, ssum = 0.0;
                layer64<ISO>(P1, P0, S0, g, acc, ssum);
                layer64<ISO>(P1, P2, S1, g, acc, ssum);
                const double xc = P1[1][1];
                const double ax = ISO ? g.K[3] * fma(-4.0 * xc, ssum, acc) : acc;
                const double diag = g.K[0] * ssum;
                if (MODE == 0) {
                    const double ad = fabs(diag);
                    const double rd = (ad > 1e-30 && ad < 1e30) ? (double)__frcp_rn((float)diag) : 1.0 / diag;
                    v = xc + omega * (bv - ax) * rd;
                } else {
                    v = bv - ax;
                    if (norm) nmax = nanmax(nmax, fabs(v) * node_inv_volume(g, i, j, k));
                }
            }
            store_with_aliases(out, g, i, j, k, v, axy || alias_k(g, k));
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                P0[a][b] = P1[a][b];
                P1[a][b] = P2[a][b];
            }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) S0[a][b] = S1[a][b];
        __syncthreads();
        if (tid == 0 && s + NS < nsteps) {
            fence_proxy_async();
            issue(s + NS);
        }
    }
    if (abort_flag && tid == 0)
        for (int q = 0; q < NS; ++q) (void)mbar_wait_bounded(&bar[q], 0, nullptr);
    if (MODE == 1 && norm) {
        nmax = block_max(nmax);
        if (tid == 0) atomic_max_nonneg(norm, nmax);
    }
}

// ------------------------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

struct MapKey {
    const void* base;
    int boxx, rows, esize;
    long long sy, sz, count;
    bool operator<(const MapKey& o) const
    {
        return std::tie(base, boxx, rows, esize, sy, sz, count) <
               std::tie(o.base, o.boxx, o.rows, o.esize, o.sy, o.sz, o.count);
    }
};

static std::mutex g_map_mu;
static std::map<MapKey, CUtensorMap> g_maps;

int make_tensor_map(const void* base, int esize, long long sy, long long sz, long long count, int boxx, int rows,
                    CUtensorMap* out)
{
    MapKey key{base, boxx, rows, esize, sy, sz, count};
    std::lock_guard<std::mutex> lk(g_map_mu);
    auto it = g_maps.find(key);
    if (it != g_maps.end()) {
        *out = it->second;
        return GBP_OK;
    }
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is unavailable from the driver");
        return GBP_CUDA_ERROR;
    }
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)sy, (cuuint64_t)(sz / sy), (cuuint64_t)(count / sz)};
    const cuuint64_t strides[2] = {(cuuint64_t)(sy * esize), (cuuint64_t)(sz * esize)};
    const cuuint32_t box[3] = {(cuuint32_t)boxx, (cuuint32_t)rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(&m, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                    const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (code " + std::to_string((int)r) + ")");
        return GBP_CUDA_ERROR;
    }
    g_maps[key] = m;
    *out = m;
    return GBP_OK;
}

void sweep_forget_maps(const void* pool_base, size_t pool_bytes)
{
    std::lock_guard<std::mutex> lk(g_map_mu);
    const char* lo = static_cast<const char*>(pool_base);
    const char* hi = lo + pool_bytes;
    for (auto it = g_maps.begin(); it != g_maps.end();) {
        const char* b = static_cast<const char*>(it->first.base);
        if (b >= lo && b < hi)
            it = g_maps.erase(it);
        else
            ++it;
    }
}

// The z-marching sweeps need a long z range per CTA to amortise their pipeline; on levels below a few
// million nodes the one-node-per-thread kernels (nodal_kernels.cu) are faster (measured: 128^3 and
// smaller levels of the 256^3 hierarchy).
constexpr long long kSweepMinNodes = 4ll << 20;

bool sweep_supported(const NodalGeom& g, int esize)
{
    const long long nodes = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    // the z-marching sweeps know Dirichlet faces only; an overset mask goes to the plain kernels
    if (nodes < kSweepMinNodes || g.mask) return false;
    if (esize == 4) return g.iso && g.nu[0] >= 32 && g.nu[1] >= 4 && g.nu[2] >= 4;
    return g.nu[0] >= 16 && g.nu[1] >= 4 && g.nu[2] >= 4;
}

int sm_count_cached();

int sm_count_cached()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// z chunking: a whole number of waves of resident CTAs, chunks of at least 16 planes
int sweep_z_chunks(const NodalGeom& g, int xy_tiles, int resident)
{
    const int slots = resident * sm_count_cached();
    // chunks of at least 4 planes: on levels whose x / y tiles alone fill few SMs (128^3: 16 tiles) the
    // z chunks supply the parallelism (128^3 Jacobi 54.6 -> 37.5 us against a 16-plane minimum; the
    // 256^3 projection 11.91 -> 11.24 ms), and the wave / halo efficiency below picks the length
    const int max_chunks = (g.nu[2] + 3) / 4;
    int best = 1;
    double best_eff = 0.0;
    for (int nz = 1; nz <= max_chunks; ++nz) {
        const int kchunk = (g.nu[2] + nz - 1) / nz;
        const int nzc = (g.nu[2] + kchunk - 1) / kchunk;
        const long long ctas = (long long)xy_tiles * nzc;
        const long long waves = (ctas + slots - 1) / slots;
        const double eff = (double)ctas / (double)(waves * slots) * (double)kchunk / (double)(kchunk + 2);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = nzc;
        }
    }
    return best;
}

template <typename T, int MODE, bool ISO>
struct SweepKernel;
template <int MODE, bool ISO>
struct SweepKernel<double, MODE, ISO> {
    static constexpr auto fn = k_sweep64<MODE, ISO>;
};

template <typename T, int MODE, bool ISO>
static int launch_sweep(const CUtensorMap& mx, const CUtensorMap& ms, const CUtensorMap& mb, const NodalGeom& g,
                        T* out, double omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using S = SweepShape<T>;
    auto kern = SweepKernel<T, MODE, ISO>::fn;
    static int resident = 0;
    if (!resident) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, S::THREADS, S::SMEM) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + S::NX - 1) / S::NX, ty = (g.nu[1] + S::TY - 1) / S::TY;
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    kern<<<grid, dim3(32, S::TY), S::SMEM, st>>>(mx, ms, mb, g, out, (T)omega, kchunk, err, norm);
    return GBP_OK;
}

template <int MODE>
static int launch_sweep32t(const CUtensorMap& mx, const CUtensorMap& ms, const CUtensorMap& mb, const NodalGeom& g,
                           float* out, float omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using S = SweepShape<float>;
    auto kern = k_sweep32t<MODE>;
    static int resident = 0;
    if (!resident) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, S::THREADS, S::SMEM) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + S::NX - 1) / S::NX, ty = (g.nu[1] + S::TY - 1) / S::TY;
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    kern<<<grid, dim3(32, S::TY), S::SMEM, st>>>(mx, ms, mb, g, out, (float)g.K[0], (float)g.K[3], omega, kchunk, err,
                                                 norm);
    return GBP_OK;
}

int sweep32_run(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using S = SweepShape<float>;
    CUtensorMap mx, ms, mb;
    int rc = make_tensor_map(x, 4, g.sy, g.sz, g.count, S::BXX, S::TY + 2, &mx);
    if (!rc) rc = make_tensor_map(s, 4, g.sy, g.sz, g.count, S::BXS, S::TY + 1, &ms);
    if (!rc) rc = make_tensor_map(b, 4, g.sy, g.sz, g.count, S::BXB, S::TY, &mb);
    if (rc) return rc;
    return mode == 0 ? launch_sweep32t<0>(mx, ms, mb, g, out, omega, err, norm, st)
                     : launch_sweep32t<1>(mx, ms, mb, g, out, omega, err, norm, st);
}

template <>
int nodal_sweep<double>(const NodalGeom& g, int mode, const double* s, const double* x, const double* b, double* out,
                        double omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using S = SweepShape<double>;
    CUtensorMap mx, ms, mb;
    int rc = make_tensor_map(x, sizeof(double), g.sy, g.sz, g.count, S::BXX, S::TY + 2, &mx);
    if (!rc) rc = make_tensor_map(s, sizeof(double), g.sy, g.sz, g.count, S::BXS, S::TY + 1, &ms);
    if (!rc) rc = make_tensor_map(b, sizeof(double), g.sy, g.sz, g.count, S::BXB, S::TY, &mb);
    if (rc) return rc;
    if (mode == 0)
        return g.iso ? launch_sweep<double, 0, true>(mx, ms, mb, g, out, omega, err, norm, st)
                     : launch_sweep<double, 0, false>(mx, ms, mb, g, out, omega, err, norm, st);
    return g.iso ? launch_sweep<double, 1, true>(mx, ms, mb, g, out, omega, err, norm, st)
                 : launch_sweep<double, 1, false>(mx, ms, mb, g, out, omega, err, norm, st);
}

template <>
int nodal_sweep<float>(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out,
                       double omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    return sweep32_run(g, mode, s, x, b, out, (float)omega, err, norm, st);
}
}  // namespace gbp
