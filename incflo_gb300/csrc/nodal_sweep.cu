// Level sweeps of the nodal operator staged through shared memory by TMA.
//
// A CTA owns a 32 x TY column of nodes in (x, y) and marches up a chunk of z planes. Per plane it
// needs x on plane k+1 with a one-node halo, sigma on cell plane k with a one-cell halo and b on
// plane k; one elected thread brings these in with three cp.async.bulk.tensor loads that complete
// on one mbarrier per pipeline slot (NS slots, prefetch distance NS). Planes k-1 and k of the 3x3
// neighbourhood and cell plane k-1 stay in registers, so each node reads 9 + 4 + 1 values from
// shared memory and each array is read from HBM once (halos come from L2).
//
// FP32 sweeps are HBM-bound: 32 x 16 tiles and 4 slots keep ~60 KB per SM in flight, and the z
// chunking is chosen so the grid is a whole number of waves of resident CTAs. FP64 sweeps are
// bound by the FP64 issue rate of GB300, so their tile is smaller (32 x 8, 3 slots).
//
// Boundary handling follows the padded layout of gbp_internal.cuh: a TMA box may start at the
// ghost row/plane (-1) and run past the padded end (zero fill); tile x origins are multiples of 32
// nodes, so every box starts on a 16-byte boundary of its row (padded index x0 = node x0 - 1).
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

template <typename T>
struct SweepCfg;
template <>
struct SweepCfg<float> {
    static constexpr int TX = 32, TY = 16, NS = 4;
};
template <>
struct SweepCfg<double> {
    static constexpr int TX = 32, TY = 8, NS = 3;
};

template <typename T>
struct SweepShape {
    static constexpr int TX = SweepCfg<T>::TX, TY = SweepCfg<T>::TY, NS = SweepCfg<T>::NS;
    static constexpr int BX = (((TX + 2) * (int)sizeof(T) + 15) / 16 * 16) / (int)sizeof(T);
    static constexpr int XB = (TY + 2) * BX * (int)sizeof(T);
    static constexpr int SB = (TY + 1) * BX * (int)sizeof(T);
    static constexpr int BB = TY * BX * (int)sizeof(T);
    static constexpr int XO = 0;
    static constexpr int SO = (XB + 127) / 128 * 128;
    static constexpr int BO = SO + (SB + 127) / 128 * 128;
    static constexpr int STAGE = BO + (BB + 127) / 128 * 128;
    static constexpr uint32_t TX_BYTES = (uint32_t)(XB + SB + BB);
};

__device__ __forceinline__ bool has_alias(const NodalGeom& g, int i, int j, int k)
{
    return (g.per[0] && (i <= 1 || i == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1)) ||
           (g.per[2] && (k <= 1 || k == g.n[2] - 1));
}

// One cell layer of (A x)_i from the register planes: Pn = plane k, Pd = the layer's far plane
// (k-1 or k+1), sg = sigma of the layer's 2x2 cells; accumulates into acc and the sigma sum.
template <typename T, bool ISO>
__device__ __forceinline__ void layer(const T (&Pn)[3][3], const T (&Pd)[3][3], const T (&sg)[2][2], const NodalGeom& g,
                                      T& acc, T& ssum)
{
    const T xc = Pn[1][1];
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
        for (int cx = 0; cx < 2; ++cx) {
            const int ox = cx ? 2 : 0, oy = cy ? 2 : 0;
            const T s = sg[cy][cx];
            ssum += s;
            if (ISO) {
                if constexpr (sizeof(T) == 8) {
                    const T S = (Pn[oy][ox] + Pd[1][ox]) + (Pd[oy][1] + Pd[oy][ox]);
                    acc = fma(s, S, acc);
                } else {
                    const T S = ((Pn[oy][ox] - xc) + (Pd[1][ox] - xc)) + ((Pd[oy][1] - xc) + (Pd[oy][ox] - xc));
                    acc = fmaf(s, S, acc);
                }
            } else {
                const T t = (T)g.K[1] * (Pn[1][ox] - xc) + (T)g.K[2] * (Pn[oy][1] - xc) + (T)g.K[4] * (Pd[1][1] - xc) +
                            (T)g.K[3] * (Pn[oy][ox] - xc) + (T)g.K[5] * (Pd[1][ox] - xc) +
                            (T)g.K[6] * (Pd[oy][1] - xc) + (T)g.K[7] * (Pd[oy][ox] - xc);
                acc += s * t;
            }
        }
}

template <typename T, int MODE, bool ISO>
__global__ void __launch_bounds__(SweepCfg<T>::TX* SweepCfg<T>::TY)
    k_nodal_sweep(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap ms,
                  const __grid_constant__ CUtensorMap mb, NodalGeom g, T* __restrict__ out, T omega, int kchunk,
                  unsigned* err, unsigned long long* norm)
{
    using S = SweepShape<T>;
    constexpr int BX = S::BX, TX = S::TX, NS = S::NS;
    __shared__ __align__(1024) unsigned char smem[NS * S::STAGE];
    __shared__ uint64_t bar[NS];
    __shared__ int abort_flag;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + TX * ty;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * S::TY;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    const int nsteps = kend - kbeg + 2;
    const int i = x0 + tx, j = y0 + ty;
    const bool active = i < g.nu[0] && j < g.nu[1];

    auto issue = [&](int s) {
        const int slot = s % NS;
        unsigned char* base = smem + slot * S::STAGE;
        const int k = kbeg - 2 + s;
        mbar_arrive_expect_tx(&bar[slot], S::TX_BYTES);
        // padded coordinates: node / cell index q sits at q + 1
        tma_load_3d(base + S::XO, &mx, &bar[slot], x0, y0, k + 2);      // x nodes y0-1.., plane k+1
        tma_load_3d(base + S::SO, &ms, &bar[slot], x0, y0, k + 1);      // sigma cells y0-1.., plane k
        tma_load_3d(base + S::BO, &mb, &bar[slot], x0, y0 + 1, k + 1);  // b nodes y0.., plane k
    };

    if (tid == 0) {
        for (int q = 0; q < NS; ++q) mbar_init(&bar[q], 1);
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NS && s < nsteps; ++s) issue(s);

    T P0[3][3], P1[3][3], P2[3][3], S0[2][2], S1[2][2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) P0[a][b] = P1[a][b] = T(0);
    S0[0][0] = S0[0][1] = S0[1][0] = S0[1][1] = T(0);
    double nmax = 0.0;

    for (int s = 0; s < nsteps; ++s) {
        const int slot = s % NS;
        const unsigned char* base = smem + slot * S::STAGE;
        if (!mbar_wait_bounded(&bar[slot], (uint32_t)((s / NS) & 1), err)) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
        const T* sx = reinterpret_cast<const T*>(base + S::XO);
        const T* ss = reinterpret_cast<const T*>(base + S::SO);
        const T* sb = reinterpret_cast<const T*>(base + S::BO);
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) P2[a][b] = sx[(ty + a) * BX + tx + b];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) S1[a][b] = ss[(ty + a) * BX + tx + b];
        const T bv = sb[ty * BX + tx + 1];
        const int k = kbeg - 2 + s;
        if (s >= 2 && active) {
            T v = T(0);
            if (!node_is_dirichlet(g, i, j, k)) {
                T acc = T(0), ssum = T(0);
                layer<T, ISO>(P1, P0, S0, g, acc, ssum);
                layer<T, ISO>(P1, P2, S1, g, acc, ssum);
                const T xc = P1[1][1];
                T ax;
                if (ISO) {
                    if constexpr (sizeof(T) == 8)
                        ax = (T)g.K[3] * fma(-4.0 * xc, ssum, acc);
                    else
                        ax = (T)g.K[3] * acc;
                } else {
                    ax = acc;
                }
                const T diag = (T)g.K[0] * ssum;
                if (MODE == 0) {
                    T rd;
                    if constexpr (sizeof(T) == 8) {
                        const double ad = fabs(diag);
                        rd = (ad > 1e-30 && ad < 1e30) ? (double)__frcp_rn((float)diag) : 1.0 / diag;
                    } else {
                        rd = __frcp_rn(diag);
                    }
                    v = xc + omega * (bv - ax) * rd;
                } else {
                    v = bv - ax;
                    if (norm) nmax = nanmax(nmax, fabs((double)v) * node_inv_volume(g, i, j, k));
                }
            }
            const long long p = pidx(g.sy, g.sz, i, j, k);
            if (has_alias(g, i, j, k))
                store_node(out, g, i, j, k, v);
            else
                out[p] = v;
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
        __syncthreads();  // every thread is done with this slot
        if (tid == 0 && s + NS < nsteps) {
            fence_proxy_async();
            issue(s + NS);
        }
    }
    if (abort_flag && tid == 0) {
        // drain the loads still in flight (bounded) before the CTA's shared memory goes away
        for (int q = 0; q < NS; ++q) (void)mbar_wait_bounded(&bar[q], 0, nullptr);
    }
    if (MODE == 1 && norm) {
        nmax = block_max(nmax);
        if (tid == 0) atomic_max_nonneg(norm, nmax);
    }
}

// ------------------------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
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
    auto fn = encode_fn();
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

bool sweep_supported(const NodalGeom& g) { return g.nu[0] >= 16 && g.nu[1] >= 4 && g.nu[2] >= 4; }

static int sm_count()
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
template <typename T, int MODE, bool ISO>
static int z_chunks(const NodalGeom& g, int xy_tiles)
{
    static int resident = 0;
    if (!resident) {
        using C = SweepCfg<T>;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_nodal_sweep<T, MODE, ISO>, C::TX * C::TY, 0) !=
                cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int slots = resident * sm_count();
    const int max_chunks = (g.nu[2] + 15) / 16;
    int best = 1;
    double best_eff = 0.0;
    for (int nz = 1; nz <= max_chunks; ++nz) {
        const int kchunk = (g.nu[2] + nz - 1) / nz;
        const int nzc = (g.nu[2] + kchunk - 1) / kchunk;
        const long long ctas = (long long)xy_tiles * nzc;
        const long long waves = (ctas + slots - 1) / slots;
        // efficiency: useful CTA slots over occupied ones, discounted by the 2 warm-up planes per chunk
        const double eff = (double)ctas / (double)(waves * slots) * (double)kchunk / (double)(kchunk + 2);
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = nzc;
        }
    }
    return best;
}

template <typename T, int MODE, bool ISO>
static void launch_sweep(const CUtensorMap& mx, const CUtensorMap& ms, const CUtensorMap& mb, const NodalGeom& g,
                         T* out, double omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using C = SweepCfg<T>;
    const int tx = (g.nu[0] + C::TX - 1) / C::TX, ty = (g.nu[1] + C::TY - 1) / C::TY;
    const int nz = z_chunks<T, MODE, ISO>(g, tx * ty);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    k_nodal_sweep<T, MODE, ISO><<<grid, dim3(C::TX, C::TY), 0, st>>>(mx, ms, mb, g, out, (T)omega, kchunk, err, norm);
}

template <typename T>
int nodal_sweep(const NodalGeom& g, int mode, const T* s, const T* x, const T* b, T* out, double omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    using S = SweepShape<T>;
    CUtensorMap mx, ms, mb;
    int rc = make_tensor_map(x, sizeof(T), g.sy, g.sz, g.count, S::BX, S::TY + 2, &mx);
    if (!rc) rc = make_tensor_map(s, sizeof(T), g.sy, g.sz, g.count, S::BX, S::TY + 1, &ms);
    if (!rc) rc = make_tensor_map(b, sizeof(T), g.sy, g.sz, g.count, S::BX, S::TY, &mb);
    if (rc) return rc;
    if (mode == 0) {
        if (g.iso)
            launch_sweep<T, 0, true>(mx, ms, mb, g, out, omega, err, norm, st);
        else
            launch_sweep<T, 0, false>(mx, ms, mb, g, out, omega, err, norm, st);
    } else {
        if (g.iso)
            launch_sweep<T, 1, true>(mx, ms, mb, g, out, omega, err, norm, st);
        else
            launch_sweep<T, 1, false>(mx, ms, mb, g, out, omega, err, norm, st);
    }
    return GBP_OK;
}

template int nodal_sweep<double>(const NodalGeom&, int, const double*, const double*, const double*, double*, double,
                                 unsigned*, unsigned long long*, cudaStream_t);
template int nodal_sweep<float>(const NodalGeom&, int, const float*, const float*, const float*, float*, double,
                                unsigned*, unsigned long long*, cudaStream_t);

}  // namespace gbp
