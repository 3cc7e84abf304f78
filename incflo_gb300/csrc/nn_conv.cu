// BF16 3x3x3 convolutions of the warm-start U-Net as implicit GEMMs on tcgen05.
//
// Forward / data-gradient kernel (k_conv): a persistent CTA walks output tiles of 128 consecutive
// rows of the zero-haloed channels-last grid. For each K step (input tensor, 16..64-channel chunk,
// tap) warp 0 issues two TMA loads into a ring stage: the 128-row activation box at row p0 + off(tap)
// (a K-major, swizzled A operand; rows outside the array read as zeros) and the N-row weight box of
// that tap (the B operand). Warp 1 issues the MMAs (M = 128, N = output channels, K = 16 per
// instruction) into one of two FP32 tensor-memory accumulators, so the epilogue of tile t overlaps
// the MMAs of tile t+1. Warps 2..5 read the accumulator with tcgen05.ld (one row per thread), apply
// bias + GELU (forward) or gradient accumulation + GELU derivative (backward), zero the halo rows
// and store BF16.
//
// Weight-gradient kernel (k_wgrad): dw[tap][co][ci] = sum_p gout[p][co] in[p + off(tap)][ci] is a GEMM
// with M = (taps x input channels) in blocks of 128, N = output channels and K = grid rows. Both
// operands arrive MN-major (channels contiguous) straight from the activation arrays by TMA; each CTA
// reduces one slice of rows in tensor memory and adds its FP32 partial into dw.
//
// Every mbarrier wait is bounded; a wait that runs out sets the error word, stops the CTA's loops,
// drains the copies and MMAs it issued and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <string>

#include "gbp_internal.cuh"
#include "nn.h"
#include "nn_tc.cuh"
#include "nodal_sweep.h"
#include "tma.cuh"

namespace gbp {
namespace nn {

namespace {

constexpr int kBM = 128;       // output rows per tile (MMA M)
constexpr int kThreads = 192;  // warp 0 TMA producer, warp 1 MMA issuer, warps 2..5 epilogue
constexpr int kMaxStages = 32;
constexpr int kWgradRows = 64;  // K rows per pipeline stage of the weight-gradient kernel

struct ConvParams {
    CUtensorMap amap[2];
    CUtensorMap wmap[2];
    int nin, ntaps, N, ntiles;
    int cb[2], nchunk[2], wc0[2];
    // K steps walk tap groups: a 3x3x3 convolution has 9 groups (dz, dy), each one activation box of
    // kBM + 2 rows shared by its 3 dx taps (tap q starts tap_row[q] rows into the box); a 1x1x1 one
    // has one group of one tap
    int ngroups, gtaps, a_rows, wbox_rows;
    int goff[9];
    int tap_row[3];
    int off[27];
    int X, Y, Z;
    long long PX, PXY, R;
    int nseg, flags;
    __nv_bfloat16* out[2];
    __nv_bfloat16* aux[2];
    int seg_c0[2], seg_nc[2];
    const float* bias;
    unsigned* err;
    int ns;
    uint32_t a_bytes, stage_bytes, tmem_cols, idesc;
};

__device__ __forceinline__ bool row_interior(long long p, int X, int Y, int Z, long long PX, long long PXY)
{
    const long long z = p / PXY;
    const long long rem = p - z * PXY;
    const long long y = rem / PX;
    const long long x = rem - y * PX;
    return x >= 1 && x <= X && y >= 1 && y <= Y && z >= 1 && z <= Z;
}

__device__ __forceinline__ void unpack16(const uint4 (&u)[2], float (&v)[16])
{
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u[0]);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float2 f = __bfloat1622float2(h[q]);
        v[2 * q] = f.x;
        v[2 * q + 1] = f.y;
    }
}

__device__ __forceinline__ void pack16(const float (&v)[16], uint4 (&u)[2])
{
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u[0]);
#pragma unroll
    for (int q = 0; q < 8; ++q) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
}

__device__ __forceinline__ void load16(const __nv_bfloat16* p, float (&v)[16])
{
    uint4 u[2];
    u[0] = *reinterpret_cast<const uint4*>(p);
    u[1] = *reinterpret_cast<const uint4*>(p + 8);
    unpack16(u, v);
}

__device__ __forceinline__ void store16(__nv_bfloat16* p, const float (&v)[16])
{
    uint4 u[2];
    pack16(v, u);
    *reinterpret_cast<uint4*>(p) = u[0];
    *reinterpret_cast<uint4*>(p + 8) = u[1];
}

__device__ __forceinline__ uint32_t aligned_smem_base(unsigned char* raw)
{
    return (smem_u32(raw) + 1023u) & ~1023u;
}

__global__ void __launch_bounds__(kThreads, 1) k_conv(const __grid_constant__ ConvParams P)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kMaxStages], empty[kMaxStages], accf[2], acce[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sbase = aligned_smem_base(smem_raw);
    unsigned char* sgen = smem_raw + (sbase - smem_u32(smem_raw));

    if (threadIdx.x == 0) {
        for (int s = 0; s < P.ns; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], 4);
        }
        mbar_init(&done, 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(&tmem_slot, 2 * P.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            for (int tile = blockIdx.x; tile < P.ntiles && !abort_flag; tile += gridDim.x) {
                const int p0 = tile * kBM;
                for (int i = 0; i < P.nin; ++i)
                    for (int j = 0; j < P.nchunk[i]; ++j)
                        for (int gq = 0; gq < P.ngroups; ++gq) {
                            const uint32_t s = it % P.ns;
                            if (it >= (uint32_t)P.ns && !mbar_wait_bounded(&empty[s], ((it / P.ns) + 1) & 1, P.err)) {
                                abort_flag = 1;
                                goto produced;
                            }
                            const uint32_t bytes = (uint32_t)(P.a_rows + P.gtaps * P.N) * P.cb[i] * 2u;
                            mbar_arrive_expect_tx(&full[s], bytes);
                            unsigned char* a = sgen + s * P.stage_bytes;
                            tma_load_2d(a, &P.amap[i], &full[s], j * P.cb[i], p0 + P.goff[gq]);
                            const int wrow0 = gq * P.gtaps * P.N;
                            for (int r = 0; r < P.gtaps * P.N; r += P.wbox_rows)
                                tma_load_2d(a + P.a_bytes + (uint32_t)r * P.cb[i] * 2u, &P.wmap[i], &full[s],
                                            P.wc0[i] + j * P.cb[i], wrow0 + r);
                            ++it;
                        }
            }
        produced:
            // drain: the last load into each stage must have landed before the CTA exits
            for (uint32_t s = 0; s < (uint32_t)P.ns && s < it; ++s) {
                const uint32_t last = it - 1 - ((it - 1 - s) % P.ns);
                (void)mbar_wait_bounded(&full[s], (last / P.ns) & 1, P.err);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t it = 0, tl = 0;
            for (int tile = blockIdx.x; tile < P.ntiles && !abort_flag; tile += gridDim.x, ++tl) {
                const uint32_t buf = tl & 1;
                if (tl >= 2 && !mbar_wait_bounded(&acce[buf], ((tl >> 1) + 1) & 1, P.err)) {
                    abort_flag = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t d = tmem + buf * P.tmem_cols;
                uint32_t acc = 0;
                for (int i = 0; i < P.nin; ++i) {
                    const uint32_t rowb = P.cb[i] * 2u;
                    const int swz = tc::swizzle_code((int)rowb);
                    for (int j = 0; j < P.nchunk[i]; ++j)
                        for (int gq = 0; gq < P.ngroups; ++gq) {
                            const uint32_t s = it % P.ns;
                            if (!mbar_wait_bounded(&full[s], (it / P.ns) & 1, P.err)) {
                                abort_flag = 1;
                                goto issued;
                            }
                            tc::fence_after_sync();
                            const uint32_t a = sbase + s * P.stage_bytes, b = a + P.a_bytes;
                            for (int q = 0; q < P.gtaps; ++q) {
                                // the tap's 128 rows start tap_row[q] rows into the shared box; the
                                // swizzle follows the absolute shared-memory address, so a start on
                                // any row of the 8-row pattern reads the rows TMA wrote there
                                const uint32_t aq = a + (uint32_t)P.tap_row[q] * rowb;
                                const uint32_t bq = b + (uint32_t)(q * P.N) * rowb;
                                for (uint32_t kk = 0; kk < rowb / 32u; ++kk) {
                                    tc::mma_bf16(d, tc::sdesc(aq + 32u * kk, 16, 8 * rowb, swz),
                                                 tc::sdesc(bq + 32u * kk, 16, 8 * rowb, swz), P.idesc, acc);
                                    acc = 1;
                                }
                            }
                            tc::mma_commit(&empty[s]);
                            ++it;
                        }
                }
                tc::mma_commit(&accf[buf]);
            }
        issued:
            tc::mma_commit(&done);
            (void)mbar_wait_bounded(&done, 0, P.err);
        }
    } else {
        const int q = warp & 3;  // tensor-memory lane quarter this warp may read
        const int row = q * 32 + lane;
        uint32_t tl = 0;
        for (int tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x, ++tl) {
            const uint32_t buf = tl & 1;
            if (!mbar_wait_bounded(&accf[buf], (tl >> 1) & 1, P.err)) abort_flag = 1;
            if (__any_sync(0xffffffffu, abort_flag)) break;
            tc::fence_after_sync();
            const long long p = (long long)tile * kBM + row;
            const bool valid = p < P.R;
            const bool inside = valid && row_interior(p, P.X, P.Y, P.Z, P.PX, P.PXY);
            const uint32_t taddr = tmem + buf * P.tmem_cols + ((uint32_t)(q * 32) << 16);
            for (int sg = 0; sg < P.nseg; ++sg) {
                const int nc = P.seg_nc[sg], c0 = P.seg_c0[sg];
                __nv_bfloat16* orow = P.out[sg] + p * nc;
                __nv_bfloat16* arow = P.aux[sg] ? P.aux[sg] + p * nc : nullptr;
                for (int c = 0; c < nc; c += 16) {
                    float v[16];
                    tc::tmem_ld16(taddr + (uint32_t)(c0 + c), v);
                    if (!valid) continue;
                    if (!inside) {
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] = 0.f;
                        store16(orow + c, v);
                        if (arow && (P.flags & kGelu)) store16(arow + c, v);
                        continue;
                    }
                    if (P.bias) {
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] += __ldg(P.bias + c0 + c + e);
                    }
                    if (P.flags & kAccum) {
                        float o[16];
                        load16(orow + c, o);
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] += o[e];
                    }
                    if (P.flags & kDGelu) {
                        float a[16];
                        load16(arow + c, a);
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] *= dgelu_f(a[e]);
                    }
                    if (P.flags & kGelu) {
                        if (arow) store16(arow + c, v);
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] = gelu_f(v[e]);
                    }
                    store16(orow + c, v);
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[buf]);
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 2 * P.tmem_cols);
    }
}

// ------------------------------------------------------------------ weight gradient
struct WgradParams {
    CUtensorMap amap;  // input activations, box {ca, kWgradRows}
    CUtensorMap gmap;  // output gradient, box {cg, kWgradRows}
    int ca, natom_a;   // channels per A atom (<= 64); atoms per 128-row M tile
    int cg, natom_g;   // channels per B atom; atoms (N = natom_g * cg = cout)
    int cin, ci0, cin_tot, cout, ntaps;
    int off[27];
    int k_steps_per_cta, k_steps_total;
    float* dw;
    unsigned* err;
    int ns;
    uint32_t a_bytes, stage_bytes, tmem_cols, idesc;
};

__global__ void __launch_bounds__(kThreads, 1) k_wgrad(const __grid_constant__ WgradParams P)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kMaxStages], empty[kMaxStages], accf;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t sbase = aligned_smem_base(smem_raw);
    unsigned char* sgen = smem_raw + (sbase - smem_u32(smem_raw));
    const int mt = blockIdx.x;  // M tile: taps [mt * taps_per_tile, ...)
    const int taps_per_tile = kBM / P.cin >= 1 ? kBM / P.cin : 1;
    const int k_begin = blockIdx.y * P.k_steps_per_cta;
    const int k_end = min(P.k_steps_total, k_begin + P.k_steps_per_cta);

    if (threadIdx.x == 0) {
        for (int s = 0; s < P.ns; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&accf, 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(&tmem_slot, P.tmem_cols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t a_atom_bytes = (uint32_t)kWgradRows * P.ca * 2u;
    const uint32_t g_atom_bytes = (uint32_t)kWgradRows * P.cg * 2u;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            for (int ks = k_begin; ks < k_end; ++ks, ++it) {
                const uint32_t s = it % P.ns;
                if (it >= (uint32_t)P.ns && !mbar_wait_bounded(&empty[s], ((it / P.ns) + 1) & 1, P.err)) {
                    abort_flag = 1;
                    break;
                }
                const int q0 = ks * kWgradRows;
                mbar_arrive_expect_tx(&full[s], a_atom_bytes * P.natom_a + g_atom_bytes * P.natom_g);
                unsigned char* a = sgen + s * P.stage_bytes;
                const int chunks = P.cin / P.ca;
                for (int m = 0; m < P.natom_a; ++m) {
                    const int tap = mt * taps_per_tile + m / chunks;
                    const int ch = m % chunks;
                    // taps past the last one load a valid tap (their rows of D are never stored)
                    const int tt = tap < P.ntaps ? tap : P.ntaps - 1;
                    tma_load_2d(a + m * a_atom_bytes, &P.amap, &full[s], ch * P.ca, q0 + P.off[tt]);
                }
                for (int m = 0; m < P.natom_g; ++m)
                    tma_load_2d(a + P.a_bytes + m * g_atom_bytes, &P.gmap, &full[s], m * P.cg, q0);
            }
            for (uint32_t s = 0; s < (uint32_t)P.ns && s < it; ++s) {
                const uint32_t last = it - 1 - ((it - 1 - s) % P.ns);
                (void)mbar_wait_bounded(&full[s], (last / P.ns) & 1, P.err);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const int swa = tc::swizzle_code(P.ca * 2), swg = tc::swizzle_code(P.cg * 2);
            uint32_t it = 0, acc = 0;
            for (int ks = k_begin; ks < k_end; ++ks, ++it) {
                const uint32_t s = it % P.ns;
                if (abort_flag || !mbar_wait_bounded(&full[s], (it / P.ns) & 1, P.err)) {
                    abort_flag = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t a = sbase + s * P.stage_bytes, b = a + P.a_bytes;
                // MN-major swizzled operands: MN atoms at LBO = atom bytes, 8-row K groups at SBO
                for (int kk = 0; kk < kWgradRows / 16; ++kk) {
                    const uint64_t ad = tc::sdesc(a + kk * 16u * P.ca * 2u, a_atom_bytes, 8u * P.ca * 2u, swa);
                    const uint64_t bd = tc::sdesc(b + kk * 16u * P.cg * 2u, g_atom_bytes, 8u * P.cg * 2u, swg);
                    tc::mma_bf16(tmem, ad, bd, P.idesc, acc);
                    acc = 1;
                }
                tc::mma_commit(&empty[s]);
            }
            tc::mma_commit(&accf);
        }
    } else {
        const int q = warp & 3;
        const int row = q * 32 + lane;  // M row = (tap in tile, input channel)
        const bool ok = mbar_wait_bounded(&accf, 0, P.err);
        tc::fence_after_sync();
        const int tap = mt * taps_per_tile + row / P.cin;
        const int ci = row % P.cin;
        const bool store = ok && !abort_flag && k_end > k_begin && tap < P.ntaps && row < taps_per_tile * P.cin;
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16);
        for (int c = 0; c < P.cout; c += 16) {
            float v[16];
            tc::tmem_ld16(taddr + (uint32_t)c, v);
            if (!store) continue;
            float* dst = P.dw + ((long long)tap * P.cout + c) * P.cin_tot + P.ci0 + ci;
#pragma unroll
            for (int e = 0; e < 16; ++e) atomicAdd(dst + (long long)e * P.cin_tot, v[e]);
        }
    }

    tc::fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, P.tmem_cols);
    }
}

// ------------------------------------------------------------------ host side
int encode_rows(const void* base, int C, long long R, int box_c, int box_rows, CUtensorMap* m)
{
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is unavailable from the driver");
        return GBP_CUDA_ERROR;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)C, (cuuint64_t)R};
    const cuuint64_t strides[1] = {(cuuint64_t)C * 2};
    const cuuint32_t box[2] = {(cuuint32_t)box_c, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUtensorMapSwizzle swz = box_c == 64   ? CU_TENSOR_MAP_SWIZZLE_128B
                                   : box_c == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                 : CU_TENSOR_MAP_SWIZZLE_32B;
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed for a BF16 activation map (code " + std::to_string((int)r) + ")");
        return GBP_CUDA_ERROR;
    }
    return GBP_OK;
}

int chunk_of(int c) { return c >= 64 ? 64 : c; }

bool channels_ok(int c) { return c == 16 || c == 32 || (c >= 64 && c % 64 == 0); }

uint32_t pow2_cols(int n)
{
    uint32_t c = 32;
    while (c < (uint32_t)n) c <<= 1;
    return c;
}

void tap_offsets(const Grid3& g, int ntaps, int flip, int* off)
{
    if (ntaps == 1) {
        off[0] = 0;
        return;
    }
    int t = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx, ++t) {
                const long long o = dz * g.PXY + dy * g.PX + dx;
                off[t] = (int)(flip ? -o : o);
            }
}

}  // namespace

int conv3d(const ConvLaunch& L, cudaStream_t st)
{
    if (L.nin < 1 || L.nin > 2 || (L.ntaps != 1 && L.ntaps != 27) || L.N < 16 || L.N > 256 || L.N % 16 ||
        L.nseg < 1 || L.nseg > 2 || !L.w || L.g.R <= 0 || L.g.R > (1ll << 30)) {
        set_error("conv3d: bad launch shape");
        return GBP_BAD_ARG;
    }
    ConvParams P;
    memset(&P, 0, sizeof(P));
    int cin_tot = 0, cbmax = 16;
    for (int i = 0; i < L.nin; ++i) {
        if (!L.in[i] || !channels_ok(L.cin[i]) || (reinterpret_cast<uintptr_t>(L.in[i]) & 15)) {
            set_error("conv3d: input channels must be 16, 32 or a multiple of 64, data 16-byte aligned");
            return GBP_BAD_ARG;
        }
        P.cb[i] = chunk_of(L.cin[i]);
        P.nchunk[i] = L.cin[i] / P.cb[i];
        P.wc0[i] = cin_tot;
        cin_tot += L.cin[i];
        cbmax = std::max(cbmax, P.cb[i]);
    }
    int segsum = 0;
    for (int s = 0; s < L.nseg; ++s) {
        if (!L.out[s] || L.seg_c[s] < 16 || L.seg_c[s] % 16 || (reinterpret_cast<uintptr_t>(L.out[s]) & 15) ||
            (reinterpret_cast<uintptr_t>(L.aux[s]) & 15) || (!L.aux[s] && (L.flags & kDGelu))) {
            set_error("conv3d: bad output segment");
            return GBP_BAD_ARG;
        }
        P.out[s] = L.out[s];
        P.aux[s] = L.aux[s];
        P.seg_c0[s] = segsum;
        P.seg_nc[s] = L.seg_c[s];
        segsum += L.seg_c[s];
    }
    if (segsum != L.N) {
        set_error("conv3d: output segments must cover N channels");
        return GBP_BAD_ARG;
    }
    P.nin = L.nin;
    P.ntaps = L.ntaps;
    P.N = L.N;
    P.ntiles = (int)((L.g.R + kBM - 1) / kBM);
    tap_offsets(L.g, L.ntaps, L.flip, P.off);
    if (L.ntaps == 27) {
        P.ngroups = 9;
        P.gtaps = 3;
        P.a_rows = kBM + 2;
        for (int gq = 0; gq < 9; ++gq) P.goff[gq] = std::min(P.off[3 * gq], P.off[3 * gq + 2]);
        // dx = -1, 0, +1 of a group sit at rows +0, +1, +2 of the box (+2, +1, +0 for flipped taps)
        for (int q = 0; q < 3; ++q) P.tap_row[q] = P.off[q] - P.goff[0];
    } else {
        P.ngroups = 1;
        P.gtaps = 1;
        P.a_rows = kBM;
        P.goff[0] = P.off[0];
        P.tap_row[0] = 0;
    }
    P.wbox_rows = P.gtaps * L.N <= 256 ? P.gtaps * L.N : L.N;
    for (int i = 0; i < L.nin; ++i) {
        int rc = encode_rows(L.in[i], L.cin[i], L.g.R, P.cb[i], P.a_rows, &P.amap[i]);
        if (!rc) rc = encode_rows(L.w, cin_tot, (long long)L.ntaps * L.N, P.cb[i], P.wbox_rows, &P.wmap[i]);
        if (rc) return rc;
    }
    P.X = L.g.X;
    P.Y = L.g.Y;
    P.Z = L.g.Z;
    P.PX = L.g.PX;
    P.PXY = L.g.PXY;
    P.R = L.g.R;
    P.nseg = L.nseg;
    P.flags = L.flags;
    P.bias = L.bias;
    P.err = L.err;
    P.a_bytes = ((uint32_t)P.a_rows * cbmax * 2u + 1023u) & ~1023u;
    P.stage_bytes = P.a_bytes + (((uint32_t)(P.gtaps * L.N) * cbmax * 2u + 1023u) & ~1023u);
    P.tmem_cols = pow2_cols(L.N);
    P.idesc = tc::idesc_bf16(kBM, L.N, 0, 0);
    const int max_smem = 200 * 1024;
    P.ns = std::min(kMaxStages, (int)((max_smem - 1024) / P.stage_bytes));
    if (P.ns < 2) {
        set_error("conv3d: stage does not fit in shared memory");
        return GBP_BAD_ARG;
    }
    const size_t smem = (size_t)P.ns * P.stage_bytes + 1024;
    static bool attr_set = false;
    if (!attr_set) {
        GBP_CUDA(cudaFuncSetAttribute(k_conv, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_set = true;
    }
    const int grid = std::min(P.ntiles, sm_count_cached());
    k_conv<<<grid, kThreads, smem, st>>>(P);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int conv3d_wgrad(const WgradLaunch& L, cudaStream_t st)
{
    if (!L.in || !L.gout || !L.dw || (L.ntaps != 1 && L.ntaps != 27) || !channels_ok(L.cin) || L.cin > 128 ||
        !channels_ok(L.cout) || L.cout > 128 || L.ci0 < 0 || L.ci0 + L.cin > L.cin_tot || L.g.R <= 0 ||
        L.g.R > (1ll << 30)) {
        set_error("conv3d_wgrad: bad launch shape");
        return GBP_BAD_ARG;
    }
    WgradParams P;
    memset(&P, 0, sizeof(P));
    P.ca = chunk_of(L.cin);
    P.cg = chunk_of(L.cout);
    const int taps_per_tile = std::max(1, 128 / L.cin);
    P.natom_a = taps_per_tile * L.cin / P.ca;  // = 128 / ca
    P.natom_g = L.cout / P.cg;
    int rc = encode_rows(L.in, L.cin, L.g.R, P.ca, kWgradRows, &P.amap);
    if (!rc) rc = encode_rows(L.gout, L.cout, L.g.R, P.cg, kWgradRows, &P.gmap);
    if (rc) return rc;
    P.cin = L.cin;
    P.ci0 = L.ci0;
    P.cin_tot = L.cin_tot;
    P.cout = L.cout;
    P.ntaps = L.ntaps;
    tap_offsets(L.g, L.ntaps, 0, P.off);
    P.dw = L.dw;
    P.err = L.err;
    P.a_bytes = (uint32_t)kWgradRows * 128u * 2u;
    P.stage_bytes = P.a_bytes + (uint32_t)kWgradRows * L.cout * 2u;
    P.stage_bytes = (P.stage_bytes + 1023u) & ~1023u;
    P.tmem_cols = pow2_cols(L.cout);
    P.idesc = tc::idesc_bf16(kBM, L.cout, 1, 1);
    P.ns = std::min(kMaxStages, (int)((200 * 1024 - 1024) / P.stage_bytes));
    const int mtiles = (L.ntaps + taps_per_tile - 1) / taps_per_tile;
    P.k_steps_total = (int)((L.g.R + kWgradRows - 1) / kWgradRows);
    const int want = std::max(1, 2 * sm_count_cached() / mtiles);
    P.k_steps_per_cta = std::max(8, (P.k_steps_total + want - 1) / want);
    const int splits = (P.k_steps_total + P.k_steps_per_cta - 1) / P.k_steps_per_cta;
    static bool attr_set = false;
    if (!attr_set) {
        GBP_CUDA(cudaFuncSetAttribute(k_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_set = true;
    }
    const size_t smem = (size_t)P.ns * P.stage_bytes + 1024;
    k_wgrad<<<dim3(mtiles, splits), kThreads, smem, st>>>(P);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

}  // namespace nn
}  // namespace gbp
