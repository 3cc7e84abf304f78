// FP32 level sweep of the nodal operator (Jacobi sweep or residual), the HBM-bound hot kernel of the
// FP32 V-cycles of the mixed-precision solve.
//
// Pipeline: a CTA owns 64 x 16 nodes in (x, y) and marches up a chunk of z planes. One producer
// warp streams, per plane, x (plane k+1, one-node halo), sigma (cell layer k, one-cell halo) and b
// (plane k) into a 4-slot shared-memory ring with cp.async.bulk.tensor; each slot has a "full"
// mbarrier (TMA transaction bytes) and an "empty" mbarrier (one arrival per consumer warp). The 16
// consumer warps never synchronise with each other: a warp waits on "full", copies its window of
// the slot into registers, releases the slot on "empty" and computes. No HBM array is read twice.
//
// Each consumer thread owns two x-adjacent nodes of one row. Per plane it keeps only two register
// windows (planes k and k+1) and two cell layers: the coupling of node (i,j,k+1) to plane k through
// cell layer (k,k+1) is evaluated one plane early and carried as a scalar, so planes swap roles every
// step and the loop is unrolled by two with no register moves.
//
// Isotropic Q1 operator, written per neighbour with the summed sigma of the cells shared by the two
// nodes (x/y-edge pairs, in-plane diagonals below+above, corners single), always as differences to
// the centre so FP32 rounding scales with the local variation of x, not with x itself.
#include <cuda.h>

#include "gbp_internal.cuh"
#include "nodal_sweep.h"
#include "tma.cuh"

namespace gbp {

namespace {

constexpr int NX = 64, TY = 16, NS = 4, W = 4;
constexpr int CONSUMERS = TY;                // one consumer warp per row
constexpr int THREADS = 32 * (CONSUMERS + 1);  // + one producer warp
constexpr int BXX = 72;                      // x box: nodes x0-4 .. x0+67 (69 used), 16-byte rows
constexpr int BXS = 68;                      // sigma box: cells x0-4 .. x0+63
constexpr int BXB = 64;                      // b box: nodes x0 .. x0+63
constexpr int XB = (TY + 2) * BXX * 4, SB = (TY + 1) * BXS * 4, BB = TY * BXB * 4;
constexpr int SO = (XB + 127) / 128 * 128;
constexpr int BO = SO + (SB + 127) / 128 * 128;
constexpr int STAGE = BO + (BB + 127) / 128 * 128;
constexpr int SMEM = NS * STAGE;
constexpr uint32_t TX_BYTES = XB + SB + BB;

struct Consts {
    float k0, k3, omega;
};

struct Win {
    float p[3][W];  // x window of one plane: rows j-1..j+1, columns = nodes i0-1 .. i0+2
};
struct Lay {
    float s[2][W - 1];  // sigma of one cell layer: rows j-1, j; columns = cells i0-1 .. i0+1
};

__device__ __forceinline__ void load_window(const float* sx, int ty, Win& w)
{
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float* row = sx + (ty + r) * BXX;
        w.p[r][0] = row[0];
        const float2 m = *reinterpret_cast<const float2*>(row + 1);
        w.p[r][1] = m.x;
        w.p[r][2] = m.y;
        w.p[r][3] = row[3];
    }
}

__device__ __forceinline__ void load_layer(const float* ss, int ty, Lay& l)
{
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const float* row = ss + (ty + r) * BXS;
        l.s[r][0] = row[0];
        const float2 m = *reinterpret_cast<const float2*>(row + 1);
        l.s[r][1] = m.x;
        l.s[r][2] = m.y;
    }
}

// Couplings of the centre node (window column c of plane `ctr`) to the plane `far` through cell layer
// `L` (the layer between them): edge pairs and corners, as differences to the centre value xc.
__device__ __forceinline__ float far_terms(const Win& far, const Lay& L, int c, float xc, float& ssum_layer)
{
    const float ax0 = L.s[0][c - 1] + L.s[1][c - 1], ax1 = L.s[0][c] + L.s[1][c];  // x-edge pairs
    const float ay0 = L.s[0][c - 1] + L.s[0][c], ay1 = L.s[1][c - 1] + L.s[1][c];  // y-edge pairs
    ssum_layer = ax0 + ax1;
    float acc = ax0 * (far.p[1][c - 1] - xc);
    acc = fmaf(ax1, far.p[1][c + 1] - xc, acc);
    acc = fmaf(ay0, far.p[0][c] - xc, acc);
    acc = fmaf(ay1, far.p[2][c] - xc, acc);
    acc = fmaf(L.s[0][c - 1], far.p[0][c - 1] - xc, acc);
    acc = fmaf(L.s[0][c], far.p[0][c + 1] - xc, acc);
    acc = fmaf(L.s[1][c - 1], far.p[2][c - 1] - xc, acc);
    acc = fmaf(L.s[1][c], far.p[2][c + 1] - xc, acc);
    return acc;
}

// in-plane face diagonals of the centre node: weight = sigma below + sigma above
__device__ __forceinline__ float inplane_terms(const Win& ctr, const Lay& Lb, const Lay& La, int c, float xc)
{
    float acc = (Lb.s[0][c - 1] + La.s[0][c - 1]) * (ctr.p[0][c - 1] - xc);
    acc = fmaf(Lb.s[0][c] + La.s[0][c], ctr.p[0][c + 1] - xc, acc);
    acc = fmaf(Lb.s[1][c - 1] + La.s[1][c - 1], ctr.p[2][c - 1] - xc, acc);
    acc = fmaf(Lb.s[1][c] + La.s[1][c], ctr.p[2][c + 1] - xc, acc);
    return acc;
}

template <int MODE>
__global__ void __launch_bounds__(THREADS, 1)
    k_sweep32(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap ms,
              const __grid_constant__ CUtensorMap mb, NodalGeom g, float* __restrict__ out, Consts cst, int kchunk,
              unsigned* err, unsigned long long* norm)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[NS], empty[NS];

    const int lane = threadIdx.x, warp = threadIdx.y;
    const int x0 = blockIdx.x * NX, y0 = blockIdx.y * TY;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    const int nsteps = kend - kbeg + 2;

    if (warp == 0 && lane == 0) {
        for (int q = 0; q < NS; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], CONSUMERS);
        }
        mbar_fence_init();
    }
    __syncthreads();

    if (warp == CONSUMERS) {
        // ---------------------------------------------------------------- producer warp
        if (lane == 0) {
            bool ok = true;
            for (int s = 0; s < nsteps && ok; ++s) {
                const int slot = s % NS;
                if (s >= NS) ok = mbar_wait_bounded(&empty[slot], (uint32_t)(((s / NS) - 1) & 1), err);
                if (!ok) break;
                unsigned char* base = smem + slot * STAGE;
                const int k = kbeg - 2 + s;
                mbar_arrive_expect_tx(&full[slot], TX_BYTES);
                tma_load_3d(base, &mx, &full[slot], x0, y0, k + 2);                 // x plane k+1, rows j-1..
                tma_load_3d(base + SO, &ms, &full[slot], x0, y0, k + 1);            // sigma layer k, rows j-1..
                tma_load_3d(base + BO, &mb, &full[slot], x0 + kOX, y0 + 1, k + 1);  // b plane k, rows j..
            }
            // the loads already issued complete before the CTA exits: wait for them (bounded)
            if (!ok)
                for (int q = 0; q < NS; ++q) (void)mbar_wait_bounded(&full[q], 0, nullptr);
        }
        return;
    }

    // -------------------------------------------------------------------- consumer warps
    const int ty = warp;
    const int i0 = x0 + 2 * lane, j = y0 + ty;
    const bool actA = i0 < g.nu[0] && j < g.nu[1], actB = i0 + 1 < g.nu[0] && j < g.nu[1];
    const bool dirA = (g.dlo[0] && i0 == 0) || (g.dhi[0] && i0 == g.n[0]) || (g.dlo[1] && j == 0) ||
                      (g.dhi[1] && j == g.n[1]);
    const bool dirB = (g.dlo[0] && i0 + 1 == 0) || (g.dhi[0] && i0 + 1 == g.n[0]) || (g.dlo[1] && j == 0) ||
                      (g.dhi[1] && j == g.n[1]);
    const bool aliA = (g.per[0] && (i0 <= 1 || i0 == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1));
    const bool aliB = (g.per[0] && (i0 + 1 <= 1 || i0 + 1 == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1));
    float* optr = out + pidx(g.sy, g.sz, i0, j, kbeg);

    Win WA, WB;
    Lay LA, LB;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < W; ++q) WA.p[r][q] = WB.p[r][q] = 0.f;
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int q = 0; q < W - 1; ++q) LA.s[r][q] = LB.s[r][q] = 0.f;
    float carryA = 0.f, carryB = 0.f, sbA = 0.f, sbB = 0.f;  // below-layer coupling and sigma sum
    float nmax = 0.f;
    bool ok = true;

    // one plane: ctr = plane k (loaded last step), nxt <- plane k+1, lb = layer k-1 (last step), la <- layer k
    auto step = [&](Win& ctr, Win& nxt, Lay& lb, Lay& la, int s) {
        const int slot = s % NS;
        if (!mbar_wait_bounded(&full[slot], (uint32_t)((s / NS) & 1), err)) {
            ok = false;
            return;
        }
        const unsigned char* base = smem + slot * STAGE;
        load_window(reinterpret_cast<const float*>(base) + 2 * lane + 3, ty, nxt);
        load_layer(reinterpret_cast<const float*>(base + SO) + 2 * lane + 3, ty, la);
        const float2 bv = *reinterpret_cast<const float2*>(reinterpret_cast<const float*>(base + BO) + ty * BXB + 2 * lane);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);

        const int k = kbeg - 2 + s;
        const float xa = ctr.p[1][1], xb = ctr.p[1][2];
        float saA, saB;
        const float accA = carryA + inplane_terms(ctr, lb, la, 1, xa) + far_terms(nxt, la, 1, xa, saA);
        const float accB = carryB + inplane_terms(ctr, lb, la, 2, xb) + far_terms(nxt, la, 2, xb, saB);
        // coupling of the node above (plane k+1) to this plane through layer k, carried one plane
        float dumA, dumB;
        const float nxtA = far_terms(ctr, la, 1, nxt.p[1][1], dumA);
        const float nxtB = far_terms(ctr, la, 2, nxt.p[1][2], dumB);
        if (s >= 2 && actA) {
            const float axA = cst.k3 * accA, axB = cst.k3 * accB;
            float vA, vB;
            if (MODE == 0) {
                vA = fmaf(cst.omega * (bv.x - axA), __frcp_rn(cst.k0 * (sbA + saA)), xa);
                vB = fmaf(cst.omega * (bv.y - axB), __frcp_rn(cst.k0 * (sbB + saB)), xb);
            } else {
                vA = bv.x - axA;
                vB = bv.y - axB;
            }
            const bool dk = (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]);
            if (dk || dirA) vA = 0.f;
            if (dk || dirB || !actB) vB = 0.f;
            if (MODE == 1 && norm) {
                nmax = fmaxf(nmax, fabsf(vA) * (float)node_inv_volume(g, i0, j, k));
                if (actB) nmax = fmaxf(nmax, fabsf(vB) * (float)node_inv_volume(g, i0 + 1, j, k));
                if (vA != vA || vB != vB) nmax = __int_as_float(0x7fc00000);
            }
            const bool ak = g.per[2] && (k <= 1 || k == g.n[2] - 1);
            if (actB && !(ak || aliA || aliB)) {
                *reinterpret_cast<float2*>(optr) = make_float2(vA, vB);
            } else {
                if (ak || aliA)
                    store_node(out, g, i0, j, k, vA);
                else
                    optr[0] = vA;
                if (actB) {
                    if (ak || aliB)
                        store_node(out, g, i0 + 1, j, k, vB);
                    else
                        optr[1] = vB;
                }
            }
        }
        if (s >= 2) optr += g.sz;
        carryA = nxtA;
        carryB = nxtB;
        sbA = saA;
        sbB = saB;
    };

    int s = 0;
    for (; s + 1 < nsteps && ok; s += 2) {
        step(WA, WB, LA, LB, s);
        if (!ok) break;
        step(WB, WA, LB, LA, s + 1);
    }
    if (ok && s < nsteps) step(WA, WB, LA, LB, s);

    if (MODE == 1 && norm) {
        // warp-level max, one atomic per warp (consumers only; the producer warp has returned)
        float m = nmax;
        for (int o = 16; o > 0; o >>= 1) {
            const float v = __shfl_xor_sync(0xffffffffu, m, o);
            m = (m != m || v != v) ? __int_as_float(0x7fc00000) : fmaxf(m, v);
        }
        if (lane == 0) atomic_max_nonneg(norm, (double)m);
    }
}

template <int MODE>
int launch(const CUtensorMap& mx, const CUtensorMap& ms, const CUtensorMap& mb, const NodalGeom& g, float* out,
           float omega, unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    static int resident = 0;
    if (!resident) {
        cudaFuncSetAttribute(k_sweep32<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_sweep32<MODE>, THREADS, SMEM) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + NX - 1) / NX, ty = (g.nu[1] + TY - 1) / TY;
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    const Consts c{(float)g.K[0], (float)g.K[3], omega};
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    k_sweep32<MODE><<<grid, dim3(32, CONSUMERS + 1), SMEM, st>>>(mx, ms, mb, g, out, c, kchunk, err, norm);
    return GBP_OK;
}

}  // namespace

int sweep32_run(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    CUtensorMap mx, ms, mb;
    int rc = make_tensor_map(x, 4, g.sy, g.sz, g.count, BXX, TY + 2, &mx);
    if (!rc) rc = make_tensor_map(s, 4, g.sy, g.sz, g.count, BXS, TY + 1, &ms);
    if (!rc) rc = make_tensor_map(b, 4, g.sy, g.sz, g.count, BXB, TY, &mb);
    if (rc) return rc;
    return mode == 0 ? launch<0>(mx, ms, mb, g, out, omega, err, norm, st)
                     : launch<1>(mx, ms, mb, g, out, omega, err, norm, st);
}

}  // namespace gbp
