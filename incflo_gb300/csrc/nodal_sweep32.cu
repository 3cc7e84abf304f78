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
#include <stdlib.h>

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

// ----------------------------------------------------------------------------------------------
// Register-queue z-march without shared memory: one node per thread, 32 x 8 threads per CTA, all
// loads through the read-only path (the 3x3 windows of neighbouring threads overlap in L1). High
// occupancy (no shared memory, few registers) hides the latency that the TMA pipeline cannot at
// one CTA per SM. Same carried-coupling formulation as above; accumulations split in two chains.
constexpr int ZX = 32, ZY = 8;

struct Win1 {
    float p[3][3];
};
struct Lay1 {
    float s[2][2];
};

__device__ __forceinline__ void far1(const Win1& far, const Lay1& L, float xc, float& acc0, float& acc1, float& ssum)
{
    const float ax0 = L.s[0][0] + L.s[1][0], ax1 = L.s[0][1] + L.s[1][1];
    const float ay0 = L.s[0][0] + L.s[0][1], ay1 = L.s[1][0] + L.s[1][1];
    ssum = ax0 + ax1;
    acc0 = fmaf(ax0, far.p[1][0] - xc, acc0);
    acc1 = fmaf(ax1, far.p[1][2] - xc, acc1);
    acc0 = fmaf(ay0, far.p[0][1] - xc, acc0);
    acc1 = fmaf(ay1, far.p[2][1] - xc, acc1);
    acc0 = fmaf(L.s[0][0], far.p[0][0] - xc, acc0);
    acc1 = fmaf(L.s[0][1], far.p[0][2] - xc, acc1);
    acc0 = fmaf(L.s[1][0], far.p[2][0] - xc, acc0);
    acc1 = fmaf(L.s[1][1], far.p[2][2] - xc, acc1);
}

template <int MODE>
__global__ void __launch_bounds__(ZX* ZY) k_zmarch32(NodalGeom g, const float* __restrict__ sg, const float* __restrict__ xin,
                                                     const float* __restrict__ bin, float* __restrict__ out, Consts cst,
                                                     int kchunk, unsigned long long* norm)
{
    const int i = blockIdx.x * ZX + threadIdx.x, j = blockIdx.y * ZY + threadIdx.y;
    const int kbeg = blockIdx.z * kchunk;
    // inactive threads march nothing but still take part in the block reduction below
    const int kend = (i < g.nu[0] && j < g.nu[1]) ? min(kbeg + kchunk, g.nu[2]) : kbeg;
    const long long sy = g.sy, sz = g.sz;
    const bool dxy = (g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]);
    const bool axy = (g.per[0] && (i <= 1 || i == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1));
    // node (i,j,k) at c0 + k*sz; the window of plane q starts at node (i-1, j-1, q); the cell layer q
    // (between node planes q and q+1) starts at cell (i-1, j-1, q)
    const long long c0 = pidx(sy, sz, i, j, 0);
    const float* xw = xin + c0 - 1 - sy;
    const float* sw = sg + c0 - 1 - sy;
    auto load_win = [&](int q, Win1& w) {
        const float* p = xw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) w.p[r][c] = __ldg(p + r * sy + c);
    };
    auto load_lay = [&](int q, Lay1& l) {
        const float* p = sw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int c = 0; c < 2; ++c) l.s[r][c] = __ldg(p + r * sy + c);
    };
    Win1 WA, WB;
    Lay1 LA, LB;
    float carry = 0.f, sb = 0.f;
    if (kend > kbeg) {
        // prologue: plane kbeg-1 and kbeg, layer kbeg-1, and the coupling of node kbeg to plane kbeg-1
        load_win(kbeg - 1, WA);
        load_win(kbeg, WB);
        load_lay(kbeg - 1, LA);
        float carry0 = 0.f, carry1 = 0.f;
        far1(WA, LA, WB.p[1][1], carry0, carry1, sb);
        carry = carry0 + carry1;
    }
    float nmax = 0.f;
    float* op = out + c0 + (long long)kbeg * sz;
    const float* bp = bin + c0 + (long long)kbeg * sz;

    // ctr = plane k, nxt <- plane k+1, lb = layer k-1, la <- layer k
    auto step = [&](Win1& ctr, Win1& nxt, Lay1& lb, Lay1& la, int k) {
        load_win(k + 1, nxt);
        load_lay(k, la);
        const float bv = __ldg(bp);
        const float xc = ctr.p[1][1];
        float a0 = carry, a1 = 0.f, sa;
        // in-plane diagonals (sigma below + above)
        a0 = fmaf(lb.s[0][0] + la.s[0][0], ctr.p[0][0] - xc, a0);
        a1 = fmaf(lb.s[0][1] + la.s[0][1], ctr.p[0][2] - xc, a1);
        a0 = fmaf(lb.s[1][0] + la.s[1][0], ctr.p[2][0] - xc, a0);
        a1 = fmaf(lb.s[1][1] + la.s[1][1], ctr.p[2][2] - xc, a1);
        far1(nxt, la, xc, a0, a1, sa);
        // coupling of node k+1 to this plane through layer k, carried to the next step
        float n0 = 0.f, n1 = 0.f, dummy;
        far1(ctr, la, nxt.p[1][1], n0, n1, dummy);
        const float ax = cst.k3 * (a0 + a1);
        float v;
        if (MODE == 0)
            v = fmaf(cst.omega * (bv - ax), __frcp_rn(cst.k0 * (sb + sa)), xc);
        else
            v = bv - ax;
        if (dxy || (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2])) v = 0.f;
        if (MODE == 1 && norm) nmax = (v != v || nmax != nmax) ? __int_as_float(0x7fc00000)
                                                              : fmaxf(nmax, fabsf(v) * (float)node_inv_volume(g, i, j, k));
        if (axy || (g.per[2] && (k <= 1 || k == g.n[2] - 1)))
            store_node(out, g, i, j, k, v);
        else
            *op = v;
        op += sz;
        bp += sz;
        carry = n0 + n1;
        sb = sa;
    };
    int k = kbeg;
    for (; k + 1 < kend; k += 2) {
        step(WB, WA, LA, LB, k);
        step(WA, WB, LB, LA, k + 1);
    }
    if (k < kend) step(WB, WA, LA, LB, k);
    if (MODE == 1 && norm) {
        const double m = block_max((double)nmax);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(norm, m);
    }
}

template <int MODE>
int launch_zmarch(const NodalGeom& g, const float* s, const float* x, const float* b, float* out, float omega,
                  unsigned long long* norm, cudaStream_t st)
{
    static int resident = 0;
    if (!resident) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_zmarch32<MODE>, ZX * ZY, 0) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + ZX - 1) / ZX, ty = (g.nu[1] + ZY - 1) / ZY;
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    const Consts c{(float)g.K[0], (float)g.K[3], omega};
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    k_zmarch32<MODE><<<grid, dim3(ZX, ZY), 0, st>>>(g, s, x, b, out, c, kchunk, norm);
    return GBP_OK;
}

// ----------------------------------------------------------------------------------------------
// Packed-pair z-march: a thread owns two x-adjacent nodes and does all stencil arithmetic in packed
// FP32x2 (one fma.rn.f32x2 per coupling for both nodes), halving the FP32 instruction count that
// bounds the scalar variants. The windows of plane k+2 and cell layer k+1 are loaded one step ahead
// (three-way register rotation, loop unrolled by three) so their latency overlaps the arithmetic.
constexpr int PX = 32, PY = 8;  // threads; a CTA covers 64 x 8 nodes

struct PWin {
    float2 c[3];     // rows j-1..j+1: (x[i0], x[i0+1])
    float l[3], r[3];  // x[i0-1], x[i0+2]
};
struct PLay {
    float2 c[2];  // rows j-1, j: (s[i0], s[i0+1])
    float l[2];   // s[i0-1]
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 lft(const PWin& w, int r) { return f2(w.l[r], w.c[r].x); }   // node i-1
__device__ __forceinline__ float2 rgt(const PWin& w, int r) { return f2(w.c[r].y, w.r[r]); }   // node i+1
__device__ __forceinline__ float2 slo(const PLay& L, int r) { return f2(L.l[r], L.c[r].x); }  // cell i-1
__device__ __forceinline__ float2 shi(const PLay& L, int r) { return L.c[r]; }                // cell i

// couplings of the centre pair to the far plane through layer L (edge pairs + corners), packed;
// returns the layer's sigma sum for each node
__device__ __forceinline__ float2 pfar(const PWin& far, const PLay& L, float2 xc, float2& a0, float2& a1)
{
    const float2 s00 = slo(L, 0), s01 = shi(L, 0), s10 = slo(L, 1), s11 = shi(L, 1);
    const float2 ax0 = __fadd2_rn(s00, s10), ax1 = __fadd2_rn(s01, s11);
    const float2 ay0 = __fadd2_rn(s00, s01), ay1 = __fadd2_rn(s10, s11);
    const float2 nxc = f2(-xc.x, -xc.y);
    a0 = __ffma2_rn(ax0, __fadd2_rn(lft(far, 1), nxc), a0);
    a1 = __ffma2_rn(ax1, __fadd2_rn(rgt(far, 1), nxc), a1);
    a0 = __ffma2_rn(ay0, __fadd2_rn(far.c[0], nxc), a0);
    a1 = __ffma2_rn(ay1, __fadd2_rn(far.c[2], nxc), a1);
    a0 = __ffma2_rn(s00, __fadd2_rn(lft(far, 0), nxc), a0);
    a1 = __ffma2_rn(s01, __fadd2_rn(rgt(far, 0), nxc), a1);
    a0 = __ffma2_rn(s10, __fadd2_rn(lft(far, 2), nxc), a0);
    a1 = __ffma2_rn(s11, __fadd2_rn(rgt(far, 2), nxc), a1);
    return __fadd2_rn(ax0, ax1);
}

template <int MODE>
__global__ void __launch_bounds__(PX* PY) k_zpair32(NodalGeom g, const float* __restrict__ sg, const float* __restrict__ xin,
                                                    const float* __restrict__ bin, float* __restrict__ out, Consts cst,
                                                    int kchunk, unsigned long long* norm)
{
    const int i0 = 2 * (blockIdx.x * PX + threadIdx.x), j = blockIdx.y * PY + threadIdx.y;
    const int kbeg = blockIdx.z * kchunk;
    const bool act = i0 < g.nu[0] && j < g.nu[1];
    const bool actB = i0 + 1 < g.nu[0];
    const int kend = act ? min(kbeg + kchunk, g.nu[2]) : kbeg;
    const long long sy = g.sy, sz = g.sz;
    const bool dA = (g.dlo[0] && i0 == 0) || (g.dhi[0] && i0 == g.n[0]) || (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]);
    const bool dB = !actB || (g.dlo[0] && i0 + 1 == 0) || (g.dhi[0] && i0 + 1 == g.n[0]) || (g.dlo[1] && j == 0) ||
                    (g.dhi[1] && j == g.n[1]);
    const bool axy = (g.per[0] && (i0 <= 1 || i0 + 1 >= g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1));
    const long long c0 = pidx(sy, sz, i0, j, 0);  // node (i0, j, 0); even i0: 8-byte aligned pair
    const float* xw = xin + c0 - sy;              // node (i0, j-1, 0)
    const float* sw = sg + c0 - sy;               // cell (i0, j-1, 0)
    auto load_win = [&](int q, PWin& w) {
        const float* p = xw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float* rp = p + r * sy;
            w.c[r] = __ldg(reinterpret_cast<const float2*>(rp));
            w.l[r] = __ldg(rp - 1);
            w.r[r] = __ldg(rp + 2);
        }
    };
    auto load_lay = [&](int q, PLay& l) {
        const float* p = sw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const float* rp = p + r * sy;
            l.c[r] = __ldg(reinterpret_cast<const float2*>(rp));
            l.l[r] = __ldg(rp - 1);
        }
    };

    PWin W0, W1, W2;
    PLay L0, L1, L2;
    float2 carry = f2(0.f, 0.f), sb = f2(0.f, 0.f);
    float nmax = 0.f;
    float* op = out + c0 + (long long)kbeg * sz;
    const float* bp = bin + c0 + (long long)kbeg * sz;
    if (kend > kbeg) {
        load_win(kbeg - 1, W2);  // plane kbeg-1 (temporarily in W2)
        load_win(kbeg, W0);
        load_lay(kbeg - 1, L2);
        float2 a0 = f2(0.f, 0.f), a1 = f2(0.f, 0.f);
        sb = pfar(W2, L2, W0.c[1], a0, a1);
        carry = __fadd2_rn(a0, a1);
        load_lay(kbeg - 1, L0);
        load_win(kbeg + 1, W1);  // planes beyond the chunk are in the padded box (<= n+1)
        load_lay(kbeg, L1);
    }
    const float2 k3 = f2(cst.k3, cst.k3), k0 = f2(cst.k0, cst.k0), om = f2(cst.omega, cst.omega);

    // ctr = plane k, nxt = plane k+1 (both loaded), pre <- plane k+2; lb = layer k-1, la = layer k, lp <- layer k+1
    auto step = [&](PWin& ctr, PWin& nxt, PWin& pre, PLay& lb, PLay& la, PLay& lp, int k) {
        if (k + 1 < kend) {
            load_win(k + 2, pre);
            load_lay(k + 1, lp);
        }
        const float2 bv = __ldg(reinterpret_cast<const float2*>(bp));
        const float2 xc = ctr.c[1];
        const float2 nxc = f2(-xc.x, -xc.y);
        float2 a0 = carry, a1 = f2(0.f, 0.f);
        // in-plane face diagonals: sigma below + above
        a0 = __ffma2_rn(__fadd2_rn(slo(lb, 0), slo(la, 0)), __fadd2_rn(lft(ctr, 0), nxc), a0);
        a1 = __ffma2_rn(__fadd2_rn(shi(lb, 0), shi(la, 0)), __fadd2_rn(rgt(ctr, 0), nxc), a1);
        a0 = __ffma2_rn(__fadd2_rn(slo(lb, 1), slo(la, 1)), __fadd2_rn(lft(ctr, 2), nxc), a0);
        a1 = __ffma2_rn(__fadd2_rn(shi(lb, 1), shi(la, 1)), __fadd2_rn(rgt(ctr, 2), nxc), a1);
        const float2 sa = pfar(nxt, la, xc, a0, a1);
        // coupling of node k+1 to this plane through layer k, carried to the next step
        float2 n0 = f2(0.f, 0.f), n1 = f2(0.f, 0.f);
        (void)pfar(ctr, la, nxt.c[1], n0, n1);
        const float2 ax = __fmul2_rn(k3, __fadd2_rn(a0, a1));
        const float2 rr = __fadd2_rn(bv, f2(-ax.x, -ax.y));
        float2 v;
        if (MODE == 0) {
            const float2 dg = __fmul2_rn(k0, __fadd2_rn(sb, sa));
            v = __ffma2_rn(__fmul2_rn(om, rr), f2(__frcp_rn(dg.x), __frcp_rn(dg.y)), xc);
        } else {
            v = rr;
        }
        const bool dk = (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]);
        if (dk || dA) v.x = 0.f;
        if (dk || dB) v.y = 0.f;
        if (MODE == 1 && norm) {
            const float m = fmaxf(fabsf(v.x) * (float)node_inv_volume(g, i0, j, k),
                                  actB ? fabsf(v.y) * (float)node_inv_volume(g, i0 + 1, j, k) : 0.f);
            nmax = (v.x != v.x || v.y != v.y || nmax != nmax) ? __int_as_float(0x7fc00000) : fmaxf(nmax, m);
        }
        if (axy || (g.per[2] && (k <= 1 || k == g.n[2] - 1)) || !actB) {
            store_node(out, g, i0, j, k, v.x);
            if (actB) store_node(out, g, i0 + 1, j, k, v.y);
        } else {
            *reinterpret_cast<float2*>(op) = v;
        }
        op += sz;
        bp += sz;
        carry = __fadd2_rn(n0, n1);
        sb = sa;
    };
    int k = kbeg;
    for (; k + 2 < kend; k += 3) {
        step(W0, W1, W2, L0, L1, L2, k);
        step(W1, W2, W0, L1, L2, L0, k + 1);
        step(W2, W0, W1, L2, L0, L1, k + 2);
    }
    if (k < kend) step(W0, W1, W2, L0, L1, L2, k);
    if (k + 1 < kend) step(W1, W2, W0, L1, L2, L0, k + 1);
    if (MODE == 1 && norm) {
        const double m = block_max((double)nmax);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(norm, m);
    }
}

template <int MODE>
int launch_zpair(const NodalGeom& g, const float* s, const float* x, const float* b, float* out, float omega,
                 unsigned long long* norm, cudaStream_t st)
{
    static int resident = 0;
    if (!resident) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_zpair32<MODE>, PX * PY, 0) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + 2 * PX - 1) / (2 * PX), ty = (g.nu[1] + PY - 1) / PY;
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    const Consts c{(float)g.K[0], (float)g.K[3], omega};
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    k_zpair32<MODE><<<grid, dim3(PX, PY), 0, st>>>(g, s, x, b, out, c, kchunk, norm);
    return GBP_OK;
}

// ----------------------------------------------------------------------------------------------
// Register-blocked z-march: a thread owns an x-pair of nodes in RY consecutive rows (2 x RY nodes),
// packed FP32x2 arithmetic, windows of RY+2 rows and cell layers of RY+1 rows shared by the RY node
// rows, so loads and loop overhead are amortised over 2*RY nodes and the RY independent rows give
// the scheduler parallel FMA chains. Two planes in registers, the far-plane coupling carried.
constexpr int QX = 32, QY = 4;  // threads per CTA: 32 x-pairs (64 nodes) x QY row blocks

template <int RY>
struct BWin {
    float2 c[RY + 2];
    float l[RY + 2], r[RY + 2];
};
template <int RY>
struct BLay {
    float2 c[RY + 1];
    float l[RY + 1];
};

template <int RY>
__device__ __forceinline__ float2 blft(const BWin<RY>& w, int r) { return f2(w.l[r], w.c[r].x); }
template <int RY>
__device__ __forceinline__ float2 brgt(const BWin<RY>& w, int r) { return f2(w.c[r].y, w.r[r]); }
template <int RY>
__device__ __forceinline__ float2 bslo(const BLay<RY>& L, int r) { return f2(L.l[r], L.c[r].x); }

// couplings of node row q of the centre pair to the far plane through layer L, packed
template <int RY>
__device__ __forceinline__ float2 bfar(const BWin<RY>& far, const BLay<RY>& L, int q, float2 xc, float2& a0, float2& a1)
{
    const float2 s00 = bslo(L, q), s01 = L.c[q], s10 = bslo(L, q + 1), s11 = L.c[q + 1];
    const float2 ax0 = __fadd2_rn(s00, s10), ax1 = __fadd2_rn(s01, s11);
    const float2 ay0 = __fadd2_rn(s00, s01), ay1 = __fadd2_rn(s10, s11);
    const float2 nxc = f2(-xc.x, -xc.y);
    a0 = __ffma2_rn(ax0, __fadd2_rn(blft(far, q + 1), nxc), a0);
    a1 = __ffma2_rn(ax1, __fadd2_rn(brgt(far, q + 1), nxc), a1);
    a0 = __ffma2_rn(ay0, __fadd2_rn(far.c[q], nxc), a0);
    a1 = __ffma2_rn(ay1, __fadd2_rn(far.c[q + 2], nxc), a1);
    a0 = __ffma2_rn(s00, __fadd2_rn(blft(far, q), nxc), a0);
    a1 = __ffma2_rn(s01, __fadd2_rn(brgt(far, q), nxc), a1);
    a0 = __ffma2_rn(s10, __fadd2_rn(blft(far, q + 2), nxc), a0);
    a1 = __ffma2_rn(s11, __fadd2_rn(brgt(far, q + 2), nxc), a1);
    return __fadd2_rn(ax0, ax1);
}

template <int MODE, int RY>
__global__ void __launch_bounds__(QX* QY) k_zblock32(NodalGeom g, const float* __restrict__ sg, const float* __restrict__ xin,
                                                     const float* __restrict__ bin, float* __restrict__ out, Consts cst,
                                                     int kchunk, unsigned long long* norm)
{
    const int i0 = 2 * (blockIdx.x * QX + threadIdx.x);
    const int j0 = (blockIdx.y * QY + threadIdx.y) * RY;
    const int kbeg = blockIdx.z * kchunk;
    const bool act = i0 < g.nu[0] && j0 < g.nu[1];
    const bool actB = i0 + 1 < g.nu[0];
    const int kend = act ? min(kbeg + kchunk, g.nu[2]) : kbeg;
    const long long sy = g.sy, sz = g.sz;
    const bool dxA = (g.dlo[0] && i0 == 0) || (g.dhi[0] && i0 == g.n[0]);
    const bool dxB = !actB || (g.dlo[0] && i0 + 1 == 0) || (g.dhi[0] && i0 + 1 == g.n[0]);
    const bool ax_ = g.per[0] && (i0 <= 1 || i0 + 1 >= g.n[0] - 1);
    const long long c0 = pidx(sy, sz, i0, j0, 0);
    const float* xw = xin + c0 - sy;  // node (i0, j0-1, 0)
    const float* sw = sg + c0 - sy;   // cell (i0, j0-1, 0)
    auto load_win = [&](int q, BWin<RY>& w) {
        const float* p = xw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < RY + 2; ++r) {
            const float* rp = p + r * sy;
            w.c[r] = __ldg(reinterpret_cast<const float2*>(rp));
            w.l[r] = __ldg(rp - 1);
            w.r[r] = __ldg(rp + 2);
        }
    };
    auto load_lay = [&](int q, BLay<RY>& l) {
        const float* p = sw + (long long)q * sz;
#pragma unroll
        for (int r = 0; r < RY + 1; ++r) {
            const float* rp = p + r * sy;
            l.c[r] = __ldg(reinterpret_cast<const float2*>(rp));
            l.l[r] = __ldg(rp - 1);
        }
    };
    BWin<RY> WA, WB;
    BLay<RY> LA, LB;
    float2 carry[RY], sb[RY];
#pragma unroll
    for (int q = 0; q < RY; ++q) carry[q] = sb[q] = f2(0.f, 0.f);
    float nmax = 0.f;
    if (kend > kbeg) {
        load_win(kbeg - 1, WA);
        load_win(kbeg, WB);
        load_lay(kbeg - 1, LA);
#pragma unroll
        for (int q = 0; q < RY; ++q) {
            float2 a0 = f2(0.f, 0.f), a1 = f2(0.f, 0.f);
            sb[q] = bfar(WA, LA, q, WB.c[q + 1], a0, a1);
            carry[q] = __fadd2_rn(a0, a1);
        }
    }
    const float2 k3 = f2(cst.k3, cst.k3), k0 = f2(cst.k0, cst.k0), om = f2(cst.omega, cst.omega);
    float* op = out + c0 + (long long)kbeg * sz;
    const float* bp = bin + c0 + (long long)kbeg * sz;

    auto step = [&](BWin<RY>& ctr, BWin<RY>& nxt, BLay<RY>& lb, BLay<RY>& la, int k) {
        load_win(k + 1, nxt);
        load_lay(k, la);
        const bool dk = (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]);
        const bool ak = g.per[2] && (k <= 1 || k == g.n[2] - 1);
#pragma unroll
        for (int q = 0; q < RY; ++q) {
            const int j = j0 + q;
            const float2 bv = __ldg(reinterpret_cast<const float2*>(bp + q * sy));
            const float2 xc = ctr.c[q + 1];
            const float2 nxc = f2(-xc.x, -xc.y);
            float2 a0 = carry[q], a1 = f2(0.f, 0.f);
            a0 = __ffma2_rn(__fadd2_rn(bslo(lb, q), bslo(la, q)), __fadd2_rn(blft(ctr, q), nxc), a0);
            a1 = __ffma2_rn(__fadd2_rn(lb.c[q], la.c[q]), __fadd2_rn(brgt(ctr, q), nxc), a1);
            a0 = __ffma2_rn(__fadd2_rn(bslo(lb, q + 1), bslo(la, q + 1)), __fadd2_rn(blft(ctr, q + 2), nxc), a0);
            a1 = __ffma2_rn(__fadd2_rn(lb.c[q + 1], la.c[q + 1]), __fadd2_rn(brgt(ctr, q + 2), nxc), a1);
            const float2 sa = bfar(nxt, la, q, xc, a0, a1);
            float2 n0 = f2(0.f, 0.f), n1 = f2(0.f, 0.f);
            (void)bfar(ctr, la, q, nxt.c[q + 1], n0, n1);
            const float2 ax = __fmul2_rn(k3, __fadd2_rn(a0, a1));
            const float2 rr = __fadd2_rn(bv, f2(-ax.x, -ax.y));
            float2 v;
            if (MODE == 0) {
                const float2 dg = __fmul2_rn(k0, __fadd2_rn(sb[q], sa));
                v = __ffma2_rn(__fmul2_rn(om, rr), f2(__frcp_rn(dg.x), __frcp_rn(dg.y)), xc);
            } else {
                v = rr;
            }
            carry[q] = __fadd2_rn(n0, n1);
            sb[q] = sa;
            if (j < g.nu[1]) {
                const bool dy = (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]);
                if (dk || dy || dxA) v.x = 0.f;
                if (dk || dy || dxB) v.y = 0.f;
                if (MODE == 1 && norm) {
                    const float m = fmaxf(fabsf(v.x) * (float)node_inv_volume(g, i0, j, k),
                                          actB ? fabsf(v.y) * (float)node_inv_volume(g, i0 + 1, j, k) : 0.f);
                    nmax = (v.x != v.x || v.y != v.y || nmax != nmax) ? __int_as_float(0x7fc00000) : fmaxf(nmax, m);
                }
                const bool ay = g.per[1] && (j <= 1 || j == g.n[1] - 1);
                if (ak || ay || ax_ || !actB) {
                    store_node(out, g, i0, j, k, v.x);
                    if (actB) store_node(out, g, i0 + 1, j, k, v.y);
                } else {
                    *reinterpret_cast<float2*>(op + q * sy) = v;
                }
            }
        }
        op += sz;
        bp += sz;
    };
    int k = kbeg;
    for (; k + 1 < kend; k += 2) {
        step(WB, WA, LA, LB, k);
        step(WA, WB, LB, LA, k + 1);
    }
    if (k < kend) step(WB, WA, LA, LB, k);
    if (MODE == 1 && norm) {
        const double m = block_max((double)nmax);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(norm, m);
    }
}

template <int MODE, int RY>
int launch_zblock(const NodalGeom& g, const float* s, const float* x, const float* b, float* out, float omega,
                  unsigned long long* norm, cudaStream_t st)
{
    static int resident = 0;
    if (!resident) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_zblock32<MODE, RY>, QX * QY, 0) != cudaSuccess ||
            resident < 1)
            resident = 1;
    }
    const int tx = (g.nu[0] + 2 * QX - 1) / (2 * QX), ty = (g.nu[1] + QY * RY - 1) / (QY * RY);
    const int nz = sweep_z_chunks(g, tx * ty, resident);
    const int kchunk = (g.nu[2] + nz - 1) / nz;
    const Consts c{(float)g.K[0], (float)g.K[3], omega};
    dim3 grid(tx, ty, (g.nu[2] + kchunk - 1) / kchunk);
    k_zblock32<MODE, RY><<<grid, dim3(QX, QY), 0, st>>>(g, s, x, b, out, c, kchunk, norm);
    return GBP_OK;
}

int sweep_variant()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("GBP_SWEEP32");
        // 5: k_sweep32t (default), 6: k_sweep32p (packed FP32x2), 3: register-blocked 2x4,
        // 4: register-blocked 2x2, 2: packed pair, 0: scalar z-march, 1: TMA producer/consumer
        v = 5;
        if (e) {
            if (e[0] == 'q') v = 6;  // k_sweep32p, packed FP32x2 (measured 7 % slower)
            else if (e[0] == 'b') v = 3;
            else if (e[0] == 't') v = 1;
            else if (e[0] == 's') v = 0;
            else if (e[0] == 'p') v = 2;
            else if (e[0] == '2') v = 4;
        }
    }
    return v;
}

}  // namespace

int sweep32_run(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st)
{
    if (sweep_variant() >= 5) return sweep32_tma1_run(g, mode, s, x, b, out, omega, err, norm, st, sweep_variant() == 6);
    if (sweep_variant() == 3)
        return mode == 0 ? launch_zblock<0, 4>(g, s, x, b, out, omega, norm, st)
                         : launch_zblock<1, 4>(g, s, x, b, out, omega, norm, st);
    if (sweep_variant() == 4)
        return mode == 0 ? launch_zblock<0, 2>(g, s, x, b, out, omega, norm, st)
                         : launch_zblock<1, 2>(g, s, x, b, out, omega, norm, st);
    if (sweep_variant() == 2)
        return mode == 0 ? launch_zpair<0>(g, s, x, b, out, omega, norm, st)
                         : launch_zpair<1>(g, s, x, b, out, omega, norm, st);
    if (sweep_variant() == 0)
        return mode == 0 ? launch_zmarch<0>(g, s, x, b, out, omega, norm, st)
                         : launch_zmarch<1>(g, s, x, b, out, omega, norm, st);
    CUtensorMap mx, ms, mb;
    int rc = make_tensor_map(x, 4, g.sy, g.sz, g.count, BXX, TY + 2, &mx);
    if (!rc) rc = make_tensor_map(s, 4, g.sy, g.sz, g.count, BXS, TY + 1, &ms);
    if (!rc) rc = make_tensor_map(b, 4, g.sy, g.sz, g.count, BXB, TY, &mb);
    if (rc) return rc;
    return mode == 0 ? launch<0>(mx, ms, mb, g, out, omega, err, norm, st)
                     : launch<1>(mx, ms, mb, g, out, omega, err, norm, st);
}

}  // namespace gbp
