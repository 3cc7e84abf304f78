// FP32 level sweeps of the isotropic nodal operator for the inner V-cycles, with the grid transfers
// fused in: Jacobi sweep, residual, residual + full-weighting restriction (the coarse right-hand side
// is written directly; the fine residual never reaches memory), and prolongation + Jacobi sweep (the
// coarse correction is interpolated into the staged tile; the corrected fine values never reach
// memory). These are the smoother / residual / transfer work of MLMG's V-cycle on MLNodeLaplacian
// (the solve behind incflo::ApplyNodalProjection, src/projection/incflo_apply_nodal_projection.cpp:215).
//
// Tiling. A CTA owns whole x rows (the full padded row, node i at position i + 4) of TY node rows and
// marches up a chunk of z planes; each thread owns 4 consecutive nodes of RPT rows (2: the loads of
// the x window and the sigma pair sums are shared by 8 nodes, and the per-step overhead by twice as
// many nodes). Per z step one
// elected thread loads by TMA the next x plane with one halo row on each side, the sigma cell layer
// below it and a b plane into a 3-slot ring of mbarrier-tracked stages. The tensor maps are 4-D
// ({bw, nbx, rows, planes} with bw * nbx = the padded row length) so that one box holds whole rows
// although a box dimension is limited to 256 elements.
//
// Layer-wise accumulation. When plane P arrives, the cell layer between planes P-1 and P contributes
// to the nodes of plane P-1 (their upper half: they are then complete) and to the nodes of plane P
// (their lower half, carried in registers to the next step), so a thread keeps two x planes of 3 rows
// x 6 values in registers. Per node and layer the isotropic Q1 element gives
//   sum over the 4 cells (a, b) of sigma_ab [(x_inplane_diag - x_c) + (x_body_diag - x_c)]
//   + sum over x sides (sigma pair along y) (x_xz_diag - x_c) + sum over y sides (sigma pair along x) (x_yz_diag - x_c),
// differences to the centre (FP32 rounding scales with the local variation of x), times K3; the
// diagonal is K0 times the sum of the 8 cell sigmas. The in-plane and body-diagonal terms of the node
// below a layer (centre c_A) and of the node above it (centre c_B) share their cells and corner values:
//   G_B = G_A - 2 (c_B - c_A) sum_layer(sigma),
// so the second costs one FMA; both are sums of local differences, so the rounding stays local.
//
// Restriction (mode 2). The CTA computes the residual of node rows y0-1 .. y0+TY-1 (one row more than
// it owns: coarse row y0/2 needs fine rows y0-1 .. y0+1), stages each residual plane in shared memory,
// restricts it in x and y, and accumulates the z weights (1/2, 1, 1/2) in registers; a z chunk starts
// one plane early for the same reason. Coarse values are written once, by one thread: no atomics.
//
// Alias values. x and sigma arrays hold valid periodic aliases (every writer stores them); b arrays
// hold only the unique positions, so b is read at mapped coordinates. A plane or row index below -1
// does not exist in the padded layout and is mapped by periodicity.
//
// Failure: every mbarrier wait is bounded; a thread whose wait runs out sets the CTA's abort flag,
// which all threads read after the next block barrier (so they leave the loop together); the issuing
// thread then waits, again bounded, for the copies still in flight.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "gbp_internal.cuh"
#include "nodal_sweep.h"
#include "tma.cuh"

namespace gbp {

namespace {

// Launch shape. Pipeline stages (TMA prefetch distance = stages - 1) for the plain sweeps (modes 0, 1)
// and the transfer sweeps (modes 2, 3, which stage more per plane), the resident threads per SM the
// register budget is set for, the rows per CTA of 256-node rows and the node rows per thread.
#ifndef GBP_VS_STAGES_PLAIN
#define GBP_VS_STAGES_PLAIN 3
#endif
#ifndef GBP_VS_STAGES_XFER
#define GBP_VS_STAGES_XFER 3
#endif
#ifndef GBP_VS_THREADS_PER_SM
#define GBP_VS_THREADS_PER_SM 512  // resident threads per SM the kernels are compiled for (registers)
#endif
#ifndef GBP_VS_TY_256
#define GBP_VS_TY_256 8
#endif
#ifndef GBP_VS_TY_512
#define GBP_VS_TY_512 2
#endif
#ifndef GBP_VS_RPT
#define GBP_VS_RPT 2  // node rows per thread
#endif
constexpr int kMaxTX = 128;  // threads per row: 4 * 128 = 512 nodes per row at most
// CTA shapes: TY rows per CTA by the row width (TX threads of 4 nodes): 8 rows for rows of <= 128
// nodes (TX <= 32), GBP_VS_TY_256 for <= 256 (TX <= 64), GBP_VS_TY_512 for <= 512 (TX <= 128)
template <int MODE>
struct Stages {
    static constexpr int N = MODE <= 1 ? GBP_VS_STAGES_PLAIN : GBP_VS_STAGES_XFER;
};

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z,
                                            int w)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

struct VsArgs {
    NodalGeom g;    // this level
    NodalGeom gc;   // the coarse level (restriction / prolongation modes)
    float* out;     // fine output (modes 0, 1, 3) or coarse right-hand side (mode 2)
    float k0, k3, omega;
    int kchunk;     // node planes per CTA (even in mode 2)
    int rowlen;     // padded fine row length (floats)
    int crowlen;    // padded coarse row length (floats)
    int rstride;    // row stride of the per-CTA scratch rows (floats)
    unsigned* err;
};

template <int MODE, int TY, int RPT>
struct VsShape {
    // node rows computed: y0 .. y0+TY-1; mode 2 also the row below, y0-1 (the restriction of coarse row
    // y0/2 needs fine rows y0-1 .. y0+1), rounded up to whole threads
    static constexpr int TYR = ((MODE == 2 ? TY + 1 : TY) + RPT - 1) / RPT * RPT;
    static constexpr int TTR = TYR / RPT;  // thread rows
    static constexpr int XR = TYR + 2;     // x rows staged: first node row - 1 .. last + 1
    static constexpr int SR = TYR + 1;     // sigma cell rows: first node row - 1 .. last
    static constexpr int BR = TYR;         // b rows
    static constexpr int CR = TY / 2 + 3;  // coarse rows (mode 3)
    // scratch rows: mode 2 the residual rows of two planes (the restriction of a plane runs one step later)
    static constexpr int RR = MODE == 2 ? 2 * TYR : 0;
};

__host__ __device__ constexpr int al128(int b) { return (b + 127) / 128 * 128; }

// Stage layout (bytes). Every TMA destination starts on a 128-byte boundary: mode 2's one-row boxes
// (the row below the tile) get areas of their own (xa, sa, ba) in front of the main boxes.
struct StageLayout {
    int xa, xo, sa, so, ba, bo, co, co1, bytes;
    uint32_t tx;  // transaction bytes per stage
};

template <int MODE, int TY, int RPT>
__host__ __device__ inline StageLayout stage_layout(int rowlen, int crowlen)
{
    using S = VsShape<MODE, TY, RPT>;
    const int one = MODE == 2 ? al128(rowlen * 4) : 0;  // the one-row area
    const int sub = MODE == 2 ? 1 : 0;
    StageLayout L;
    L.xa = 0;
    L.xo = L.xa + one;
    L.sa = L.xo + al128((S::XR - sub) * rowlen * 4);
    L.so = L.sa + one;
    L.ba = L.so + al128((S::SR - sub) * rowlen * 4);
    L.bo = L.ba + one;
    L.co = L.bo + al128((S::BR - sub) * rowlen * 4);
    const int cp = MODE == 3 ? al128(S::CR * crowlen * 4) : 0;  // one coarse plane
    L.co1 = L.co + cp;
    L.bytes = L.co1 + cp;
    L.tx = (uint32_t)((S::XR + S::SR + S::BR) * rowlen * 4 + (MODE == 3 ? 2 * S::CR * crowlen * 4 : 0));
    return L;
}

template <int MODE, int TY, int RPT>
inline int smem_bytes(int rowlen, int crowlen, int rstride)
{
    return Stages<MODE>::N * stage_layout<MODE, TY, RPT>(rowlen, crowlen).bytes +
           VsShape<MODE, TY, RPT>::RR * rstride * 4;
}

// positions below -1 do not exist in the padded layout; periodic ones map to their alias
__device__ __forceinline__ int wrapz(const NodalGeom& g, int p) { return (p < -1 && g.per[2]) ? p + g.n[2] : p; }

// Store the 4 node values of a thread row with the periodic aliases of x (node 0 -> n, 1 -> n+1,
// n-1 -> -1), y and z. Away from the periodic seams (all but a few rows and planes): one vector store.
__device__ __forceinline__ void store4(float* out, const NodalGeom& g, int i0, int j, int k, const float (&v)[4],
                                       int nact)
{
    const bool ax = g.per[0] && (i0 == 0 || i0 + 3 == g.n[0] - 1);
    const bool ay = g.per[1] && (j <= 1 || j == g.n[1] - 1);
    const bool az = g.per[2] && (k <= 1 || k == g.n[2] - 1);
    if (!(ax || ay || az) && nact == 4) {
        *reinterpret_cast<float4*>(out + pidx(g.sy, g.sz, i0, j, k)) = make_float4(v[0], v[1], v[2], v[3]);
        return;
    }
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
        const int kk = node_alias_cand(k, g.n[2], g.per[2], c);
        if (kk == kNoAlias) continue;
#pragma unroll 1
        for (int b = 0; b < 4; ++b) {
            const int jj = node_alias_cand(j, g.n[1], g.per[1], b);
            if (jj == kNoAlias) continue;
            float* row = out + pidx(g.sy, g.sz, 0, jj, kk);
            if (nact == 4) {
                *reinterpret_cast<float4*>(row + i0) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
                for (int q = 0; q < nact; ++q) row[i0 + q] = v[q];
            }
            if (g.per[0]) {
                if (i0 == 0) {
                    row[g.n[0]] = v[0];
                    row[g.n[0] + 1] = v[1];
                }
                if (i0 + 3 == g.n[0] - 1) row[-1] = v[3];
            }
        }
    }
}

// Approximate reciprocal (one MUFU operation): the Jacobi smoother only scales its update by it.
__device__ __forceinline__ float rcp_approx(float d)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    return r;
}

// MODE 0: Jacobi  out = x + omega (b - A x) / diag(A)
// MODE 1: residual out = b - A x
// MODE 2: residual + restriction: out (the coarse b) = full weighting of b - A x
// MODE 3: prolongation + Jacobi: x' = x + P e (e = the coarse correction), out = x' + omega (b - A x') / diag
template <int MODE, int TY, int TXM, int RPT>
__global__ void __launch_bounds__(TXM * VsShape<MODE, TY, RPT>::TTR,
                                  GBP_VS_THREADS_PER_SM / (TXM * VsShape<MODE, TY, RPT>::TTR) > 0
                                      ? GBP_VS_THREADS_PER_SM / (TXM * VsShape<MODE, TY, RPT>::TTR)
                                      : 1)
    k_vsweep32(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap ms,
               const __grid_constant__ CUtensorMap mb, const __grid_constant__ CUtensorMap mc,
               const __grid_constant__ CUtensorMap mx1, const __grid_constant__ CUtensorMap ms1,
               const __grid_constant__ CUtensorMap mb1, VsArgs a)
{
    using Sh = VsShape<MODE, TY, RPT>;
    constexpr int kNS = Stages<MODE>::N;
    constexpr int W = RPT + 2;  // x window rows of a thread
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar[kNS];
    __shared__ int abort_flag;
    const NodalGeom& g = a.g;
    const StageLayout L = stage_layout<MODE, TY, RPT>(a.rowlen, a.crowlen);
    float* R = reinterpret_cast<float*>(smem + kNS * L.bytes);  // mode 2: residual rows of two planes

    const int t = threadIdx.x, jr = threadIdx.y;
    const int TX = blockDim.x;
    const int nthr = TX * Sh::TTR;
    const int tid = t + TX * jr;
    const int i0 = 4 * t;
    const int y0 = blockIdx.y * TY;
    const int kbeg = blockIdx.z * a.kchunk;
    const int kend = min(kbeg + a.kchunk, g.nu[2]);
    const int kfirst = MODE == 2 ? kbeg - 1 : kbeg;  // first node plane computed
    const int nsteps = kend - kfirst + 2;
    const int ybase = MODE == 2 ? y0 - 1 : y0;       // first node row computed
    const int srow0 = RPT * jr;                      // staged row of the thread's first window row
    const int j0 = ybase + srow0;                    // the thread's first node row
    // nodes of this thread that exist (mode 2: row -1 is the periodic alias of n-1, or zero)
    const int nact = max(0, min(4, g.nu[0] - i0));
    unsigned dmask = 0;  // bit r*4+q: node (q, row r) is Dirichlet or does not exist: its value is 0
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + q, j = j0 + r;
            if ((g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]) ||
                q >= nact || j >= g.nu[1])
                dmask |= 1u << (r * 4 + q);
        }
    // mode 2: the coarse row this thread reduces, from the residual rows 2 jr .. 2 jr + 2 (fine rows
    // 2 cJ - 1 .. 2 cJ + 1)
    const int cJ = (MODE == 2 && jr < TY / 2) ? y0 / 2 + jr : -1;

    uint32_t issued = 0;
    auto issue = [&](int s) {
        unsigned char* base = smem + (s % kNS) * L.bytes;
        uint64_t* br = &bar[s % kNS];
        const int P = kfirst - 1 + s;  // x plane of this step
        mbar_arrive_expect_tx(br, L.tx);
        int pb = P - 1;  // b plane P-1, unique position
        if (g.per[2] && pb < 0) pb += g.n[2];
        const int zx = wrapz(g, P) + 1, zs = wrapz(g, P - 1) + 1;  // padded plane indices
        if (MODE == 2) {
            // the row below the tile by one-row boxes: x / sigma row y0-2 and b row y0-1 (row -2 does not
            // exist in the padded layout, and b holds no aliases: both map to their periodic image)
            int yx = y0 - 2, yb = y0 - 1;
            if (g.per[1] && yx < -1) yx += g.n[1];
            if (g.per[1] && yb < 0) yb += g.n[1];
            tma_load_4d(base + L.xa, &mx1, br, 0, 0, yx + 1, zx);
            tma_load_4d(base + L.xo, &mx, br, 0, 0, y0, zx);
            tma_load_4d(base + L.sa, &ms1, br, 0, 0, yx + 1, zs);
            tma_load_4d(base + L.so, &ms, br, 0, 0, y0, zs);
            tma_load_4d(base + L.ba, &mb1, br, 0, 0, yb + 1, pb + 1);
            tma_load_4d(base + L.bo, &mb, br, 0, 0, y0 + 1, pb + 1);
        } else {
            tma_load_4d(base + L.xo, &mx, br, 0, 0, y0, zx);  // x rows y0-1 .. (padded row y0)
            tma_load_4d(base + L.so, &ms, br, 0, 0, y0, zs);  // sigma cell rows y0-1 ..
            tma_load_4d(base + L.bo, &mb, br, 0, 0, y0 + 1, pb + 1);
        }
        if (MODE == 3) {
            const int K0 = P >> 1;         // coarse planes K0, K0 + 1
            const int J0 = (y0 - 1) >> 1;  // first coarse row
            tma_load_4d(base + L.co, &mc, br, 0, 0, J0 + 1, K0 + 1);
            tma_load_4d(base + L.co1, &mc, br, 0, 0, J0 + 1, K0 + 2);
        }
        ++issued;
    };

    if (tid == 0) {
        for (int q = 0; q < kNS; ++q) mbar_init(&bar[q], 1);
        mbar_fence_init();
        abort_flag = 0;
    }
    if (MODE == 2)
        for (int e = tid; e < Sh::RR * a.rstride; e += nthr) R[e] = 0.f;  // tail columns stay zero
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < kNS - 1 && s < nsteps; ++s) issue(s);

    float acc[RPT][4], ss[RPT][4];
    float carry0 = 0.f, carry1 = 0.f;  // mode 2: coarse nodes 2t, 2t+1 of coarse row cJ
#pragma unroll
    for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[r][q] = ss[r][q] = 0.f;

    // Mode 2: restrict residual plane k (staged in scratch buffer rb): x and y full weighting of the
    // thread's coarse row, z weights carried in registers; a coarse plane is stored once complete.
    auto restrict_plane = [&](int k, int rb) {
        if (MODE != 2 || cJ < 0) return;
        // coarse (2t, cJ), (2t+1, cJ): fine x 4t-1 .. 4t+3 of scratch rows 2 jr .. 2 jr + 2
        float c2[2] = {0.f, 0.f};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const float* rr = R + (rb * Sh::TYR + 2 * jr + r) * a.rstride + 3 + i0;
            const float w = r == 1 ? 1.f : 0.5f;
            const float x0 = rr[0], x1 = rr[1], x2 = rr[2], x3 = rr[3], x4 = rr[4];
            c2[0] = fmaf(w, fmaf(0.5f, x0 + x2, x1), c2[0]);
            c2[1] = fmaf(w, fmaf(0.5f, x2 + x4, x3), c2[1]);
        }
        int Kst = -1;
        float o0 = 0.f, o1 = 0.f;
        if (k & 1) {
            // an odd plane completes coarse plane (k-1)/2, unless it is the chunk's extra plane
            if (k > kfirst) {
                Kst = (k - 1) >> 1;
                o0 = carry0 + 0.5f * c2[0];
                o1 = carry1 + 0.5f * c2[1];
            }
            carry0 = 0.5f * c2[0];
            carry1 = 0.5f * c2[1];
        } else {
            carry0 += c2[0];
            carry1 += c2[1];
            if (!g.per[2] && k == g.nu[2] - 1) {  // the last plane of a non-periodic direction
                Kst = k >> 1;
                o0 = carry0;
                o1 = carry1;
            }
        }
        if (Kst >= 0 && cJ < a.gc.nu[1] && Kst < a.gc.nu[2]) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int I = 2 * t + h;
                if (I < a.gc.nu[0])
                    a.out[pidx(a.gc.sy, a.gc.sz, I, cJ, Kst)] =
                        node_is_dirichlet(a.gc, I, cJ, Kst) ? 0.f : (h ? o1 : o0);
            }
        }
    };

    // consumer position in the ring: the stage of step s and its mbarrier phase parity
    int cslot = 0;
    uint32_t cphase = 0;
    // One z step: Bn receives plane P (prolongated in mode 3); Ao holds plane P-1.
    // overset mask words of the thread's rows, loaded one plane ahead (a global load on the critical path of
    // every plane would stall the z march)
    unsigned mw[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) mw[r] = 0xffffffffu;
    auto step = [&](int s, const float (&Ao)[W][6], float (&Bn)[W][6]) {
        const unsigned char* base = smem + cslot * L.bytes;
        if (!mbar_wait_bounded(&bar[cslot], cphase, a.err)) abort_flag = 1;
        if (++cslot == kNS) {
            cslot = 0;
            cphase ^= 1u;
        }
        const int P = kfirst - 1 + s;
        // the residual plane staged at the previous step (its rows are complete: a barrier lies between)
        if (MODE == 2 && s >= 3) restrict_plane(P - 2, (s - 1) & 1);
        // staged row r of an array: mode 2 keeps row 0 (the row below the tile) in its own area
        auto srow = [&](int area, int main, int r) -> const float* {
            if (MODE == 2)
                return r == 0 ? reinterpret_cast<const float*>(base + area)
                              : reinterpret_cast<const float*>(base + main) + (r - 1) * a.rowlen;
            return reinterpret_cast<const float*>(base + main) + r * a.rowlen;
        };
        // plane P, window rows j0-1 .. j0+RPT (staged rows srow0 ..), nodes i0-1 .. i0+4
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const float* row = srow(L.xa, L.xo, srow0 + w) + i0 + 3;
            Bn[w][0] = row[0];
            const float4 m = *reinterpret_cast<const float4*>(row + 1);
            Bn[w][1] = m.x;
            Bn[w][2] = m.y;
            Bn[w][3] = m.z;
            Bn[w][4] = m.w;
            Bn[w][5] = row[5];
        }
        if (MODE == 3) {
            // x' = x + P e. The window rows j0-1 .. j0+RPT lie between coarse rows jc .. jc+RPT
            // (jc = (j0-1) >> 1); their coarse nodes 2t-1 .. 2t+2 sit at positions 2t+3 .. 2t+6. Blend the
            // two staged coarse planes in z (odd P), then the coarse rows in y (odd fine rows), then x.
            const float* C0 = reinterpret_cast<const float*>(base + L.co);
            const float* C1 = reinterpret_cast<const float*>(base + L.co1);
            const int cr = ((j0 - 1) >> 1) - ((y0 - 1) >> 1);
            const bool oz = P & 1;
            float Cz[RPT + 1][4];
#pragma unroll
            for (int rr = 0; rr <= RPT; ++rr) {
                const float* p0 = C0 + (cr + rr) * a.crowlen + 2 * t + 3;
                const float* p1 = C1 + (cr + rr) * a.crowlen + 2 * t + 3;
#pragma unroll
                for (int c = 0; c < 4; ++c) Cz[rr][c] = oz ? 0.5f * (p0[c] + p1[c]) : p0[c];
            }
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const int jf = j0 - 1 + w;
                const int b0 = (jf >> 1) - ((j0 - 1) >> 1);
                const bool oj = jf & 1;
                float cyv[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float lo = Cz[0][c], hi = Cz[min(1, RPT)][c];
#pragma unroll
                    for (int u = 1; u <= RPT; ++u)
                        if (b0 == u) {
                            lo = Cz[u][c];
                            hi = Cz[min(u + 1, RPT)][c];
                        }
                    cyv[c] = oj ? 0.5f * (lo + hi) : lo;
                }
                Bn[w][0] += 0.5f * (cyv[0] + cyv[1]);
                Bn[w][1] += cyv[1];
                Bn[w][2] += 0.5f * (cyv[1] + cyv[2]);
                Bn[w][3] += cyv[2];
                Bn[w][4] += 0.5f * (cyv[2] + cyv[3]);
                Bn[w][5] += cyv[3];
            }
        }
        if (s < 1) return;
        float S[RPT + 1][5], SX[RPT + 1][4], SY[RPT][5];
#pragma unroll
        for (int w = 0; w <= RPT; ++w) {
            const float* row = srow(L.sa, L.so, srow0 + w) + i0 + 3;  // cells i0-1 .. i0+3
            S[w][0] = row[0];
            const float4 m = *reinterpret_cast<const float4*>(row + 1);
            S[w][1] = m.x;
            S[w][2] = m.y;
            S[w][3] = m.z;
            S[w][4] = m.w;
        }
#pragma unroll
        for (int w = 0; w <= RPT; ++w)
#pragma unroll
            for (int q = 0; q < 4; ++q) SX[w][q] = S[w][q] + S[w][q + 1];
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int q = 0; q < 5; ++q) SY[r][q] = S[r][q] + S[r + 1][q];
        const int k = P - 1;  // node plane completed at this step (s >= 2)
        const bool dk = (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]);
        // overset mask (Jacobi and residual only): masked nodes of plane k are held at 0 like Dirichlet
        // nodes; bit r*4+q as in dmask
        unsigned mk = 0;
        if (MODE <= 1 && g.mask) {
            if (s >= 2) {
#pragma unroll
                for (int r = 0; r < RPT; ++r)
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q < nact && !((mw[r] >> (8 * q)) & 0xffu)) mk |= 1u << (r * 4 + q);
            }
            // the next plane's words (plane P, completed at the next step): the thread's 4 mask bytes as one
            // word (i0 + kOX and the row / plane strides are multiples of 4; bytes past the last node stay
            // inside the padded row)
            if (P < g.nu[2]) {
#pragma unroll
                for (int r = 0; r < RPT; ++r)
                    mw[r] = j0 + r < g.nu[1]
                                ? __ldg(reinterpret_cast<const unsigned*>(g.mask + pidx(g.sy, g.sz, i0, j0 + r, P)))
                                : 0xffffffffu;
            }
        }
        float v[RPT][4];
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            float bb[4] = {0.f, 0.f, 0.f, 0.f};
            if (s >= 2) {
                const float4 bq = *reinterpret_cast<const float4*>(srow(L.ba, L.bo, srow0 + r) + 4 + i0);
                bb[0] = bq.x;
                bb[1] = bq.y;
                bb[2] = bq.z;
                bb[3] = bq.w;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float cA = Ao[r + 1][q + 1], cB = Bn[r + 1][q + 1];
                const float sgl = SX[r][q] + SX[r + 1][q];  // sigma of the layer's 4 cells around the node
                // in-plane and body diagonals (shared by both nodes), then the xz / yz diagonals of each
                float G0 = S[r][q] * ((Ao[r][q] - cA) + (Bn[r][q] - cA));
                float G1 = S[r + 1][q] * ((Ao[r + 2][q] - cA) + (Bn[r + 2][q] - cA));
                G0 = fmaf(S[r][q + 1], (Ao[r][q + 2] - cA) + (Bn[r][q + 2] - cA), G0);
                G1 = fmaf(S[r + 1][q + 1], (Ao[r + 2][q + 2] - cA) + (Bn[r + 2][q + 2] - cA), G1);
                const float G = G0 + G1;
                float xa = SY[r][q] * (Bn[r + 1][q] - cA);
                xa = fmaf(SY[r][q + 1], Bn[r + 1][q + 2] - cA, xa);
                xa = fmaf(SX[r][q], Bn[r][q + 1] - cA, xa);
                xa = fmaf(SX[r + 1][q], Bn[r + 2][q + 1] - cA, xa);
                float xb = SY[r][q] * (Ao[r + 1][q] - cB);
                xb = fmaf(SY[r][q + 1], Ao[r + 1][q + 2] - cB, xb);
                xb = fmaf(SX[r][q], Ao[r][q + 1] - cB, xb);
                xb = fmaf(SX[r + 1][q], Ao[r + 2][q + 1] - cB, xb);
                if (s >= 2) {
                    // node plane P-1 (registers Ao) gets its upper half and is complete
                    const float ax = a.k3 * (acc[r][q] + (G + xa));
                    float val;
                    if (MODE == 1 || MODE == 2)
                        val = bb[q] - ax;
                    else
                        val = fmaf(a.omega * (bb[q] - ax), rcp_approx(a.k0 * (ss[r][q] + sgl)), cA);
                    v[r][q] = (dk || (((dmask | mk) >> (r * 4 + q)) & 1u)) ? 0.f : val;
                }
                // node plane P (registers Bn) gets its lower half
                acc[r][q] = fmaf(-2.f * (cB - cA), sgl, G) + xb;
                ss[r][q] = sgl;
            }
        }
        if (s < 2) return;
        if (MODE == 2) {
            // stage the residual rows; the plane is restricted at the next step, after its barrier
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                float* Rr = R + ((s & 1) * Sh::TYR + srow0 + r) * a.rstride;
                *reinterpret_cast<float4*>(Rr + 4 + i0) = make_float4(v[r][0], v[r][1], v[r][2], v[r][3]);
                if (t == TX - 1) Rr[3] = g.per[0] ? v[r][3] : 0.f;  // node -1 (periodic: n-1 = 4 TX - 1)
            }
        } else {
#pragma unroll
            for (int r = 0; r < RPT; ++r)
                if (j0 + r < g.nu[1] && nact > 0) store4(a.out, g, i0, j0 + r, k, v[r], nact);
        }
    };

    float A[W][6], B[W][6];
#pragma unroll
    for (int r = 0; r < W; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) A[r][c] = B[r][c] = 0.f;
    int consumed = 0;
    for (int s = 0; s < nsteps; s += 2) {
        __syncthreads();  // every thread is done with step s-1 (its stage and the scratch rows)
        if (abort_flag) break;
        if (tid == 0 && s + kNS - 1 < nsteps) {
            fence_proxy_async();
            issue(s + kNS - 1);
        }
        step(s, A, B);
        consumed = s + 1;
        if (s + 1 >= nsteps) break;
        __syncthreads();
        if (abort_flag) break;
        if (tid == 0 && s + kNS < nsteps) {
            fence_proxy_async();
            issue(s + kNS);
        }
        step(s + 1, B, A);
        consumed = s + 2;
    }
    __syncthreads();
    if (MODE == 2 && !abort_flag && nsteps >= 3) restrict_plane(kend - 1, (nsteps - 1) & 1);
    if (abort_flag && tid == 0) {
        // copies still in flight: steps consumed .. issued-1 (bounded waits)
        for (uint32_t s = (uint32_t)consumed; s < issued; ++s)
            (void)mbar_wait_bounded(&bar[s % kNS], (s / kNS) & 1, nullptr);
    }
}

// ------------------------------------------------------------------------------------- host side
// 4-D tensor map over a padded level array: {bw, nbx, rows, planes}, box {bw, nbx, box_rows, 1}
struct Map4Key {
    const void* base;
    int bw, nbx, rows;
    long long sz, count;
    bool operator<(const Map4Key& o) const
    {
        return std::tie(base, bw, nbx, rows, sz, count) < std::tie(o.base, o.bw, o.nbx, o.rows, o.sz, o.count);
    }
};
std::mutex g_map4_mu;
std::map<Map4Key, CUtensorMap> g_maps4;

int row_boxes(int rowlen, int* bw)
{
    // the largest divisor of the row length that is a multiple of 4 floats and at most 256
    for (int w = 256; w >= 4; w -= 4)
        if (rowlen % w == 0) {
            *bw = w;
            return rowlen / w;
        }
    return 0;
}

int make_map4(const void* base, long long sy, long long sz, long long count, int box_rows, CUtensorMap* out)
{
    int bw = 0;
    const int nbx = row_boxes((int)sy, &bw);
    if (nbx <= 0 || nbx > 256) {
        set_error("vsweep32: padded row length has no TMA box split");
        return GBP_BAD_ARG;
    }
    Map4Key key{base, bw, nbx, box_rows, sz, count};
    std::lock_guard<std::mutex> lk(g_map4_mu);
    auto it = g_maps4.find(key);
    if (it != g_maps4.end()) {
        *out = it->second;
        return GBP_OK;
    }
    auto fn = tensor_map_encoder();
    if (!fn) {
        set_error("cuTensorMapEncodeTiled is unavailable from the driver");
        return GBP_CUDA_ERROR;
    }
    CUtensorMap m;
    const cuuint64_t dims[4] = {(cuuint64_t)bw, (cuuint64_t)nbx, (cuuint64_t)(sz / sy), (cuuint64_t)(count / sz)};
    const cuuint64_t strides[3] = {(cuuint64_t)(bw * 4), (cuuint64_t)(sy * 4), (cuuint64_t)(sz * 4)};
    const cuuint32_t box[4] = {(cuuint32_t)bw, (cuuint32_t)nbx, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled (4-D) failed (code " + std::to_string((int)r) + ")");
        return GBP_CUDA_ERROR;
    }
    g_maps4[key] = m;
    *out = m;
    return GBP_OK;
}

template <int MODE, int TY, int TXM>
int launch(const NodalGeom& g, const NodalGeom* gc, const float* s, const float* x, const float* b,
           const float* e, float* out, float omega, unsigned* err, cudaStream_t st)
{
    constexpr int RPT = GBP_VS_RPT;
    using Sh = VsShape<MODE, TY, RPT>;
    const int TX = (g.nu[0] + 3) / 4;
    VsArgs a;
    a.g = g;
    a.gc = gc ? *gc : g;
    a.out = out;
    a.k0 = (float)g.K[0];
    a.k3 = (float)g.K[3];
    a.omega = omega;
    a.rowlen = (int)g.sy;
    a.crowlen = gc ? (int)gc->sy : 4;
    a.rstride = 4 * TX + 8;
    a.err = err;
    // mode 2 stages the row below the tile through one-row maps (x1, s1, b1)
    CUtensorMap mx, ms, mb, mc, mx1, ms1, mb1;
    const int sub = MODE == 2 ? 1 : 0;
    int rc = make_map4(x, g.sy, g.sz, g.count, Sh::XR - sub, &mx);
    if (!rc) rc = make_map4(s, g.sy, g.sz, g.count, Sh::SR - sub, &ms);
    if (!rc) rc = make_map4(b, g.sy, g.sz, g.count, Sh::BR - sub, &mb);
    if (!rc && MODE == 2) rc = make_map4(x, g.sy, g.sz, g.count, 1, &mx1);
    if (!rc && MODE == 2) rc = make_map4(s, g.sy, g.sz, g.count, 1, &ms1);
    if (!rc && MODE == 2) rc = make_map4(b, g.sy, g.sz, g.count, 1, &mb1);
    if (!rc && MODE == 3) rc = make_map4(e, gc->sy, gc->sz, gc->count, Sh::CR, &mc);
    if (rc) return rc;
    if (MODE != 3) mc = mb;
    if (MODE != 2) mx1 = mx, ms1 = ms, mb1 = mb;
    const int smem = smem_bytes<MODE, TY, RPT>(a.rowlen, a.crowlen, a.rstride);
    auto kern = k_vsweep32<MODE, TY, TXM, RPT>;
    static int configured = 0, resident = 1;
    if (configured < smem) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kern, TX * Sh::TTR, smem) == cudaSuccess && r > 0)
            resident = r;
        configured = smem;
    }
    const int ty = (g.nu[1] + TY - 1) / TY;
    // z chunks: whole waves of resident CTAs; an even chunk length in mode 2 (the restriction pairs planes)
    int nz = sweep_z_chunks(g, ty, resident);
    int kchunk = (g.nu[2] + nz - 1) / nz;
    if ((MODE == 2 || MODE == 3) && (kchunk & 1)) ++kchunk;
    a.kchunk = kchunk;
    dim3 grid(1, ty, (g.nu[2] + kchunk - 1) / kchunk);
    kern<<<grid, dim3(TX, Sh::TTR), smem, st>>>(mx, ms, mb, mc, mx1, ms1, mb1, a);
    return GBP_OK;
}

}  // namespace

bool vsweep32_supported(const NodalGeom& g)
{
    const long long nodes = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    int bw = 0;
    // isotropic, whole rows in one CTA (periodic x: a multiple of 4 nodes so that node
    // n-1 is the last thread's last node); a thread reads staged columns up to 4 TX + 4, which must lie
    // inside the padded row
    const int TX = (g.nu[0] + 3) / 4;
    return g.iso && nodes >= (1ll << 20) && g.nu[0] <= 4 * kMaxTX && g.nu[0] >= 16 && g.nu[1] >= 4 &&
           g.nu[2] >= 4 && (!g.per[0] || g.nu[0] % 4 == 0) && 4 * TX + 5 <= (int)g.sy &&
           row_boxes((int)g.sy, &bw) > 0;
}

bool vsweep32_transfer_supported(const NodalGeom& g, const NodalGeom& gc)
{
    // the coarse level is the standard coarsening by 2 of this one; no overset mask on either (the fused
    // prolongation would add the coarse correction to masked fine nodes)
    if (g.mask || gc.mask) return false;
    for (int d = 0; d < 3; ++d)
        if (gc.n[d] * 2 != g.n[d] || gc.per[d] != g.per[d]) return false;
    int bw = 0;
    // a periodic y direction needs whole CTAs of rows (TY = 8 divides it); the prolongation reads coarse
    // columns up to 2 TX + 6
    const int TX = (g.nu[0] + 3) / 4;
    return vsweep32_supported(g) && !gc.mask && row_boxes((int)gc.sy, &bw) > 0 && (!g.per[1] || g.nu[1] % 8 == 0) &&
           2 * TX + 7 <= (int)gc.sy;
}

// rows per CTA by the row width: 8 (<= 128 nodes), GBP_VS_TY_256 (<= 256), GBP_VS_TY_512 (<= 512)
template <int MODE>
static int launch_any(const NodalGeom& g, const NodalGeom* gc, const float* s, const float* x, const float* b,
                      const float* e, float* out, float omega, unsigned* err, cudaStream_t st)
{
    const int TX = (g.nu[0] + 3) / 4;
    if (TX <= 32) return launch<MODE, 8, 32>(g, gc, s, x, b, e, out, omega, err, st);
    if (TX <= 64) return launch<MODE, GBP_VS_TY_256, 64>(g, gc, s, x, b, e, out, omega, err, st);
    return launch<MODE, GBP_VS_TY_512, 128>(g, gc, s, x, b, e, out, omega, err, st);
}

int vsweep32(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
             unsigned* err, cudaStream_t st)
{
    return mode == 0 ? launch_any<0>(g, nullptr, s, x, b, nullptr, out, omega, err, st)
                     : launch_any<1>(g, nullptr, s, x, b, nullptr, out, omega, err, st);
}

int vsweep32_resid_restrict(const NodalGeom& g, const NodalGeom& gc, const float* s, const float* x, const float* b,
                            float* bc, unsigned* err, cudaStream_t st)
{
    return launch_any<2>(g, &gc, s, x, b, nullptr, bc, 0.f, err, st);
}

int vsweep32_prolong_jacobi(const NodalGeom& g, const NodalGeom& gc, const float* s, const float* x, const float* ec,
                            const float* b, float* out, float omega, unsigned* err, cudaStream_t st)
{
    return launch_any<3>(g, &gc, s, x, b, ec, out, omega, err, st);
}

void vsweep32_forget_maps(const void* pool_base, size_t pool_bytes)
{
    std::lock_guard<std::mutex> lk(g_map4_mu);
    const char* lo = static_cast<const char*>(pool_base);
    const char* hi = lo + pool_bytes;
    for (auto it = g_maps4.begin(); it != g_maps4.end();) {
        const char* p = static_cast<const char*>(it->first.base);
        if (p >= lo && p < hi)
            it = g_maps4.erase(it);
        else
            ++it;
    }
}

}  // namespace gbp
