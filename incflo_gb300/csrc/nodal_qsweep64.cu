// FP64 level-0 sweep of the isotropic nodal operator in shared-sum form.
//
// With equal spacing the Q1 element couples a node only to its face and body diagonals
// (coefficient kc, K[1] = K[2] = K[4] = 0), and
//   (A x)_n = kc * ( sum_c sigma_c Q_c  -  5 x_n sum_c sigma_c  -  sum_e W_e x_e )
// over the 8 cells c around n (Q_c = the sum of the cell's 8 corner values) and the 6 edge
// neighbours e (W_e = the sigma of the 4 cells that contain both nodes). Q_c and sigma_c Q_c are
// computed once per cell and shared by its 8 nodes; the sigma sums W_e and sum_c sigma_c do not change
// between sweeps and are precomputed per node (k_qweights64). That is about 21 FP64 operations per
// node instead of about 45 for the per-cell form: on GB300 the FP64 pipe, not HBM, bounds this kernel.
//
// Layout: a CTA of (32+1) x (8+1) threads marches a z range; thread (tx, ty) owns cell and node
// (x0-1+tx, y0-1+ty). Every thread forms sigma_c Q_c of its cell for the current cell layer into a
// double-buffered shared tile (one barrier per plane); threads with tx, ty >= 1 then add the four cells
// of the layer around their node and finish the node from the previous layer's sum, which they carry.
#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "nodal_sweep.h"

namespace gbp {

namespace {

constexpr int QX = 32, QY = 8;
constexpr int QTX = QX + 1, QTY = QY + 1;

__device__ __forceinline__ bool q_alias(const NodalGeom& g, int i, int j, int k)
{
    return (g.per[0] && (i <= 1 || i == g.n[0] - 1)) || (g.per[1] && (j <= 1 || j == g.n[1] - 1)) ||
           (g.per[2] && (k <= 1 || k == g.n[2] - 1));
}

// wsum = sum of the 8 cells around each node; wx / wy / wz = sigma sum of the 4 cells around the edge
// from node (i,j,k) to (i+1,j,k) / (i,j+1,k) / (i,j,k+1). Written over index ranges -1..nu so that the
// sweep can read the edge to a node's low neighbour; padding cells are 0, periodic ones aliased.
// z-marching tile (33 x 9 threads: node columns x0-1 .. x0+31, y0-1 .. y0+7 and the cell columns one
// lower), separable sums per cell layer: Px = x pair, Q = Px + Px(j-1) (4 cells around a z edge),
// Y = y pair; then wsum = Q(k-1) + Q(k), wz = Q(k), wx = Y(k-1) + Y(k), wy = Px(k-1) + Px(k).
__global__ void __launch_bounds__(QTX* QTY) k_qweights64(NodalGeom g, const double* __restrict__ s,
                                                         double* __restrict__ wsum, double* __restrict__ wx,
                                                         double* __restrict__ wy, double* __restrict__ wz, int kchunk)
{
    __shared__ double T[2][QTY + 1][QTX + 1];
    const int tx = threadIdx.x % QTX, ty = threadIdx.x / QTX;
    // node column of this thread: (i, j) = (x0 - 1 + tx, y0 - 1 + ty); its cells are i-1..i, j-1..j
    const int i = blockIdx.x * QX - 1 + tx, j = blockIdx.y * QY - 1 + ty;
    const int kbeg = blockIdx.z * kchunk - 1;  // node planes -1 .. nu-1
    const int kend = min(kbeg + kchunk, g.nu[2]);
    // neighbouring tiles share their edge column / row: the lower tile writes it
    const bool node = (tx >= 1 || blockIdx.x == 0) && (ty >= 1 || blockIdx.y == 0) && i < g.nu[0] && j < g.nu[1];
    double Qp = 0.0, Yp = 0.0, Pp = 0.0;
    for (int L = kbeg - 1; L < kend; ++L) {
        const int buf = (L - kbeg + 1) & 1;
        // stage cells (x0-2 .. x0+31, y0-2 .. y0+7) of layer L: tile (tx, ty) = cell (i - 1, j - 1),
        // plus the extra high column / row; cells below -1 are never read (zero)
        for (int q = threadIdx.x; q < (QTX + 1) * (QTY + 1); q += QTX * QTY) {
            const int cx = q % (QTX + 1), cy = q / (QTX + 1);
            const int a = blockIdx.x * QX - 2 + cx, b = blockIdx.y * QY - 2 + cy;
            double v = 0.0;
            if (L >= -1 && a >= -1 && b >= -1 && a <= g.nu[0] - 1 && b <= g.nu[1] - 1) v = s[pidx(g.sy, g.sz, a, b, L)];
            T[buf][cy][cx] = v;
        }
        __syncthreads();
        // this node's cells in the tile: (i-1, j-1) = (tx, ty), (i, j-1) = (tx+1, ty), (i-1, j) = (tx, ty+1), (i, j) = (tx+1, ty+1)
        const double Px = T[buf][ty + 1][tx] + T[buf][ty + 1][tx + 1];   // cells (i-1..i, j)
        const double Pxm = T[buf][ty][tx] + T[buf][ty][tx + 1];          // cells (i-1..i, j-1)
        const double Q = Px + Pxm;
        const double Y = T[buf][ty][tx + 1] + T[buf][ty + 1][tx + 1];    // cells (i, j-1..j)
        if (node && L >= kbeg) {
            // node (i, j, L): layers L-1 (previous) and L
            const int k = L;
            const long long p = pidx(g.sy, g.sz, i, j, k);
            if (i >= 0 && j >= 0 && k >= 0) wsum[p] = Qp + Q;
            if (j >= 0 && k >= 0) wx[p] = Yp + Y;
            if (i >= 0 && k >= 0) wy[p] = Pp + Px;
            if (i >= 0 && j >= 0) wz[p] = Q;
        }
        Qp = Q;
        Yp = Y;
        Pp = Px;
    }
}

template <int MODE>
__global__ void __launch_bounds__(QTX * QTY) k_qsweep64(NodalGeom g, const double* __restrict__ x,
                                                        const double* __restrict__ b, const double* __restrict__ s,
                                                        QWeights w, double* __restrict__ out, double omega,
                                                        int kchunk, unsigned long long* norm)
{
    __shared__ double T[2][QTY][QTX];
    const int tx = threadIdx.x % QTX, ty = threadIdx.x / QTX;
    const int i = blockIdx.x * QX - 1 + tx, j = blockIdx.y * QY - 1 + ty;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    // a thread whose cell lies outside the padded box still takes part in the barriers
    const bool inbox = i < g.nu[0] && j < g.nu[1];
    const bool owner = tx >= 1 && ty >= 1 && i < g.nu[0] && j < g.nu[1];
    const bool dxy = owner && ((g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) ||
                               (g.dhi[1] && j == g.n[1]));
    const long long sy = g.sy, sz = g.sz;
    const double kc = g.K[3];
    long long p = pidx(sy, sz, i, j, kbeg - 1);  // node (i, j, k) for the current k
    // q = sum of the 4 nodes (i..i+1, j..j+1) of a node plane
    auto qsum = [&](long long pp) { return (x[pp] + x[pp + 1]) + (x[pp + sy] + x[pp + sy + 1]); };
    double q_lo = inbox ? qsum(p) : 0.0;  // plane kbeg-1
    double u_lo = 0.0;                    // layer kbeg-1 sum around the node
    unsigned long long nkey = 0;
    double xm = 0.0, xc = 0.0, wzm = 0.0;
    if (owner) {
        xm = x[p];
        xc = x[p + sz];
        wzm = w.wz[p];
    }
    for (int k = kbeg - 1; k < kend; ++k) {
        // cell layer k: (i, j, k) .. (i+1, j+1, k+1)
        const long long pc = pidx(sy, sz, i, j, k);
        const double q_hi = inbox ? qsum(pc + sz) : 0.0;
        const int buf = (k - kbeg + 1) & 1;
        T[buf][ty][tx] = inbox ? s[pc] * (q_lo + q_hi) : 0.0;
        q_lo = q_hi;
        __syncthreads();
        if (owner) {
            const double u = (T[buf][ty - 1][tx - 1] + T[buf][ty - 1][tx]) + (T[buf][ty][tx - 1] + T[buf][ty][tx]);
            if (k >= kbeg) {
                // node (i, j, k): layers k-1 (u_lo) and k (u)
                const long long pn = pc;
                const double xp = x[pn + sz];
                double v = 0.0;
                if (!(dxy || (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]) || (g.mask && !g.mask[pn]))) {
                    const double ssum = w.wsum[pn];
                    const double wzp = w.wz[pn];
                    double e = x[pn + 1] * w.wx[pn];
                    e = fma(x[pn - 1], w.wx[pn - 1], e);
                    e = fma(x[pn + sy], w.wy[pn], e);
                    e = fma(x[pn - sy], w.wy[pn - sy], e);
                    e = fma(xp, wzp, e);
                    e = fma(xm, wzm, e);
                    const double ax = kc * (fma(-5.0 * xc, ssum, u_lo + u) - e);
                    const double bv = b[pn];
                    if (MODE == 0) {
                        const double diag = g.K[0] * ssum;
                        const double ad = fabs(diag);
                        const double rd = (ad > 1e-30 && ad < 1e30) ? (double)__frcp_rn((float)diag) : 1.0 / diag;
                        v = xc + omega * (bv - ax) * rd;
                    } else {
                        v = bv - ax;
                        if (norm) {
                            // |v| / V_node as an integer key (boundary nodes: V / 2^e, exact scaling)
                            const int e = (!g.per[0] && (i == 0 || i == g.n[0])) + (!g.per[1] && (j == 0 || j == g.n[1])) +
                                          (!g.per[2] && (k == 0 || k == g.n[2]));
                            const unsigned long long kb = e == 0 ? abs_key(v) : abs_key(v * (double)(1 << e));
                            nkey = kb > nkey ? kb : nkey;
                        }
                    }
                    wzm = wzp;
                } else {
                    wzm = w.wz[pn];
                }
                if (q_alias(g, i, j, k))
                    store_node(out, g, i, j, k, v);
                else
                    out[pn] = v;
                xm = xc;
                xc = xp;
            }
            u_lo = u;
        }
    }
    if (MODE == 1 && norm) {
        nkey = block_max_key(nkey);
        if (threadIdx.x == 0) atomic_max_nonneg(norm, key_value(nkey) * g.ivol);
    }
}

}  // namespace

bool qsweep_supported(const NodalGeom& g) { return g.iso != 0; }

void nodal_qweights64(const NodalGeom& g, const double* s64, const QWeights& w, cudaStream_t st)
{
    // node columns -1 .. nu-1 in tiles of 32 x 8 (tile origin x0 - 1), node planes -1 .. nu-1
    const int bx = (g.nu[0] + QX - 1) / QX, by = (g.nu[1] + QY - 1) / QY;
    const int nz = g.nu[2] + 1;
    const int want = std::max(1, 4 * sm_count_cached() * 6 / std::max(1, bx * by));
    const int kchunk = std::max(4, (nz + want - 1) / want);
    k_qweights64<<<dim3(bx, by, (nz + kchunk - 1) / kchunk), QTX * QTY, 0, st>>>(g, s64, w.wsum, w.wx, w.wy, w.wz,
                                                                                kchunk);
}

void nodal_qsweep64(const NodalGeom& g, int mode, const double* s64, const QWeights& w, const double* x,
                    const double* b, double* out, double omega, unsigned long long* norm, cudaStream_t st)
{
    const int bx = (g.nu[0] + QX - 1) / QX, by = (g.nu[1] + QY - 1) / QY;
    // z chunks: enough CTAs for about 4 waves of (33 x 9)-thread blocks
    const int want = std::max(1, 4 * sm_count_cached() * 6 / std::max(1, bx * by));
    const int kchunk = std::max(4, (g.nu[2] + want - 1) / want);
    const dim3 grid(bx, by, (g.nu[2] + kchunk - 1) / kchunk);
    if (mode == 0)
        k_qsweep64<0><<<grid, QTX * QTY, 0, st>>>(g, x, b, s64, w, out, omega, kchunk, norm);
    else
        k_qsweep64<1><<<grid, QTX * QTY, 0, st>>>(g, x, b, s64, w, out, omega, kchunk, norm);
}

}  // namespace gbp
