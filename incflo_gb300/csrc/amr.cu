// Two-level (AMR) composite nodal projection (see amr.h).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

#include "amr.h"
#include "gbp_internal.cuh"
#include "nodal_kernels.h"
#include "nodal_sweep.h"

namespace gbp {

namespace {

constexpr int kT = 256;

// fine node classes (unique nodes of the fine bounding box)
enum : unsigned char { F_OUT = 0, F_DOF = 1, F_ALIGNED = 2, F_HANGING = 3, F_FIXED = 4 };
// coarse node classes
enum : unsigned char { C_DOF = 0, C_COVERED = 1, C_IFACE = 2, C_FIXED = 3 };

__device__ __forceinline__ double* at4(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
           (long long)n * a.nstride;
}

struct BoxEntry {
    int lo[3], hi[3];  // fine cells (global)
    gbp_array4 a;      // the box's array (or data == nullptr)
};

// ------------------------------------------------------------------------------------------ set-up
// fine leaf-cell mask over the bounding box (padded cell layout, periodic aliases)
__global__ void k_amr_cmask_fine(NodalGeom gf, const BoxEntry* __restrict__ bx, int off0, int off1, int off2,
                                 unsigned char* __restrict__ m)
{
    const BoxEntry b = bx[blockIdx.y];
    const int ex = b.hi[0] - b.lo[0] + 1, ey = b.hi[1] - b.lo[1] + 1, ez = b.hi[2] - b.lo[2] + 1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)ex * ey * ez;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        split3(t, ex, ey, (long long)ex * ey * ez, i, j, k);
        i += b.lo[0] - off0;
        j += b.lo[1] - off1;
        k += b.lo[2] - off2;
        store_sigma_cell(m, gf, i, j, k, (unsigned char)1);
    }
}

// coarse leaf-cell mask: a coarse cell is covered when its first fine child is a fine cell
__global__ void k_amr_cmask_coarse(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ mf, int off0,
                                   int off1, int off2, unsigned char* __restrict__ mc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.n[0] || j >= gc.n[1] || k >= gc.n[2]) return;
    const int fi = 2 * i - off0, fj = 2 * j - off1, fk = 2 * k - off2;
    const bool in = fi >= 0 && fj >= 0 && fk >= 0 && fi < gf.n[0] && fj < gf.n[1] && fk < gf.n[2] &&
                    mf[pidx(gf.sy, gf.sz, fi, fj, fk)];
    store_sigma_cell(mc, gc, i, j, k, (unsigned char)(in ? 0 : 1));
}

// fine node class: in (all in-domain fine cells around it are fine cells), aligned interface,
// hanging interface, or outside; nodes of the region on a Dirichlet side are fixed
__global__ void k_amr_classify_fine(NodalGeom gf, const unsigned char* __restrict__ mf, int off0, int off1, int off2,
                                    int nd0, int nd1, int nd2, int dper0, int dper1, int dper2,
                                    unsigned char* __restrict__ cls)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const int off[3] = {off0, off1, off2}, nd[3] = {nd0, nd1, nd2}, dper[3] = {dper0, dper1, dper2};
    const int node[3] = {i, j, k};
    int tot = 0, in = 0;
    for (int c = 0; c < 8; ++c) {
        int cl[3];
        bool dom = true;
        for (int d = 0; d < 3; ++d) {
            int v = node[d] - 1 + ((c >> d) & 1);  // local cell index
            int gv = v + off[d];                   // global fine cell index
            if (dper[d]) {
                gv = (gv % nd[d] + nd[d]) % nd[d];
            } else if (gv < 0 || gv >= nd[d]) {
                dom = false;
            }
            if (gf.per[d]) v = (v % gf.n[d] + gf.n[d]) % gf.n[d];
            cl[d] = v;
        }
        if (!dom) continue;
        ++tot;
        if (cl[0] >= 0 && cl[1] >= 0 && cl[2] >= 0 && cl[0] < gf.n[0] && cl[1] < gf.n[1] && cl[2] < gf.n[2] &&
            mf[pidx(gf.sy, gf.sz, cl[0], cl[1], cl[2])])
            ++in;
    }
    unsigned char c = F_OUT;
    if (in > 0) {
        if (in == tot) {
            c = node_is_dirichlet(gf, i, j, k) ? F_FIXED : F_DOF;
        } else {
            const bool even = ((i + off0) % 2 == 0) && ((j + off1) % 2 == 0) && ((k + off2) % 2 == 0);
            c = even ? F_ALIGNED : F_HANGING;
        }
    }
    cls[pidx(gf.sy, gf.sz, i, j, k)] = c;
}

// local fine node of global fine node position g (periodic wrap in the fine box), or false
// v into [0, n) for arguments a few periods out at most (integer division is slow on the GPU)
__device__ __forceinline__ int wrap_period(int v, int n)
{
    while (v < 0) v += n;
    while (v >= n) v -= n;
    return v;
}

__device__ __forceinline__ bool fine_local(const NodalGeom& gf, const int off[3], const int gpos[3], int out[3])
{
    for (int d = 0; d < 3; ++d) {
        int v = gpos[d] - off[d];
        if (gf.per[d]) {
            v = wrap_period(v, gf.n[d]);
        } else if (v < 0 || v >= gf.nu[d]) {
            return false;
        }
        out[d] = v;
    }
    return true;
}

// coarse node (I, J, K) -> node of the fine box's coarsened level g1 (origin o = off / 2), or false
__device__ __forceinline__ bool coarse_to_g1(const NodalGeom& g1, const int o[3], const int I[3], int q[3])
{
    for (int d = 0; d < 3; ++d) {
        int v = I[d] - o[d];
        if (g1.per[d]) {
            v = wrap_period(v, g1.n[d]);
        } else if (v < 0 || v >= g1.nu[d]) {
            return false;
        }
        q[d] = v;
    }
    return true;
}

// out (whole coarse level) = the coarse unknowns' own residual + the full weighting r1 of the fine
// unknowns' residual (on g1, the fine box coarsened by 2), except on fixed nodes
__global__ void k_amr_combine(NodalGeom gc, NodalGeom g1, const unsigned char* __restrict__ ccls, int o0, int o1,
                              int o2, const float* __restrict__ rc, const float* __restrict__ r1, float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    float v = (c == C_DOF || c == C_IFACE) ? rc[p] : 0.f;
    const int o[3] = {o0, o1, o2}, I[3] = {i, j, k};
    int q[3];
    if (c != C_FIXED && coarse_to_g1(g1, o, I, q)) v += r1[pidx(g1.sy, g1.sz, q[0], q[1], q[2])];
    store_node(out, gc, i, j, k, v);
}

// x1 (g1, the fine box coarsened by 2) = the coarse-level values at the same positions (aliases written)
__global__ void k_amr_gather_g1(NodalGeom gc, NodalGeom g1, int o0, int o1, int o2, const float* __restrict__ xc,
                                float* x1)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= g1.nu[0] || j >= g1.nu[1] || k >= g1.nu[2]) return;
    const int o[3] = {o0, o1, o2}, q[3] = {i, j, k};
    int I[3];
    for (int d = 0; d < 3; ++d) {
        I[d] = q[d] + o[d];
        if (gc.per[d]) I[d] = wrap_period(I[d], gc.n[d]);
    }
    store_node(x1, g1, i, j, k, xc[pidx(gc.sy, gc.sz, I[0], I[1], I[2])]);
}

__global__ void k_amr_classify_coarse(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ fcls, int off0,
                                      int off1, int off2, unsigned char* __restrict__ ccls)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const int off[3] = {off0, off1, off2};
    const int gpos[3] = {2 * i, 2 * j, 2 * k};
    int m[3];
    unsigned char fc = F_OUT;
    if (fine_local(gf, off, gpos, m)) fc = fcls[pidx(gf.sy, gf.sz, m[0], m[1], m[2])];
    unsigned char c;
    if (fc == F_DOF || fc == F_FIXED)
        c = C_COVERED;
    else if (node_is_dirichlet(gc, i, j, k))
        c = C_FIXED;
    else
        c = fc == F_ALIGNED ? C_IFACE : C_DOF;
    ccls[pidx(gc.sy, gc.sz, i, j, k)] = c;
}

// overset mask of the fine solver: 1 on the fine unknowns only (int nodes 0..n of the bounding box)
__global__ void k_amr_fine_mask(NodalGeom gf, const unsigned char* __restrict__ fcls, int* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > gf.n[0] || j > gf.n[1] || k > gf.n[2]) return;
    const int iu = gf.per[0] && i == gf.n[0] ? 0 : i;
    const int ju = gf.per[1] && j == gf.n[1] ? 0 : j;
    const int ku = gf.per[2] && k == gf.n[2] ? 0 : k;
    out[i + (long long)(gf.n[0] + 1) * (j + (long long)(gf.n[1] + 1) * k)] =
        fcls[pidx(gf.sy, gf.sz, iu, ju, ku)] == F_DOF;
}

// ------------------------------------------------------------------------------ fine data in / out
// bounding-box dense cell arrays <- per-box arrays (ncomp components), batched over the boxes
__global__ void k_amr_gather(const BoxEntry* __restrict__ bx, int off0, int off1, int off2, int nb0, int nb1, int nb2,
                             int ncomp, double* __restrict__ dst)
{
    const BoxEntry b = bx[blockIdx.y];
    if (!b.a.data) return;
    const int ex = b.hi[0] - b.lo[0] + 1, ey = b.hi[1] - b.lo[1] + 1, ez = b.hi[2] - b.lo[2] + 1;
    const long long ncell = (long long)nb0 * nb1 * nb2;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)ex * ey * ez;
         t += (long long)gridDim.x * blockDim.x) {
        int gi, gj, gk;
        split3(t, ex, ey, (long long)ex * ey * ez, gi, gj, gk);
        gi += b.lo[0];
        gj += b.lo[1];
        gk += b.lo[2];
        const long long q = (gi - off0) + (long long)nb0 * ((gj - off1) + (long long)nb1 * (gk - off2));
        for (int c = 0; c < ncomp; ++c) dst[q + c * ncell] = *at4(b.a, gi, gj, gk, c);
    }
}

__global__ void k_amr_scatter(const BoxEntry* __restrict__ bx, int off0, int off1, int off2, int nb0, int nb1, int nb2,
                              int ncomp, const double* __restrict__ src)
{
    const BoxEntry b = bx[blockIdx.y];
    if (!b.a.data) return;
    const int ex = b.hi[0] - b.lo[0] + 1, ey = b.hi[1] - b.lo[1] + 1, ez = b.hi[2] - b.lo[2] + 1;
    const long long ncell = (long long)nb0 * nb1 * nb2;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)ex * ey * ez;
         t += (long long)gridDim.x * blockDim.x) {
        int gi, gj, gk;
        split3(t, ex, ey, (long long)ex * ey * ez, gi, gj, gk);
        gi += b.lo[0];
        gj += b.lo[1];
        gk += b.lo[2];
        const long long q = (gi - off0) + (long long)nb0 * ((gj - off1) + (long long)nb1 * (gk - off2));
        for (int c = 0; c < ncomp; ++c) *at4(b.a, gi, gj, gk, c) = src[q + c * ncell];
    }
}

// per-box nodal arrays (nodes lo..hi+1) <- fine phi on all bounding-box nodes (dense, 0..n)
__global__ void k_amr_scatter_nodes(const BoxEntry* __restrict__ bx, int off0, int off1, int off2, int nb0, int nb1,
                                    const double* __restrict__ src, int accumulate)
{
    const BoxEntry b = bx[blockIdx.y];
    if (!b.a.data) return;
    const int ex = b.hi[0] - b.lo[0] + 2, ey = b.hi[1] - b.lo[1] + 2, ez = b.hi[2] - b.lo[2] + 2;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)ex * ey * ez;
         t += (long long)gridDim.x * blockDim.x) {
        int gi, gj, gk;
        split3(t, ex, ey, (long long)ex * ey * ez, gi, gj, gk);
        gi += b.lo[0];
        gj += b.lo[1];
        gk += b.lo[2];
        const long long q = (gi - off0) + (long long)(nb0 + 1) * ((gj - off1) + (long long)(nb1 + 1) * (gk - off2));
        double* p = at4(b.a, gi, gj, gk, 0);
        *p = accumulate ? *p + src[q] : src[q];
    }
}

// fine sigma on the bounding box cells (dense): scale / rho on fine cells, 0 elsewhere
__global__ void k_amr_sigma_fine(NodalGeom gf, const unsigned char* __restrict__ mf, const double* __restrict__ rho,
                                 int have_rho, double scale, double rho0, double* __restrict__ sig)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.n[0] || j >= gf.n[1] || k >= gf.n[2]) return;
    const long long q = i + (long long)gf.n[0] * (j + (long long)gf.n[1] * k);
    double v = 0.0;
    if (mf[pidx(gf.sy, gf.sz, i, j, k)]) v = have_rho ? scale / rho[q] : scale / rho0;
    sig[q] = v;
}

// sigma of the coarse level's V-cycles (dense cells): scale / rho on uncovered cells, the mean of the 8
// fine sigma on covered ones (those cells are not part of the composite system; the fine average makes
// the coarse correction match the fine operator there)
__global__ void k_amr_sigma_coarse(NodalGeom gc, const unsigned char* __restrict__ mc, gbp_array4 rho, int have_rho,
                                   double scale, double rho0, const double* __restrict__ sig_f, int off0, int off1,
                                   int off2, int nb0, int nb1, double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.n[0] || j >= gc.n[1] || k >= gc.n[2]) return;
    double v;
    if (mc[pidx(gc.sy, gc.sz, i, j, k)]) {
        v = have_rho ? scale / *at4(rho, i, j, k, 0) : scale / rho0;
    } else {
        v = 0.0;
        for (int q = 0; q < 8; ++q) {
            const int fi = 2 * i - off0 + (q & 1), fj = 2 * j - off1 + ((q >> 1) & 1), fk = 2 * k - off2 + (q >> 2);
            v += sig_f[fi + (long long)nb0 * (fj + (long long)nb1 * fk)];
        }
        v *= 0.125;
    }
    out[i + (long long)gc.n[0] * (j + (long long)gc.n[1] * k)] = v;
}

// coarse sigma with covered cells zeroed (whole padded arrays, aliases included)
__global__ void k_amr_mask_sigma(long long count, const double* __restrict__ s, const unsigned char* __restrict__ m,
                                 double* __restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) out[t] = m[t] ? s[t] : 0.0;
}

// out = scale * v over whole padded arrays (FP64 -> FP32: the composite residual as the right-hand side of
// the FP32 correction equation, the masked coarse sigma)
__global__ void k_amr_to32(long long count, const double* __restrict__ v, double scale, float* __restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) out[t] = (float)(scale * v[t]);
}

// out = scale * r on the fine unknowns, 0 elsewhere (unique nodes, aliases written): the fine part of the
// correction equation's right-hand side. The interface residuals are already folded into the coarse
// interface nodes; the FP32 composite residual adds them again from -A e only.
__global__ void k_amr_rhs32_fine(NodalGeom gf, const unsigned char* __restrict__ fcls, const double* __restrict__ r,
                                 double scale, float* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    store_node(out, gf, i, j, k, fcls[p] == F_DOF ? (float)(scale * r[p]) : 0.f);
}

// acc += e over whole padded arrays (the fine hierarchy's correction: zero on the masked nodes)
__global__ void k_amr_add32(long long count, const float* __restrict__ e, float* __restrict__ acc)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) acc[t] += e[t];
}

// ------------------------------------------------------------------------------ composite operator
__device__ __forceinline__ int cwrap(const NodalGeom& gc, int d, int v)
{
    return gc.per[d] ? wrap_period(v, gc.n[d]) : v;
}

// interface values of the fine level from the coarse one: aligned nodes copy, hanging nodes
// interpolate along the coarse face they lie on
template <typename T>
__device__ __forceinline__ void fill_fine_node(const NodalGeom& gc, const NodalGeom& gf, int off0, int off1, int off2,
                                               const T* __restrict__ pc, T* pf, int i, int j, int k)
{
    const int gpos[3] = {i + off0, j + off1, k + off2};
    T acc = 0;
    int nodd = 0;
    for (int d = 0; d < 3; ++d) nodd += gpos[d] & 1;
    const T w = nodd == 0 ? T(1) : (nodd == 1 ? T(0.5) : T(0.25));
    for (int q = 0; q < 8; ++q) {
        int I[3];
        bool use = true;
        for (int d = 0; d < 3; ++d) {
            const int sel = (q >> d) & 1;
            if (gpos[d] & 1) {
                I[d] = cwrap(gc, d, (gpos[d] - 1) / 2 + sel);
            } else {
                if (sel) use = false;
                I[d] = cwrap(gc, d, gpos[d] / 2);
            }
        }
        if (use) acc += pc[pidx(gc.sy, gc.sz, I[0], I[1], I[2])];
    }
    store_node(pf, gf, i, j, k, w * acc);
}

template <typename T>
__global__ void k_amr_fill_fine(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ fcls, int off0, int off1,
                                int off2, const T* __restrict__ pc, T* pf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const unsigned char c = fcls[pidx(gf.sy, gf.sz, i, j, k)];
    if (c != F_ALIGNED && c != F_HANGING) return;
    fill_fine_node<T>(gc, gf, off0, off1, off2, pc, pf, i, j, k);
}

// the same over the listed interface nodes only
template <typename T>
__global__ void k_amr_fill_fine_list(NodalGeom gc, NodalGeom gf, int off0, int off1, int off2,
                                     const int4* __restrict__ list, int n, const T* __restrict__ pc, T* pf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int4 q = list[t];
    fill_fine_node<T>(gc, gf, off0, off1, off2, pc, pf, q.x, q.y, q.z);
}

// the fine interface nodes (aligned and hanging) as (i, j, k): counted into *count, and listed when list
// is given (in no particular order: every entry is used on its own)
__global__ void k_amr_iface_list(NodalGeom gf, const unsigned char* __restrict__ fcls, int* count, int4* list)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const unsigned char c = fcls[pidx(gf.sy, gf.sz, i, j, k)];
    if (c != F_ALIGNED && c != F_HANGING) return;
    const int t = atomicAdd(count, 1);
    if (list) list[t] = make_int4(i, j, k, 0);
}

// v_c[I] += sum of the interface fine values that map to the coarse interface node I (the aligned
// node with weight 1, hanging nodes 2I + delta with weight 2^-|delta|)
template <typename T>
__global__ void k_amr_sync(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ ccls,
                           const unsigned char* __restrict__ fcls, int off0, int off1, int off2,
                           const T* __restrict__ vf, T* __restrict__ vc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    if (ccls[p] != C_IFACE) return;
    const int off[3] = {off0, off1, off2};
    T acc = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int gpos[3] = {2 * i + dx, 2 * j + dy, 2 * k + dz};
                int m[3];
                if (!fine_local(gf, off, gpos, m)) continue;
                const long long q = pidx(gf.sy, gf.sz, m[0], m[1], m[2]);
                const unsigned char c = fcls[q];
                const int nz = (dx != 0) + (dy != 0) + (dz != 0);
                if ((nz == 0 && c == F_ALIGNED) || (nz > 0 && c == F_HANGING))
                    acc += (nz == 0 ? T(1) : (nz == 1 ? T(0.5) : T(0.25))) * vf[q];
            }
    vc[p] += acc;
}

// zero the entries that are not unknowns (both levels)
__global__ void k_amr_zero_nondof(NodalGeom gc, const unsigned char* __restrict__ ccls, double* __restrict__ vc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    if (c == C_COVERED || c == C_FIXED) vc[p] = 0.0;
}
__global__ void k_amr_zero_nondof_fine(NodalGeom gf, const unsigned char* __restrict__ fcls, double* __restrict__ vf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    if (fcls[p] != F_DOF) vf[p] = 0.0;
}

// composite max norm |v| / V over the unknowns of both levels (per-level node volumes)
__global__ void k_amr_norm_c(NodalGeom gc, const unsigned char* __restrict__ ccls, const double* __restrict__ v,
                             unsigned long long* norm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    unsigned long long key = 0;  // as in k_amr_norm_f
    if (i < gc.nu[0] && j < gc.nu[1] && k < gc.nu[2]) {
        const long long p = pidx(gc.sy, gc.sz, i, j, k);
        const unsigned char c = ccls[p];
        if (c == C_DOF || c == C_IFACE) {
            const int e = (!gc.per[0] && (i == 0 || i == gc.n[0])) + (!gc.per[1] && (j == 0 || j == gc.n[1])) +
                          (!gc.per[2] && (k == 0 || k == gc.n[2]));
            key = e == 0 ? abs_key(v[p]) : abs_key(v[p] * (double)(1 << e));
        }
    }
    key = block_max_key(key);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomic_max_nonneg(norm, key_value(key) * gc.ivol);
}
__global__ void k_amr_norm_f(NodalGeom gf, const unsigned char* __restrict__ fcls, const double* __restrict__ v,
                             unsigned long long* norm)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    // max |v| / node volume as an integer key of |v| 2^e (volume V / 2^e on e non-periodic boundary
    // planes): no FP64 instruction on interior nodes, one multiplication by 1/V per block
    unsigned long long key = 0;
    if (i < gf.nu[0] && j < gf.nu[1] && k < gf.nu[2]) {
        const long long p = pidx(gf.sy, gf.sz, i, j, k);
        if (fcls[p] == F_DOF) {
            const int e = (!gf.per[0] && (i == 0 || i == gf.n[0])) + (!gf.per[1] && (j == 0 || j == gf.n[1])) +
                          (!gf.per[2] && (k == 0 || k == gf.n[2]));
            key = e == 0 ? abs_key(v[p]) : abs_key(v[p] * (double)(1 << e));
        }
    }
    key = block_max_key(key);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomic_max_nonneg(norm, key_value(key) * gf.ivol);
}

// restriction of the composite residual to the whole coarse level: the coarse unknowns' own residual
// plus the trilinear (full-weighting) transpose of the fine unknowns' residuals
// coarse nodes away from the fine region: their own residual only
template <typename T>
__global__ void k_amr_restrict_copy(NodalGeom gc, const unsigned char* __restrict__ ccls, const T* __restrict__ rc,
                                    T* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    store_node(out, gc, i, j, k, (c == C_DOF || c == C_IFACE) ? rc[p] : T(0));
}

// the coarse nodes whose 3 x 3 x 3 fine neighbourhood meets the fine bounding box (origin c0, extent
// ce): own residual plus the fine contributions
template <typename T>
__global__ void k_amr_restrict(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ ccls,
                               const unsigned char* __restrict__ fcls, int off0, int off1, int off2,
                               const T* __restrict__ rc, const T* __restrict__ rf, T* __restrict__ out, int3 c0,
                               int3 ce)
{
    const int ti = blockIdx.x * blockDim.x + threadIdx.x;
    const int tj = blockIdx.y * blockDim.y + threadIdx.y;
    const int tk = blockIdx.z * blockDim.z + threadIdx.z;
    if (ti >= ce.x || tj >= ce.y || tk >= ce.z) return;
    const int i = c0.x + ti, j = c0.y + tj, k = c0.z + tk;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    T acc = (c == C_DOF || c == C_IFACE) ? rc[p] : T(0);
    if (c != C_FIXED) {
        const int off[3] = {off0, off1, off2};
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int gpos[3] = {2 * i + dx, 2 * j + dy, 2 * k + dz};
                    int m[3];
                    if (!fine_local(gf, off, gpos, m)) continue;
                    const long long q = pidx(gf.sy, gf.sz, m[0], m[1], m[2]);
                    if (fcls[q] != F_DOF) continue;
                    const int nz = (dx != 0) + (dy != 0) + (dz != 0);
                    acc += (nz == 0 ? T(1) : (nz == 1 ? T(0.5) : (nz == 2 ? T(0.25) : T(0.125)))) * rf[q];
                }
    }
    store_node(out, gc, i, j, k, acc);
}

// phi_c += e_c on the coarse unknowns; phi_f += (trilinear e_c) on the fine unknowns
template <typename T>
__global__ void k_amr_prolong_c(NodalGeom gc, const unsigned char* __restrict__ ccls, const T* __restrict__ e, T* pc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    if (c == C_DOF || c == C_IFACE) store_node(pc, gc, i, j, k, pc[p] + e[p]);
}
template <typename T>
__global__ void k_amr_prolong_f(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ fcls, int off0, int off1,
                                int off2, const T* __restrict__ e, T* pf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const long long q = pidx(gf.sy, gf.sz, i, j, k);
    if (fcls[q] != F_DOF) return;
    const int gpos[3] = {i + off0, j + off1, k + off2};
    // trilinear weights are 2^-(odd directions) for every coarse node used: sum the values, scale once
    // (FP64 instructions are the bound here)
    int lo[3], hi[3], nodd = 0;
    for (int d = 0; d < 3; ++d) {
        const int odd = gpos[d] & 1;
        nodd += odd;
        lo[d] = cwrap(gc, d, (gpos[d] - odd) / 2);
        hi[d] = odd ? cwrap(gc, d, (gpos[d] - 1) / 2 + 1) : lo[d];
    }
    T acc = 0;
    for (int s = 0; s < 8; ++s) {
        const int sx = s & 1, sy = (s >> 1) & 1, sz = s >> 2;
        if ((sx && !(gpos[0] & 1)) || (sy && !(gpos[1] & 1)) || (sz && !(gpos[2] & 1))) continue;
        acc += e[pidx(gc.sy, gc.sz, sx ? hi[0] : lo[0], sy ? hi[1] : lo[1], sz ? hi[2] : lo[2])];
    }
    const T scale = nodd == 0 ? T(1) : (nodd == 1 ? T(0.5) : (nodd == 2 ? T(0.25) : T(0.125)));
    store_node(pf, gf, i, j, k, fma(scale, acc, pf[q]));
}

// covered coarse nodes take the fine value at their position (output and coarse gradient)
__global__ void k_amr_inject(NodalGeom gc, NodalGeom gf, const unsigned char* __restrict__ ccls, int off0, int off1,
                             int off2, const double* __restrict__ pf, double* pc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    if (ccls[pidx(gc.sy, gc.sz, i, j, k)] != C_COVERED) return;
    const int off[3] = {off0, off1, off2};
    const int gpos[3] = {2 * i, 2 * j, 2 * k};
    int m[3];
    if (!fine_local(gf, off, gpos, m)) return;
    store_node(pc, gc, i, j, k, pf[pidx(gf.sy, gf.sz, m[0], m[1], m[2])]);
}

// sums over the unknowns of v and of the node volumes (consistency of a singular system)
__global__ void k_amr_sums_c(NodalGeom gc, const unsigned char* __restrict__ ccls, const double* __restrict__ v,
                             double* __restrict__ part)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    double a = 0.0, b = 0.0;
    if (i < gc.nu[0] && j < gc.nu[1] && k < gc.nu[2]) {
        const long long p = pidx(gc.sy, gc.sz, i, j, k);
        const unsigned char c = ccls[p];
        if (c == C_DOF || c == C_IFACE) {
            a = v[p];
            b = node_volume(gc, i, j, k);
        }
    }
    a = block_sum_all(a);
    b = block_sum_all(b);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        atomicAdd(part, a);
        atomicAdd(part + 1, b);
        (void)bid;
    }
}
__global__ void k_amr_sums_f(NodalGeom gf, const unsigned char* __restrict__ fcls, const double* __restrict__ v,
                             double* __restrict__ part)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    double a = 0.0, b = 0.0;
    if (i < gf.nu[0] && j < gf.nu[1] && k < gf.nu[2]) {
        const long long p = pidx(gf.sy, gf.sz, i, j, k);
        if (fcls[p] == F_DOF) {
            a = v[p];
            b = node_volume(gf, i, j, k);
        }
    }
    a = block_sum_all(a);
    b = block_sum_all(b);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        atomicAdd(part, a);
        atomicAdd(part + 1, b);
    }
}
// v -= V_node * (sum v / sum V) on the unknowns
__global__ void k_amr_consistent_c(NodalGeom gc, const unsigned char* __restrict__ ccls, const double* __restrict__ part,
                                   double* __restrict__ v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gc.nu[0] || j >= gc.nu[1] || k >= gc.nu[2]) return;
    const long long p = pidx(gc.sy, gc.sz, i, j, k);
    const unsigned char c = ccls[p];
    if (c == C_DOF || c == C_IFACE) v[p] -= node_volume(gc, i, j, k) * (part[0] / part[1]);
}
__global__ void k_amr_consistent_f(NodalGeom gf, const unsigned char* __restrict__ fcls, const double* __restrict__ part,
                                   double* __restrict__ v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    if (fcls[p] == F_DOF) v[p] -= node_volume(gf, i, j, k) * (part[0] / part[1]);
}
// fine phi -= c on the region's nodes (the gauge shift of the coarse level)
__global__ void k_amr_shift_f(NodalGeom gf, const unsigned char* __restrict__ fcls, const double* __restrict__ scal,
                              double* pf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= gf.nu[0] || j >= gf.nu[1] || k >= gf.nu[2]) return;
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    if (fcls[p] != F_OUT && fcls[p] != F_FIXED) store_node(pf, gf, i, j, k, pf[p] - *scal);
}

// dense copy of phi on all bounding-box nodes 0..n (periodic duplicates from the aliases)
__global__ void k_amr_fine_nodes(NodalGeom gf, const double* __restrict__ pf, double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > gf.n[0] || j > gf.n[1] || k > gf.n[2]) return;
    out[i + (long long)(gf.n[0] + 1) * (j + (long long)(gf.n[1] + 1) * k)] = pf[pidx(gf.sy, gf.sz, i, j, k)];
}

inline dim3 g3(int a, int b, int c) { return dim3((a + 31) / 32, (b + 3) / 4, (c + 1) / 2); }
const dim3 kB3(32, 4, 2);
inline dim3 gnodes(const NodalGeom& g) { return g3(g.nu[0], g.nu[1], g.nu[2]); }
inline double bits_to_double(unsigned long long b)
{
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
}

}  // namespace

CompositeNodal::~CompositeNodal()
{
    if (iface) cudaFree(iface);
    if (st) cudaStreamSynchronize(st);
    if (gstep) cudaGraphExecDestroy(gstep);
    if (capst) cudaStreamDestroy(capst);
    if (hnorm) cudaFreeHost(hnorm);
    if (dboxes) cudaFree(dboxes);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    pool.release();
}

size_t CompositeNodal::device_bytes() const
{
    return pool.bytes + crs.device_bytes() + fin.device_bytes() + sizeof(int4) * (size_t)niface;
}

int CompositeNodal::set_options(const gbp_options& o)
{
    int rc = crs.set_options(o);
    if (!rc) rc = fin.set_options(o);
    if (!rc) opt = o;
    if (gstep) cudaGraphExecDestroy(gstep);  // the step's kernels depend on the options
    gstep = nullptr;
    return rc;
}

int CompositeNodal::init(const gbp_geometry& coarse, const int bc_lo[3], const int bc_hi[3], const int* bxs, int nbox,
                         const gbp_options& o, cudaStream_t stream)
{
    opt = o;
    st = stream;
    geom_c = coarse;
    if (nbox < 1 || !bxs) {
        set_error("amr plan: at least one fine box is needed");
        return GBP_BAD_ARG;
    }
    int nd[3];
    bool per[3];
    singular = true;
    for (int d = 0; d < 3; ++d) {
        bclo[d] = bc_lo[d];
        bchi[d] = bc_hi[d];
        nd[d] = 2 * coarse.n_cell[d];
        per[d] = bc_lo[d] == GBP_BC_PERIODIC;
        for (int b : {bc_lo[d], bc_hi[d]}) {
            if (b == GBP_BC_INFLOW || b == GBP_BC_ROBIN) {
                set_error("amr plan: inflow and Robin sides are not supported by the composite solve");
                return GBP_BAD_ARG;
            }
            if (b == GBP_BC_DIRICHLET) singular = false;
        }
    }
    boxes.assign(nbox, AmrBox{});
    int blo[3] = {1 << 30, 1 << 30, 1 << 30}, bhi[3] = {-1, -1, -1};
    for (int b = 0; b < nbox; ++b) {
        for (int d = 0; d < 3; ++d) {
            boxes[b].lo[d] = bxs[6 * b + d];
            boxes[b].hi[d] = bxs[6 * b + 3 + d];
            const int lo = boxes[b].lo[d], hi = boxes[b].hi[d];
            if (lo < 0 || hi >= nd[d] || hi < lo || (lo & 1) || !(hi & 1)) {
                set_error("amr plan: fine boxes must lie in the domain and cover whole coarse cells (even lo, odd hi)");
                return GBP_BAD_ARG;
            }
            blo[d] = std::min(blo[d], lo);
            bhi[d] = std::max(bhi[d], hi);
        }
    }
    // overlap check (disjoint boxes, as in an AMReX BoxArray)
    for (int a = 0; a < nbox; ++a)
        for (int b = a + 1; b < nbox; ++b) {
            bool ov = true;
            for (int d = 0; d < 3; ++d)
                ov = ov && !(boxes[a].hi[d] < boxes[b].lo[d] || boxes[b].hi[d] < boxes[a].lo[d]);
            if (ov) {
                set_error("amr plan: fine boxes overlap");
                return GBP_BAD_ARG;
            }
        }
    // bounding box; in a periodic direction that it touches at either end it spans the whole domain
    // (the region may then continue across the periodic seam)
    int fbclo[3], fbchi[3];
    for (int d = 0; d < 3; ++d) {
        if (per[d] && (blo[d] == 0 || bhi[d] == nd[d] - 1)) {
            blo[d] = 0;
            bhi[d] = nd[d] - 1;
        }
        off[d] = blo[d];
        nfb[d] = bhi[d] - blo[d] + 1;
        if (per[d] && nfb[d] == nd[d]) {
            fbclo[d] = fbchi[d] = GBP_BC_PERIODIC;
        } else {
            fbclo[d] = (blo[d] == 0) ? (per[d] ? GBP_BC_NEUMANN : bc_lo[d]) : GBP_BC_NEUMANN;
            fbchi[d] = (bhi[d] == nd[d] - 1) ? (per[d] ? GBP_BC_NEUMANN : bc_hi[d]) : GBP_BC_NEUMANN;
        }
    }
    gbp_geometry gfine{};
    for (int d = 0; d < 3; ++d) {
        const double hf = (coarse.prob_hi[d] - coarse.prob_lo[d]) / nd[d];
        gfine.n_cell[d] = nfb[d];
        gfine.prob_lo[d] = coarse.prob_lo[d] + off[d] * hf;
        gfine.prob_hi[d] = gfine.prob_lo[d] + nfb[d] * hf;
    }
    int rc = crs.init(coarse, bc_lo, bc_hi, o, stream);
    if (rc) return rc;
    rc = fin.init(gfine, fbclo, fbchi, o, stream);
    if (rc) return rc;
    gc = crs.geom0();
    gf = fin.geom0();
    gf_nomask = gf;
    gf_nomask.mask = nullptr;
    // device storage
    size_t need = 0;
    auto add = [&](size_t cnt, size_t sz) { need = ((need + 255) & ~size_t(255)) + cnt * sz; };
    const size_t ncf = (size_t)nfb[0] * nfb[1] * nfb[2];
    const size_t nnf = (size_t)(nfb[0] + 1) * (nfb[1] + 1) * (nfb[2] + 1);
    add(gc.count, 1);
    add(gf.count, 1);
    add(gc.count, 1);
    add(gf.count, 1);
    for (int q = 0; q < 7; ++q) add(gc.count, 8);  // sc_m, sc_t, phi_c, b_c, r_c, rc_full, e_c
    for (int q = 0; q < 3; ++q) add(gf.count, 8);  // phi_f, b_f, r_f
    for (int q = 0; q < 5; ++q) add(gc.count, 4);  // bc32, rc32, ec32, rcf32, scm32
    for (int q = 0; q < 3; ++q) add(gf.count, 4);  // bf32, rf32, ef32
    xfer1 = fin.num_levels() >= 2;
    if (xfer1) {
        g1n = fin.level(1).g;
        g1n.mask = nullptr;
        for (int d = 0; d < 3; ++d)
            if (g1n.n[d] * 2 != gf.n[d] || g1n.per[d] != gf.per[d] || (off[d] & 1)) xfer1 = false;
    }
    if (xfer1) {
        add(gf.count, 4);   // rm32
        add(g1n.count, 4);  // x1_32
    }
    add(3 * ncf, 8);                               // vel_f
    add(3 * ncf, 8);                               // gp_f
    add(ncf, 8);                                   // rho_f
    add(3 * ncf, 8);                               // velo_f
    add(ncf, 8);                                   // sig_f
    add(nnf, 8);                                   // p_fb
    // the shared-sum FP64 residual on both levels (isotropic cells): four edge-weight arrays each
    qsw = qsweep_supported(gf_nomask) && qsweep_supported(gc);
    if (qsw) {
        for (int q = 0; q < 4; ++q) add(gf.count, 8);
        for (int q = 0; q < 4; ++q) add(gc.count, 8);
    }
    nparts = std::max(nodal_partials_needed(gc), 1184);
    add(nparts + 64, 8);
    add(8, 8);
    add(8, 8);
    add(8, 4);  // derr
    need += 4096;
    rc = pool.reserve(need);
    if (rc) return rc;
    cmask_c = pool.take<unsigned char>(gc.count);
    cmask_f = pool.take<unsigned char>(gf.count);
    ccls = pool.take<unsigned char>(gc.count);
    fcls = pool.take<unsigned char>(gf.count);
    if (qsw) {
        double** wf[4] = {&qwf.wsum, &qwf.wx, &qwf.wy, &qwf.wz};
        double** wc[4] = {&qwc.wsum, &qwc.wx, &qwc.wy, &qwc.wz};
        for (int q = 0; q < 4; ++q) *wf[q] = pool.take<double>(gf.count);
        for (int q = 0; q < 4; ++q) *wc[q] = pool.take<double>(gc.count);
    }
    sc_m = pool.take<double>(gc.count);
    sc_t = pool.take<double>(gc.count);
    phi_c = pool.take<double>(gc.count);
    b_c = pool.take<double>(gc.count);
    r_c = pool.take<double>(gc.count);
    rc_full = pool.take<double>(gc.count);
    e_c = pool.take<double>(gc.count);
    phi_f = pool.take<double>(gf.count);
    b_f = pool.take<double>(gf.count);
    r_f = pool.take<double>(gf.count);
    bc32 = pool.take<float>(gc.count);
    rc32 = pool.take<float>(gc.count);
    ec32 = pool.take<float>(gc.count);
    rcf32 = pool.take<float>(gc.count);
    scm32 = pool.take<float>(gc.count);
    bf32 = pool.take<float>(gf.count);
    rf32 = pool.take<float>(gf.count);
    ef32 = pool.take<float>(gf.count);
    if (xfer1) {
        rm32 = pool.take<float>(gf.count);
        x1_32 = pool.take<float>(g1n.count);
    }
    vel_f = pool.take<double>(3 * ncf);
    gp_f = pool.take<double>(3 * ncf);
    rho_f = pool.take<double>(ncf);
    velo_f = pool.take<double>(3 * ncf);
    sig_f = pool.take<double>(ncf);
    p_fb = pool.take<double>(nnf);
    part = pool.take<double>(nparts + 64);
    scal = pool.take<double>(8);
    dnorm = pool.take<unsigned long long>(8);
    derr = pool.take<unsigned>(8);
    GBP_CUDA(cudaMemsetAsync(derr, 0, 8 * sizeof(unsigned), st));
    GBP_CUDA(cudaMallocHost(&hnorm, 8 * sizeof(unsigned long long)));
    GBP_CUDA(cudaEventCreate(&ev0));
    GBP_CUDA(cudaEventCreate(&ev1));
    dboxes_bytes = sizeof(BoxEntry) * (size_t)nbox;
    GBP_CUDA(cudaMalloc(&dboxes, dboxes_bytes));
    // masks and classes
    std::vector<BoxEntry> tab(nbox);
    for (int b = 0; b < nbox; ++b) {
        memset(&tab[b], 0, sizeof(BoxEntry));
        for (int d = 0; d < 3; ++d) {
            tab[b].lo[d] = boxes[b].lo[d];
            tab[b].hi[d] = boxes[b].hi[d];
        }
    }
    GBP_CUDA(cudaMemcpyAsync(dboxes, tab.data(), dboxes_bytes, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemsetAsync(cmask_f, 0, gf.count, st));
    GBP_CUDA(cudaMemsetAsync(cmask_c, 0, gc.count, st));
    GBP_CUDA(cudaMemsetAsync(fcls, 0, gf.count, st));
    GBP_CUDA(cudaMemsetAsync(ccls, C_FIXED, gc.count, st));
    k_amr_cmask_fine<<<dim3(64, nbox), kT, 0, st>>>(gf, (const BoxEntry*)dboxes, off[0], off[1], off[2], cmask_f);
    k_amr_cmask_coarse<<<g3(gc.n[0], gc.n[1], gc.n[2]), kB3, 0, st>>>(gc, gf, cmask_f, off[0], off[1], off[2], cmask_c);
    k_amr_classify_fine<<<gnodes(gf), kB3, 0, st>>>(gf, cmask_f, off[0], off[1], off[2], nd[0], nd[1], nd[2], per[0],
                                                  per[1], per[2], fcls);
    k_amr_classify_coarse<<<gnodes(gc), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], ccls);
    GBP_CUDA(cudaGetLastError());
    // the fine solver's overset mask: the fine unknowns
    int* im = nullptr;
    GBP_CUDA(cudaMalloc(&im, sizeof(int) * nnf));
    k_amr_fine_mask<<<g3(gf.n[0] + 1, gf.n[1] + 1, gf.n[2] + 1), kB3, 0, st>>>(gf, fcls, im);
    gbp_iarray4 ma{};
    ma.data = im;
    for (int d = 0; d < 3; ++d) ma.hi[d] = nfb[d];
    ma.jstride = nfb[0] + 1;
    ma.kstride = (long long)(nfb[0] + 1) * (nfb[1] + 1);
    rc = fin.set_mask(&ma);
    cudaStreamSynchronize(st);
    cudaFree(im);
    if (rc) return rc;
    gf = fin.geom0();  // now carries the mask
    // the interface node list: count, then fill
    {
        int* dcount = reinterpret_cast<int*>(dnorm + 4);
        GBP_CUDA(cudaMemsetAsync(dcount, 0, sizeof(int), st));
        k_amr_iface_list<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, dcount, nullptr);
        GBP_CUDA(cudaMemcpyAsync(&niface, dcount, sizeof(int), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        if (niface > 0) {
            GBP_CUDA(cudaMalloc(&iface, sizeof(int4) * (size_t)niface));
            GBP_CUDA(cudaMemsetAsync(dcount, 0, sizeof(int), st));
            k_amr_iface_list<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, dcount, iface);
            GBP_CUDA(cudaStreamSynchronize(st));
        }
        GBP_CUDA(cudaGetLastError());
    }
    return GBP_OK;
}

int CompositeNodal::check_fields(const AmrFields& f)
{
    if (!f.vel_c || !f.vel_f || !f.gp_c || !f.gp_f) {
        set_error("amr project: velocity and gp are required on both levels");
        return GBP_BAD_ARG;
    }
    for (size_t b = 0; b < boxes.size(); ++b) {
        if (!f.vel_f[b] || !f.vel_f[b]->data || !f.gp_f[b] || !f.gp_f[b]->data) {
            set_error("amr project: every fine box needs its velocity and gp");
            return GBP_BAD_ARG;
        }
        const gbp_array4* arr[4] = {f.vel_f[b], f.gp_f[b], f.rho_f ? f.rho_f[b] : nullptr,
                                    f.vel_old_f ? f.vel_old_f[b] : nullptr};
        for (const gbp_array4* a : arr) {
            if (!a || !a->data) continue;
            for (int d = 0; d < 3; ++d)
                if (a->lo[d] > boxes[b].lo[d] || a->hi[d] < boxes[b].hi[d]) {
                    set_error("amr project: a fine array does not cover its box");
                    return GBP_BAD_ARG;
                }
        }
        if (f.p_f && f.p_f[b] && f.p_f[b]->data)
            for (int d = 0; d < 3; ++d)
                if (f.p_f[b]->lo[d] > boxes[b].lo[d] || f.p_f[b]->hi[d] < boxes[b].hi[d] + 1) {
                    set_error("amr project: a fine p_nd array does not cover its box's nodes");
                    return GBP_BAD_ARG;
                }
    }
    return GBP_OK;
}

// FP64 residuals of the composite operator's two parts (fine bounding box without the overset mask,
// coarse level with covered cells' sigma zeroed): the shared-sum form when the cells are isotropic
void CompositeNodal::resid_f(const double* x, const double* b, double* r)
{
    if (qsw)
        nodal_qsweep64(gf_nomask, 1, fin.sigma64(), qwf, x, b, r, 1.0, nullptr, st);
    else
        nodal_resid<double>(gf_nomask, fin.sigma64(), x, b, r, nullptr, st);
}
void CompositeNodal::resid_c(const double* x, const double* b, double* r)
{
    if (qsw)
        nodal_qsweep64(gc, 1, sc_m, qwc, x, b, r, 1.0, nullptr, st);
    else
        nodal_resid<double>(gc, sc_m, x, b, r, nullptr, st);
}

// v_c (coarse interface nodes) += the restricted interface values of v_f
void CompositeNodal::sync(double* vc, const double* vf)
{
    k_amr_sync<<<gnodes(gc), kB3, 0, st>>>(gc, gf, ccls, fcls, off[0], off[1], off[2], vf, vc);
}

// r = b - A phi on both levels (fine interface values filled first), with the fine interface
// residuals restricted into the coarse interface nodes; norm (if given) = composite max norm
void CompositeNodal::composite_residual(const double* bc, const double* bf, unsigned long long* norm)
{
    k_amr_fill_fine<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], phi_c, phi_f);
    resid_f(phi_f, bf, r_f);
    resid_c(phi_c, bc, r_c);
    sync(r_c, r_f);
    if (norm) {
        k_amr_norm_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, r_c, norm);
        k_amr_norm_f<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, r_f, norm);
    }
}

// out (whole coarse level) = the coarse unknowns' composite residual rc plus the full-weighting transpose
// of the fine unknowns' residual rf
template <typename T>
void CompositeNodal::restrict_to_coarse(const T* rc, const T* rf, T* out)
{
    k_amr_restrict_copy<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, rc, out);
    int lo[3], ext[3];
    for (int d = 0; d < 3; ++d) {
        // fine global node positions 2i-1 .. 2i+1 against the box's off .. off + nfb
        lo[d] = std::max(0, (off[d] - 1) / 2);
        const int hi = std::min(gc.nu[d] - 1, (off[d] + nfb[d] + 1) / 2 + 1);
        if (gf.per[d]) {
            lo[d] = 0;
            ext[d] = gc.nu[d];
        } else {
            ext[d] = std::max(0, hi - lo[d] + 1);
        }
    }
    if (ext[0] > 0 && ext[1] > 0 && ext[2] > 0) {
        const dim3 grid((unsigned)((ext[0] + kB3.x - 1) / kB3.x), (unsigned)((ext[1] + kB3.y - 1) / kB3.y),
                        (unsigned)((ext[2] + kB3.z - 1) / kB3.z));
        k_amr_restrict<<<grid, kB3, 0, st>>>(gc, gf, ccls, fcls, off[0], off[1], off[2], rc, rf, out,
                                             make_int3(lo[0], lo[1], lo[2]), make_int3(ext[0], ext[1], ext[2]));
    }
}

// One refinement step on st (plain FP64 form): coarse correction on the restricted composite residual,
// fine correction on the fresh fine residual with the interface held, then the composite residual and
// its norm (read back into hnorm[1]).
void CompositeNodal::issue_step(double scale32)
{
    const int m = 1;  // V-cycles per level per step (one is the fastest on the benchmark's workload)
    restrict_to_coarse(r_c, r_f, rc_full);
    cudaMemsetAsync(e_c, 0, sizeof(double) * gc.count, st);
    crs.apply_vcycles(rc_full, e_c, m, scale32, st);
    k_amr_prolong_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, e_c, phi_c);
    k_amr_prolong_f<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], e_c, phi_f);
    // fine correction on the fresh fine residual, interface held
    k_amr_fill_fine<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], phi_c, phi_f);
    resid_f(phi_f, b_f, r_f);
    fin.apply_vcycles(r_f, phi_f, m, scale32, st);
    // composite residual and its norm
    cudaMemsetAsync(dnorm + 1, 0, sizeof(unsigned long long), st);
    composite_residual(b_c, b_f, dnorm + 1);
    cudaMemcpyAsync(hnorm + 1, dnorm + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
}

// launch errors and bounded-wait time-outs of the level sweeps issued by a step (both solvers' and this
// object's own); the error words are cleared
int CompositeNodal::sweep_status()
{
    int rc = launch_rc;
    launch_rc = 0;
    for (NodalSolver* sv : {&crs, &fin}) {
        const int r = sv->take_sweep_status(st);
        if (!rc) rc = r;
    }
    unsigned herr = 0;
    GBP_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        GBP_CUDA(cudaMemsetAsync(derr, 0, sizeof(unsigned), st));
        if (!rc) {
            set_error("amr solve: a bounded device wait (TMA pipeline) ran out");
            rc = GBP_TIMEOUT;
        }
    }
    return rc;
}

void CompositeNodal::resid32(const NodalGeom& g, const float* s, const float* x, const float* b, float* r)
{
    if (vsweep32_supported(g)) {
        const int rc = vsweep32(g, 1, s, x, b, r, 0.f, derr, st);
        if (rc && !launch_rc) launch_rc = rc;
    } else {
        nodal_resid<float>(g, s, x, b, r, nullptr, st);
    }
}

// One refinement step of the mixed form: the FP64 composite residual (r_c, r_f), scaled into FP32, is the
// right-hand side of the correction equation A e = r, which kInner two-level steps solve in FP32
// arithmetic (the same steps as issue_step on e, with FP32 composite residuals between them); then
// phi += e / scale on both levels in FP64 and the FP64 composite residual with its norm.
void CompositeNodal::issue_outer32(double scale32)
{
    const unsigned ncb = (unsigned)((gc.count + kT - 1) / kT), nfb_ = (unsigned)((gf.count + kT - 1) / kT);
    k_amr_to32<<<ncb, kT, 0, st>>>(gc.count, r_c, scale32, bc32);
    k_amr_rhs32_fine<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, r_f, scale32, bf32);
    cudaMemsetAsync(ec32, 0, sizeof(float) * gc.count, st);
    cudaMemsetAsync(ef32, 0, sizeof(float) * gf.count, st);
    // FP32 composite residual of e into rc32 / rf32 (fine unknowns) and rm32 (fine interface nodes)
    auto composite32 = [&]() {
        resid32(gf, fin.sigma32(), ef32, bf32, rf32);
        nodal_resid_list<float>(gf_nomask, fin.sigma32(), ef32, bf32, rm32, (const int4*)iface, niface, st);
        resid32(gc, scm32, ec32, bc32, rc32);
        k_amr_sync<<<gnodes(gc), kB3, 0, st>>>(gc, gf, ccls, fcls, off[0], off[1], off[2], (const float*)rm32, rc32);
    };
    for (int q = 0; q < kInner; ++q) {
        const float* rc = q == 0 ? bc32 : rc32;
        const float* rf = q == 0 ? bf32 : rf32;
        const int o0 = off[0] / 2, o1 = off[1] / 2, o2 = off[2] / 2;
        if (xfer1) {
            // rf holds the fine unknowns' residuals and 0 elsewhere (bf32, or the masked fine residual)
            nodal_restrict<float>(gf_nomask, g1n, rf, x1_32, st);
            k_amr_combine<<<gnodes(gc), kB3, 0, st>>>(gc, g1n, ccls, o0, o1, o2, rc, x1_32, rcf32);
        } else {
            restrict_to_coarse(rc, rf, rcf32);
        }
        crs.apply_vcycles32(rcf32, 1, st);
        k_amr_prolong_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, crs.correction32(), ec32);
        if (xfer1) {
            k_amr_gather_g1<<<gnodes(g1n), kB3, 0, st>>>(gc, g1n, o0, o1, o2, crs.correction32(), x1_32);
            nodal_prolong_add<float>(gf, g1n, x1_32, ef32, st);
        } else {
            k_amr_prolong_f<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], crs.correction32(),
                                                        ef32);
        }
        if (xfer1) {
            if (niface > 0)
                k_amr_fill_fine_list<<<(unsigned)((niface + kT - 1) / kT), kT, 0, st>>>(
                    gc, gf, off[0], off[1], off[2], (const int4*)iface, niface, (const float*)ec32, ef32);
            resid32(gf, fin.sigma32(), ef32, bf32, rf32);  // the fine unknowns only (the mask holds the rest)
        } else {
            k_amr_fill_fine<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], (const float*)ec32,
                                                        ef32);
            resid32(gf_nomask, fin.sigma32(), ef32, bf32, rf32);
        }
        if (kFineSweeps > 0)
            fin.smooth32(rf32, kFineSweeps, st);
        else
            fin.apply_vcycles32(rf32, 1, st);
        k_amr_add32<<<nfb_, kT, 0, st>>>(gf.count, fin.correction32(), ef32);
        if (q + 1 < kInner) {
            // FP32 composite residual of e (the interface values of e_f are those of e_c already)
            if (xfer1) {
                // the fine unknowns' residuals, and the interface nodes' into rm32 for the coarse interface
                composite32();
            } else {
                resid32(gf_nomask, fin.sigma32(), ef32, bf32, rf32);
                resid32(gc, scm32, ec32, bc32, rc32);
                k_amr_sync<<<gnodes(gc), kB3, 0, st>>>(gc, gf, ccls, fcls, off[0], off[1], off[2], (const float*)rf32,
                                                       rc32);
            }
        }
    }
    nodal_add_correction<float>(gc, phi_c, ec32, 1.0 / scale32, st);
    nodal_add_correction<float>(gf_nomask, phi_f, ef32, 1.0 / scale32, st);
    cudaMemsetAsync(dnorm + 1, 0, sizeof(unsigned long long), st);
    composite_residual(b_c, b_f, dnorm + 1);
    cudaMemcpyAsync(hnorm + 1, dnorm + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
}

int CompositeNodal::project(const AmrFields& f, gbp_stats* stats)
{
    int rc = check_fields(f);
    if (rc) return rc;
    const int nbox = (int)boxes.size();
    const size_t ncf = (size_t)nfb[0] * nfb[1] * nfb[2];
    GBP_CUDA(cudaEventRecord(ev0, st));
    // fine inputs into the bounding box (cells outside the fine boxes: zero)
    std::vector<BoxEntry> tab(nbox);
    auto gather = [&](const gbp_array4* const* arr, int ncomp, double* dst) -> int {
        GBP_CUDA(cudaMemsetAsync(dst, 0, sizeof(double) * ncomp * ncf, st));
        if (!arr) return GBP_OK;
        for (int b = 0; b < nbox; ++b) {
            memset(&tab[b], 0, sizeof(BoxEntry));
            for (int d = 0; d < 3; ++d) {
                tab[b].lo[d] = boxes[b].lo[d];
                tab[b].hi[d] = boxes[b].hi[d];
            }
            if (arr[b]) tab[b].a = *arr[b];
        }
        GBP_CUDA(cudaMemcpyAsync(dboxes, tab.data(), dboxes_bytes, cudaMemcpyHostToDevice, st));
        k_amr_gather<<<dim3(64, nbox), kT, 0, st>>>((const BoxEntry*)dboxes, off[0], off[1], off[2], nfb[0], nfb[1],
                                                    nfb[2], ncomp, dst);
        // the table is reused by the next gather: let this one finish reading it
        GBP_CUDA(cudaStreamSynchronize(st));
        return GBP_OK;
    };
    if ((rc = gather((const gbp_array4* const*)f.vel_f, 3, vel_f))) return rc;
    if ((rc = gather((const gbp_array4* const*)f.gp_f, 3, gp_f))) return rc;
    if ((rc = gather(f.rho_f, 1, rho_f))) return rc;
    if ((rc = gather(f.vel_old_f, 3, velo_f))) return rc;
    // sigma on both levels (coarse: whole level for the V-cycles, covered cells zeroed for the
    // composite operator; fine: zero outside the fine cells)
    k_amr_sigma_fine<<<g3(nfb[0], nfb[1], nfb[2]), kB3, 0, st>>>(gf, cmask_f, rho_f, f.rho_f != nullptr, f.scale,
                                                                 f.rho0, sig_f);
    {
        gbp_array4 rc_a{};
        if (f.rho_c) rc_a = *f.rho_c;
        k_amr_sigma_coarse<<<g3(gc.n[0], gc.n[1], gc.n[2]), kB3, 0, st>>>(gc, cmask_c, rc_a, f.rho_c != nullptr,
                                                                          f.scale, f.rho0, sig_f, off[0], off[1],
                                                                          off[2], nfb[0], nfb[1], rc_full);
        gbp_array4 ca{};
        ca.data = rc_full;  // scratch until the solve starts
        for (int d = 0; d < 3; ++d) ca.hi[d] = gc.n[d] - 1;
        ca.ncomp = 1;
        ca.jstride = gc.n[0];
        ca.kstride = (long long)gc.n[0] * gc.n[1];
        ca.nstride = (long long)gc.n[0] * gc.n[1] * gc.n[2];
        rc = crs.set_sigma(&ca, 0.0);
        if (rc) return rc;
    }
    // s / rho on every coarse cell: the gp add-back and the velocity correction of the coarse level;
    // covered cells zeroed: the coarse part of the composite operator
    GBP_CUDA(cudaMemsetAsync(sc_t, 0, sizeof(double) * gc.count, st));
    nodal_sigma_from_rho(gc, f.rho_c, f.scale, f.rho0, sc_t, nullptr, st);
    k_amr_mask_sigma<<<(unsigned)((gc.count + kT - 1) / kT), kT, 0, st>>>(gc.count, sc_t, cmask_c, sc_m);
    k_amr_to32<<<(unsigned)((gc.count + kT - 1) / kT), kT, 0, st>>>(gc.count, sc_m, 1.0, scm32);
    gbp_array4 sa{};
    sa.data = sig_f;
    for (int d = 0; d < 3; ++d) sa.hi[d] = nfb[d] - 1;
    sa.ncomp = 1;
    sa.jstride = nfb[0];
    sa.kstride = (long long)nfb[0] * nfb[1];
    sa.nstride = (long long)ncf;
    rc = fin.set_sigma(&sa, 0.0);
    if (rc) return rc;
    if (qsw) {
        nodal_qweights64(gf_nomask, fin.sigma64(), qwf, st);
        nodal_qweights64(gc, sc_m, qwc, st);
    }
    // right-hand sides: leaf cells of each level, then the fine interface into the coarse interface
    const bool sub_old = f.incremental && f.vel_old_c;
    auto cellsf = [&](double* d, int nc_) {
        gbp_array4 a{};
        a.data = d;
        for (int q = 0; q < 3; ++q) a.hi[q] = nfb[q] - 1;
        a.ncomp = nc_;
        a.jstride = nfb[0];
        a.kstride = (long long)nfb[0] * nfb[1];
        a.nstride = (long long)ncf;
        return a;
    };
    RhsArgs rac{}, raf{};
    for (int d = 0; d < 3; ++d) {
        const double hc[3] = {gc.h[0], gc.h[1], gc.h[2]};
        const int e = d == 0 ? 1 : 0, q = d == 2 ? 1 : 2;
        rac.cf[d] = hc[e] * hc[q] / 4.0;
        raf.cf[d] = gf.h[e] * gf.h[q] / 4.0;
    }
    rac.vel = *f.vel_c;
    rac.gp = *f.gp_c;
    rac.add_gp = !f.incremental;
    rac.sub_old = sub_old;
    if (sub_old) rac.vel_old = *f.vel_old_c;
    rac.cmask = cmask_c;
    raf.vel = cellsf(vel_f, 3);
    raf.gp = cellsf(gp_f, 3);
    raf.add_gp = !f.incremental;
    raf.sub_old = sub_old;
    if (sub_old) raf.vel_old = cellsf(velo_f, 3);
    raf.cmask = cmask_f;
    nodal_rhs(gc, rac, sc_t, b_c, nullptr, st);
    nodal_rhs(gf_nomask, raf, fin.sigma64(), b_f, nullptr, st);
    sync(b_c, b_f);
    k_amr_zero_nondof<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, b_c);
    k_amr_zero_nondof_fine<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, b_f);
    if (singular) {
        GBP_CUDA(cudaMemsetAsync(part, 0, 2 * sizeof(double), st));
        k_amr_sums_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, b_c, part);
        k_amr_sums_f<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, b_f, part);
        k_amr_consistent_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, part, b_c);
        k_amr_consistent_f<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, part, b_f);
    }
    GBP_CUDA(cudaMemsetAsync(dnorm, 0, 2 * sizeof(unsigned long long), st));
    k_amr_norm_c<<<gnodes(gc), kB3, 0, st>>>(gc, ccls, b_c, dnorm);
    k_amr_norm_f<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, b_f, dnorm);
    // initial_guess = previous: both levels start from the last converged composite phi of this box layout
    // (phi_c / phi_f keep it between calls); the tolerance refers to that start's residual, as in the
    // single-level solve
    const bool from_prev = opt.initial_guess == 1 && have_last;
    have_last = false;
    if (!from_prev) {
        GBP_CUDA(cudaMemsetAsync(phi_c, 0, sizeof(double) * gc.count, st));
        GBP_CUDA(cudaMemsetAsync(phi_f, 0, sizeof(double) * gf.count, st));
    }
    composite_residual(b_c, b_f, dnorm + 1);
    GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    GBP_CUDA(cudaGetLastError());
    const double bnorm = bits_to_double(hnorm[0]);
    double rn = bits_to_double(hnorm[1]);
    if (!isfinite(bnorm) || !isfinite(rn)) {
        set_error("amr solve: right-hand side is not finite");
        return GBP_NAN;
    }
    const double target = std::max(opt.rtol * (opt.always_use_bnorm ? bnorm : rn), opt.atol);
    double scale32 = 1.0;
    if (bnorm > 0.0) {
        int ex = 0;
        frexp(bnorm * gc.vol, &ex);
        scale32 = ldexp(1.0, -ex);
    }
    int it = 0, status = GBP_OK;
    const double r0 = rn;
    const bool mixed = opt.precision == GBP_PREC_MIXED;
    auto issue = [&](double sc) {
        if (mixed)
            issue_outer32(sc);
        else
            issue_step(sc);
    };
    while (rn > target) {
        if (it >= opt.maxiter) {
            status = GBP_NOT_CONVERGED;
            set_error("amr solve: maxiter reached before the tolerance");
            break;
        }
        if (opt.use_graphs && (!gstep || gstep_scale != scale32 || gstep_prec != opt.precision)) {
            // capture the step once on a stream of its own (the caller's may be the legacy default
            // stream), with every kernel of the step issued there
            if (gstep) cudaGraphExecDestroy(gstep);
            gstep = nullptr;
            if (!capst) GBP_CUDA(cudaStreamCreateWithFlags(&capst, cudaStreamNonBlocking));
            cudaStream_t keep = st;
            st = capst;
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(capst, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                issue(scale32);
                e = cudaStreamEndCapture(capst, &graph);
            }
            st = keep;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&gstep, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                gstep = nullptr;
                return cuda_fail(e, "amr: capture of the refinement step");
            }
            gstep_scale = scale32;
            gstep_prec = opt.precision;
        }
        if (opt.use_graphs)
            GBP_CUDA(cudaGraphLaunch(gstep, st));
        else
            issue(scale32);
        GBP_CUDA(cudaStreamSynchronize(st));
        GBP_CUDA(cudaGetLastError());
        if ((rc = sweep_status())) return rc;
        rn = bits_to_double(hnorm[1]);
        ++it;
        if (opt.verbose > 1) fprintf(stderr, "gbp amr: iter %d rel resid %.3e\n", it, bnorm > 0 ? rn / bnorm : rn);
        if (!isfinite(rn)) {
            status = GBP_NAN;
            set_error("amr solve: residual became NaN/Inf");
            break;
        }
    }
    // outputs: interface values, covered coarse nodes from the fine level, gauge of a singular system
    k_amr_fill_fine<<<gnodes(gf), kB3, 0, st>>>(gc, gf, fcls, off[0], off[1], off[2], phi_c, phi_f);
    k_amr_inject<<<gnodes(gc), kB3, 0, st>>>(gc, gf, ccls, off[0], off[1], off[2], phi_f, phi_c);
    if (singular) {
        nodal_remove_mean(gc, phi_c, part, scal, 1, 0, 0, nullptr, st);
        k_amr_shift_f<<<gnodes(gf), kB3, 0, st>>>(gf, fcls, scal, phi_f);
    }
    // corrections per level
    CorrArgs cac{}, caf{};
    for (int d = 0; d < 3; ++d) {
        cac.inv4h[d] = 1.0 / (4.0 * gc.h[d]);
        caf.inv4h[d] = 1.0 / (4.0 * gf.h[d]);
    }
    cac.vel = *f.vel_c;
    cac.gp = *f.gp_c;
    cac.add_gp = !f.incremental;
    cac.incremental = f.incremental;
    caf.vel = cellsf(vel_f, 3);
    caf.gp = cellsf(gp_f, 3);
    caf.add_gp = !f.incremental;
    caf.incremental = f.incremental;
    if (f.p_c && f.p_c->data) nodal_store_phi(gc, *f.p_c, phi_c, f.incremental, st);
    nodal_correct(gc, cac, sc_t, phi_c, st);
    nodal_correct(gf_nomask, caf, fin.sigma64(), phi_f, st);
    k_amr_fine_nodes<<<g3(nfb[0] + 1, nfb[1] + 1, nfb[2] + 1), kB3, 0, st>>>(gf, phi_f, p_fb);
    // fine outputs back into the boxes
    auto scatter = [&](gbp_array4* const* arr, int ncomp, const double* src, bool nodes) -> int {
        if (!arr) return GBP_OK;
        for (int b = 0; b < nbox; ++b) {
            memset(&tab[b], 0, sizeof(BoxEntry));
            for (int d = 0; d < 3; ++d) {
                tab[b].lo[d] = boxes[b].lo[d];
                tab[b].hi[d] = boxes[b].hi[d];
            }
            if (arr[b]) tab[b].a = *arr[b];
        }
        GBP_CUDA(cudaMemcpyAsync(dboxes, tab.data(), dboxes_bytes, cudaMemcpyHostToDevice, st));
        if (nodes)
            k_amr_scatter_nodes<<<dim3(64, nbox), kT, 0, st>>>((const BoxEntry*)dboxes, off[0], off[1], off[2], nfb[0],
                                                               nfb[1], src, f.incremental);
        else
            k_amr_scatter<<<dim3(64, nbox), kT, 0, st>>>((const BoxEntry*)dboxes, off[0], off[1], off[2], nfb[0], nfb[1],
                                                         nfb[2], ncomp, src);
        GBP_CUDA(cudaStreamSynchronize(st));
        return GBP_OK;
    };
    if ((rc = scatter(f.vel_f, 3, vel_f, false))) return rc;
    if ((rc = scatter(f.gp_f, 3, gp_f, false))) return rc;
    if ((rc = scatter(f.p_f, 1, p_fb, true))) return rc;
    GBP_CUDA(cudaEventRecord(ev1, st));
    GBP_CUDA(cudaEventSynchronize(ev1));
    GBP_CUDA(cudaGetLastError());
    have_last = status == GBP_OK;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->status = status;
        stats->outer_iters = it + 1;
        stats->prev_rel_resid = from_prev ? (bnorm > 0 ? r0 / bnorm : r0) : 0.0;
        // V-cycles: the coarse one of every two-level step, and the fine one where the fine correction is a
        // V-cycle (the plain form; the mixed form with kFineSweeps = 0)
        stats->vcycles = it * (mixed ? kInner * (kFineSweeps > 0 ? 1 : 2) : 2);
        stats->num_levels = 2;
        stats->rhs_norm = bnorm;
        stats->initial_rel_resid = bnorm > 0 ? r0 / bnorm : r0;
        stats->final_rel_resid = bnorm > 0 ? rn / bnorm : rn;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        stats->ms_total = ms;
    }
    return status;
}

}  // namespace gbp
