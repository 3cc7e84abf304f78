// Cut cells (embedded boundary) in the nodal projection, finest level. Regular cells keep the
// 27-point kernels of the level (their sigma is zeroed on cut and covered cells); each cut cell carries
// its exact Q1 element matrix over the fluid part (from the cell's second moments, built on the host
// once per geometry) in a table. Nodes that touch a cut cell ("EB nodes", about 1 % of the nodes around
// a body) are recomputed by the node-centric kernels below after the level kernel has run, from the
// same input, so the level kernel's output there is simply overwritten:
//   k_eb_node<MODE>   Jacobi update (MODE 0) or residual (MODE 1) of the EB nodes over their 8 cells
//   k_eb_rhs          the cut cells' int u . grad N added to the right-hand side of the EB nodes
//   k_eb_correct      u -= sigma grad phi at the fluid centroid of every cut cell, gp / grad phi out
#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "nodal_eb.h"

namespace gbp {

namespace {

__device__ __forceinline__ double* at4(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
           (long long)n * a.nstride;
}

// padded offset of corner b of a cell from the cell's low corner
__device__ __forceinline__ long long corner_off(const NodalGeom& g, int b)
{
    return (long long)(b & 1) + ((b >> 1) & 1) * g.sy + ((b >> 2) & 1) * g.sz;
}

template <typename T>
__device__ __forceinline__ const T* sig_true(const EbNodal& e);
template <>
__device__ __forceinline__ const double* sig_true<double>(const EbNodal& e) { return e.sig64; }
template <>
__device__ __forceinline__ const float* sig_true<float>(const EbNodal& e) { return e.sig32; }

template <typename T, int MODE>
__global__ void __launch_bounds__(128) k_eb_node(NodalGeom g, EbNodal e, const T* __restrict__ x, const T* __restrict__ b,
                                                 T* out, T omega)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= e.nnodes) return;
    const EbNodeEntry nd = e.nodes[t];
    T v = T(0);
    if (!node_is_dirichlet(g, nd.i, nd.j, nd.k)) {
        const long long p = pidx(g.sy, g.sz, nd.i, nd.j, nd.k);
        const T* sg = sig_true<T>(e);
        // damped Jacobi with the row's own diagonal, as the level kernels do on the regular nodes
        T ax = T(0), diag = T(0);
        for (int c = 0; c < 8; ++c) {
            const int cc = nd.cell[c];
            if (cc == kEbCovered) continue;
            // cell c = (i - 1 + dx, j - 1 + dy, k - 1 + dz); this node is its corner a
            const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
            const int a = (1 - dx) | ((1 - dy) << 1) | ((1 - dz) << 2);
            const long long p0 = p - corner_off(g, a);  // the cell's low corner (and the cell's index)
            const T s = sg[p0];
            if (cc == kEbRegular) {
                for (int q = 0; q < 8; ++q) {
                    const T kq = s * (T)g.K[a ^ q];
                    if (x) ax += kq * x[p0 + corner_off(g, q)];
                    if (q == a) diag += kq;
                }
            } else {
                const double* K = e.cells[cc].K + 8 * a;
                for (int q = 0; q < 8; ++q) {
                    const T kq = s * (T)K[q];
                    if (x) ax += kq * x[p0 + corner_off(g, q)];
                    if (q == a) diag += kq;
                }
            }
        }
        // x == nullptr: a zero start
        const T xc = x ? x[p] : T(0);
        if (MODE == 0)
            v = diag > T(0) ? xc + omega * (b[p] - ax) / diag : xc;
        else
            v = b[p] - ax;
    }
    store_node(out, g, nd.i, nd.j, nd.k, v);
}

__global__ void __launch_bounds__(128) k_eb_rhs(NodalGeom g, EbNodal e, RhsArgs a, double* __restrict__ rhs)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= e.nnodes) return;
    const EbNodeEntry nd = e.nodes[t];
    if (node_is_dirichlet(g, nd.i, nd.j, nd.k)) return;
    const long long p = pidx(g.sy, g.sz, nd.i, nd.j, nd.k);
    double acc = 0.0;
    for (int c = 0; c < 8; ++c) {
        const int cc = nd.cell[c];
        if (cc < 0) continue;  // regular cells are in the level kernel's sum, covered ones carry nothing
        const EbNodeCell& ec = e.cells[cc];
        const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
        const int corner = (1 - dx) | ((1 - dy) << 1) | ((1 - dz) << 2);
        for (int d = 0; d < 3; ++d) {
            double u = *at4(a.vel, ec.i, ec.j, ec.k, d);
            if (a.add_gp) u += *at4(a.gp, ec.i, ec.j, ec.k, d) * e.sig64[ec.p];
            if (a.sub_old) u -= *at4(a.vel_old, ec.i, ec.j, ec.k, d);
            acc += ec.G[3 * corner + d] * u;
        }
    }
    // the embedded boundary's inflow: - int_EB (u_eb . n) N_n dA by the cell's one-point rule
    if (e.inflow)
        for (int c = 0; c < 8; ++c) {
            const int cc = nd.cell[c];
            if (cc < 0) continue;
            const int corner = (1 - (c & 1)) | ((1 - ((c >> 1) & 1)) << 1) | ((1 - (c >> 2)) << 2);
            acc -= e.inflow[8 * cc + corner];
        }
    // the level kernel's convention: g_n = sum over cells of int u . grad N_n
    rhs[p] += acc;
}

__global__ void __launch_bounds__(128) k_eb_inflow_shares(NodalGeom g, EbNodal e, gbp_array4 ev, gbp_array4 dap,
                                                          gbp_array4 bc, double* __restrict__ out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= e.ncells) return;
    const EbNodeCell& ec = e.cells[t];
    double F = 0.0, xb[3];
    for (int d = 0; d < 3; ++d) {
        F += *at4(ev, ec.i, ec.j, ec.k, d) * *at4(dap, ec.i, ec.j, ec.k, d) * (g.vol / g.h[d]);
        xb[d] = *at4(bc, ec.i, ec.j, ec.k, d);
    }
    for (int b = 0; b < 8; ++b) {
        double w = F;
        for (int d = 0; d < 3; ++d) w *= ((b >> d) & 1) ? 0.5 + xb[d] : 0.5 - xb[d];
        out[8 * t + b] = w;
    }
}

__global__ void __launch_bounds__(128) k_eb_correct(NodalGeom g, EbNodal e, CorrArgs a, const double* __restrict__ phi)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= e.ncells) return;
    const EbNodeCell& ec = e.cells[t];
    double G[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 8; ++q) {
        const double f = phi[ec.p + corner_off(g, q)];
        G[0] += ec.Gc[3 * q] * f;
        G[1] += ec.Gc[3 * q + 1] * f;
        G[2] += ec.Gc[3 * q + 2] * f;
    }
    const double sg = e.sig64[ec.p];
    for (int d = 0; d < 3; ++d) {
        double* up = at4(a.vel, ec.i, ec.j, ec.k, d);
        double u = *up;
        double gpo = 0.0;
        if (a.gp.data) gpo = *at4(a.gp, ec.i, ec.j, ec.k, d);
        if (a.add_gp) u = fma(gpo, sg, u);
        *up = fma(-sg, G[d], u);
        if (a.gradphi.data) *at4(a.gradphi, ec.i, ec.j, ec.k, d) = G[d];
        if (a.gp.data) *at4(a.gp, ec.i, ec.j, ec.k, d) = a.incremental ? gpo + G[d] : G[d];
    }
}

// level-0 sigma with cut cells: true sigma kept aside, the level kernels' sigma = sigma on regular
// cells only, the coarsening source = sigma x volume fraction
__global__ void k_eb_pack(gbp_array4 in, int c, int n0, int n1, int n2, double* __restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int i, j, k;
    split3(t, n0, n1, (long long)n0 * n1 * n2, i, j, k);
    out[t] = *at4(in, i, j, k, c);
}

__global__ void k_eb_sigma(long long count, const double* __restrict__ s, const double* __restrict__ kap,
                           const unsigned char* __restrict__ reg, double* __restrict__ st64, float* __restrict__ st32,
                           double* __restrict__ s64, float* __restrict__ s32, double* __restrict__ sk)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const double v = s[t];
    st64[t] = v;
    st32[t] = (float)v;
    const double r = reg[t] ? v : 0.0;
    s64[t] = r;
    s32[t] = (float)r;
    sk[t] = v * kap[t];
}

}  // namespace

template <typename T>
void eb_nodes(const NodalGeom& g, const EbNodal& e, int mode, const T* x, const T* b, T* out, double omega,
              cudaStream_t st)
{
    if (e.nnodes <= 0) return;
    const unsigned nb = (unsigned)((e.nnodes + 127) / 128);
    if (mode == 0)
        k_eb_node<T, 0><<<nb, 128, 0, st>>>(g, e, x, b, out, (T)omega);
    else
        k_eb_node<T, 1><<<nb, 128, 0, st>>>(g, e, x, b, out, (T)omega);
}
template void eb_nodes<double>(const NodalGeom&, const EbNodal&, int, const double*, const double*, double*, double,
                               cudaStream_t);
template void eb_nodes<float>(const NodalGeom&, const EbNodal&, int, const float*, const float*, float*, double,
                              cudaStream_t);

void eb_rhs(const NodalGeom& g, const EbNodal& e, const RhsArgs& a, double* rhs, cudaStream_t st)
{
    if (e.nnodes <= 0) return;
    k_eb_rhs<<<(unsigned)((e.nnodes + 127) / 128), 128, 0, st>>>(g, e, a, rhs);
}

void eb_inflow_shares(const NodalGeom& g, const EbNodal& e, const gbp_array4& eb_vel, const gbp_array4& dap,
                      const gbp_array4& bcent, double* out, cudaStream_t st)
{
    if (e.ncells <= 0) return;
    k_eb_inflow_shares<<<(unsigned)((e.ncells + 127) / 128), 128, 0, st>>>(g, e, eb_vel, dap, bcent, out);
}

void eb_correct(const NodalGeom& g, const EbNodal& e, const CorrArgs& a, const double* phi, cudaStream_t st)
{
    if (e.ncells <= 0) return;
    k_eb_correct<<<(unsigned)((e.ncells + 127) / 128), 128, 0, st>>>(g, e, a, phi);
}

void eb_sigma(const NodalGeom& g, const EbNodal& e, const double* s_in, double* s64, float* s32, double* sk,
              cudaStream_t st)
{
    k_eb_sigma<<<(unsigned)((g.count + 255) / 256), 256, 0, st>>>(g.count, s_in, e.kap, e.reg,
                                                                  const_cast<double*>(e.sig64),
                                                                  const_cast<float*>(e.sig32), s64, s32, sk);
}

}  // namespace gbp

namespace gbp {
void eb_pack_cells(const gbp_array4& in, int c, const int n[3], double* out, cudaStream_t st)
{
    const long long cnt = (long long)n[0] * n[1] * n[2];
    k_eb_pack<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(in, c, n[0], n[1], n[2], out);
}
}  // namespace gbp

namespace gbp {
namespace {
__global__ void k_mask_and(long long count, const unsigned char* a, const unsigned char* b, unsigned char* out,
                           unsigned* zeros)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const unsigned char v = (a ? a[t] : 1) && (b ? b[t] : 1);
    out[t] = v;
    (void)zeros;
}
}  // namespace
void mask_and(long long count, const unsigned char* a, const unsigned char* b, unsigned char* out, cudaStream_t st)
{
    k_mask_and<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(count, a, b, out, nullptr);
}
}  // namespace gbp

namespace gbp {
namespace {
// max |v| / V_fluid over the unique non-Dirichlet nodes (ivol = 1 / fluid volume of the node's dual
// cell, 0 on nodes that touch no fluid)
__global__ void __launch_bounds__(256) k_eb_norm(NodalGeom g, const double* __restrict__ v,
                                                 const double* __restrict__ ivol, unsigned long long* norm)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y,
        k = blockIdx.z * blockDim.z + threadIdx.z;
    double nv = 0.0;
    if (i < g.nu[0] && j < g.nu[1] && k < g.nu[2] && !node_is_dirichlet(g, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
        nv = v[p] != v[p] ? v[p] : fabs(v[p]) * ivol[p];
    }
    nv = block_max(nv);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomic_max_nonneg(norm, nv);
}
}  // namespace
void eb_norm(const NodalGeom& g, const double* v, const double* ivol, unsigned long long* norm, cudaStream_t st)
{
    k_eb_norm<<<dim3((g.nu[0] + 31) / 32, (g.nu[1] + 3) / 4, (g.nu[2] + 1) / 2), dim3(32, 4, 2), 0, st>>>(g, v, ivol,
                                                                                                      norm);
}
}  // namespace gbp
