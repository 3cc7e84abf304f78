// Tensor (velocity) diffusion solve and div tau: the kernels and the defect-correction driver
// (DiffusionTensorOp::diffuse_velocity / compute_divtau, src/diffusion/DiffusionTensorOp.cpp:104-317).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "gbp_internal.cuh"
#include "tensor.h"

namespace gbp {

namespace {

constexpr double kFourThirds = 4.0 / 3.0;

__device__ __forceinline__ double at(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data[(long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
                  (long long)n * a.nstride];
}
__device__ __forceinline__ double* atp(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
           (long long)n * a.nstride;
}

__device__ __forceinline__ bool cell3(const CellGeom& g, int& i, int& j, int& k)
{
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    k = blockIdx.z * blockDim.z + threadIdx.z;
    return i < g.n[0] && j < g.n[1] && k < g.n[2];
}

template <typename T>
struct V3 {
    T* c[3];
};
template <typename T>
struct CV3 {
    const T* c[3];
};
using U3 = V3<double>;
using CU3 = CV3<double>;

// raw face eta of direction d (no boundary factors): source 0 = face arrays, 1 = constant, 3 = the face
// average of a cell field with the adjacent cell on non-periodic domain sides
// (incflo::average_velocity_eta_to_faces + fixup_eta_on_domain_faces)
__global__ void k_tensor_eta(CellGeom g, int d, int source, gbp_array4 src, double cval, double* __restrict__ out)
{
    int f[3] = {(int)(blockIdx.x * blockDim.x + threadIdx.x), (int)(blockIdx.y * blockDim.y + threadIdx.y),
                (int)(blockIdx.z * blockDim.z + threadIdx.z)};
    for (int e = 0; e < 3; ++e)
        if (f[e] >= g.n[e] + (e == d ? 1 : 0)) return;
    const bool per = g.per[d];
    int q[3] = {f[0], f[1], f[2]};
    if (per && f[d] == g.n[d]) q[d] = 0;
    double v;
    if (source == 0) {
        v = at(src, q[0], q[1], q[2], 0);
    } else if (source == 1) {
        v = cval;
    } else {
        int lo[3] = {q[0], q[1], q[2]};
        lo[d] -= 1;
        if (per && lo[d] < 0) lo[d] += g.n[d];
        if (!per && f[d] == 0)
            v = at(src, q[0], q[1], q[2], 0);
        else if (!per && f[d] == g.n[d])
            v = at(src, lo[0], lo[1], lo[2], 0);
        else
            v = 0.5 * (at(src, lo[0], lo[1], lo[2], 0) + at(src, q[0], q[1], q[2], 0));
    }
    out[pidx(g.sy, g.sz, f[0], f[1], f[2])] = v;
}

__global__ void k_tensor_load(CellGeom g, gbp_array4 vel, U3 u)
{
    int i, j, k;
    if (!cell3(g, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
#pragma unroll
    for (int c = 0; c < 3; ++c) u.c[c][p] = at(vel, i, j, k, c);
}

__global__ void k_tensor_store(CellGeom g, CU3 u, gbp_array4 vel)
{
    int i, j, k;
    if (!cell3(g, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
#pragma unroll
    for (int c = 0; c < 3; ++c) *atp(vel, i, j, k, c) = u.c[c][p];
}

// V rhs into the padded right-hand sides, and max |rhs| into *norm
__global__ void k_tensor_rhs(CellGeom g, gbp_array4 rhs, U3 b, unsigned long long* norm)
{
    int i, j, k;
    double nv = 0.0;
    if (cell3(g, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double v = at(rhs, i, j, k, c);
            b.c[c][p] = g.vol * v;
            nv = fmax(nv, v != v ? v : fabs(v));
        }
    }
    nv = block_max(nv);
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomic_max_nonneg(norm, nv);
}

// weights of the face value at tangential index q of a side (q = -1 or n: continued past the edge,
// wrapped across a periodic direction, else extrapolated linearly from the last two faces)
__device__ __forceinline__ int edge_weights(int q, int n, int per, int idx[2], double w[2])
{
    if (q >= 0 && q < n) {
        idx[0] = q;
        w[0] = 1.0;
        return 1;
    }
    if (per) {
        idx[0] = q < 0 ? n - 1 : 0;
        w[0] = 1.0;
        return 1;
    }
    if (q < 0) {
        idx[0] = 0;
        idx[1] = 1;
    } else {
        idx[0] = n - 1;
        idx[1] = n - 2;
    }
    w[0] = 2.0;
    w[1] = -1.0;
    return 2;
}

// Ghost cells of direction d on both sides, all three components. Tangential ranges: directions before
// d over their ghosts too (-1 .. n), directions after d over the interior (they are filled later).
// bc[2][3]: the types of the low / high side per component. Dirichlet values come from vel's ghost cells.
// homog: the boundary values are zero (the correction equation of the FP32 inner steps)
template <typename T>
__global__ void k_tensor_ghost(CellGeom g, int d, int bl0, int bl1, int bl2, int bh0, int bh1, int bh2, V3<T> u,
                               gbp_array4 vel, int homog)
{
    const int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
    const int ext_e = e < d ? 1 : 0, ext_f = f < d ? 1 : 0;
    const int qe = (int)(blockIdx.x * blockDim.x + threadIdx.x) - ext_e;
    const int qf = (int)(blockIdx.y * blockDim.y + threadIdx.y) - ext_f;
    if (qe >= g.n[e] + ext_e || qf >= g.n[f] + ext_f) return;
    const int side = blockIdx.z;
    const int bcs[2][3] = {{bl0, bl1, bl2}, {bh0, bh1, bh2}};
    const int gd = side ? g.n[d] : -1;
    const int id = side ? g.n[d] - 1 : 0;   // the inner cell
    const int wd = side ? 0 : g.n[d] - 1;   // the periodic partner
    int cg[3], ci[3], cw[3];
    cg[d] = gd;
    ci[d] = id;
    cw[d] = wd;
    cg[e] = ci[e] = cw[e] = qe;
    cg[f] = ci[f] = cw[f] = qf;
    const long long pg = pidx(g.sy, g.sz, cg[0], cg[1], cg[2]);
    const long long pi = pidx(g.sy, g.sz, ci[0], ci[1], ci[2]);
    const long long pw = pidx(g.sy, g.sz, cw[0], cw[1], cw[2]);
    int ie[2], iff[2];
    double we[2], wf[2];
    const int ne = edge_weights(qe, g.n[e], g.per[e], ie, we);
    const int nf = edge_weights(qf, g.n[f], g.per[f], iff, wf);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int bc = bcs[side][c];
        T v;
        if (bc == GBP_BC_PERIODIC) {
            v = u.c[c][pw];
        } else if (bc == GBP_BC_NEUMANN) {
            v = u.c[c][pi];
        } else if (homog) {
            v = -u.c[c][pi];
        } else {
            double ub = 0.0;
            for (int a = 0; a < ne; ++a)
                for (int b = 0; b < nf; ++b) {
                    int q[3];
                    q[d] = gd;
                    q[e] = ie[a];
                    q[f] = iff[b];
                    ub += we[a] * wf[b] * at(vel, q[0], q[1], q[2], c);
                }
            v = (T)(2.0 * ub - u.c[c][pi]);
        }
        u.c[c][pg] = v;
    }
}

// Host-computed scale factors (FP64 division and most FP64 arithmetic are kept out of the kernels: GB300
// issues FP64 at 1/64 of the FP32 rate, and these kernels are bound by it)
template <typename T>
struct FaceKT {
    T ih[3];   // 1 / h_d
    T q[3];    // 1 / (4 h_e): tangential derivative from the four-cell difference sum
    T n43[3];  // (4/3) / h_d
    T t23[3];  // (2/3) / (4 h_e)
};
using FaceK = FaceKT<double>;

// tau_{c,d} / h_d (c = 0..2) on the face between cells L and R of direction d
template <int d, typename T>
__device__ __forceinline__ void face_tau(const CV3<T>& u, long long L, long long R, const long long s[3],
                                         const FaceKT<T>& K, T eta, T tau[3])
{
    constexpr int e1 = d == 0 ? 1 : 0, e2 = d == 2 ? 1 : 2;
    const T* u0 = u.c[d];
    const T* u1 = u.c[e1];
    const T* u2 = u.c[e2];
    // four-cell difference sums (tangential derivatives times 4 h_e)
    const T Tdd1 = (u0[R + s[e1]] - u0[R - s[e1]]) + (u0[L + s[e1]] - u0[L - s[e1]]);
    const T Tdd2 = (u0[R + s[e2]] - u0[R - s[e2]]) + (u0[L + s[e2]] - u0[L - s[e2]]);
    const T T11 = (u1[R + s[e1]] - u1[R - s[e1]]) + (u1[L + s[e1]] - u1[L - s[e1]]);
    const T T22 = (u2[R + s[e2]] - u2[R - s[e2]]) + (u2[L + s[e2]] - u2[L - s[e2]]);
    const T a = eta * K.ih[d];
    T t = K.n43[d] * (u0[R] - u0[L]);
    t = fma(-K.t23[e1], T11, t);
    t = fma(-K.t23[e2], T22, t);
    tau[d] = a * t;
    tau[e1] = a * fma(K.q[e1], Tdd1, K.ih[d] * (u1[R] - u1[L]));
    tau[e2] = a * fma(K.q[e2], Tdd2, K.ih[d] * (u2[R] - u2[L]));
}

// tau_{c,d} / h_d of every face of direction d (faces 0 .. n_d), once per face: fl[c] at the face's
// padded index
template <int d, typename T>
__global__ void __launch_bounds__(256) k_tensor_flux(CellGeom g, CV3<T> u, const T* __restrict__ eta, V3<T> fl,
                                                     FaceKT<T> K)
{
    int f[3] = {(int)(blockIdx.x * blockDim.x + threadIdx.x), (int)(blockIdx.y * blockDim.y + threadIdx.y),
                (int)(blockIdx.z * blockDim.z + threadIdx.z)};
    for (int e = 0; e < 3; ++e)
        if (f[e] >= g.n[e] + (e == d ? 1 : 0)) return;
    const long long s[3] = {1, g.sy, g.sz};
    const long long R = pidx(g.sy, g.sz, f[0], f[1], f[2]);
    T tau[3];
    face_tau<d, T>(u, R - s[d], R, s, K, eta[R], tau);
#pragma unroll
    for (int c = 0; c < 3; ++c) fl.c[c][R] = tau[c];
}

template <typename T>
struct Fl9T {
    const T* f[3][3];  // [direction][component]
};
using Fl9 = Fl9T<double>;

// MODE 0: r = b - (alpha a V u - beta V div tau) per component, max |r| / V into *norm when given (bvol =
// beta V). MODE 1: out(i, j, k, c) = div tau (FP64).
template <int MODE, typename T>
__global__ void __launch_bounds__(256) k_tensor_div(CellGeom g, Fl9T<T> fl, CV3<T> u, const T* __restrict__ a, T bvol,
                                                    double ivol, CV3<T> b, V3<T> r, unsigned long long* norm,
                                                    gbp_array4 out)
{
    int i, j, k;
    unsigned long long key = 0;
    if (cell3(g, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
        const long long s[3] = {1, g.sy, g.sz};
        T div[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            div[c] = ((fl.f[0][c][p + s[0]] - fl.f[0][c][p]) + (fl.f[1][c][p + s[1]] - fl.f[1][c][p])) +
                     (fl.f[2][c][p + s[2]] - fl.f[2][c][p]);
        if constexpr (MODE == 0) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T ax = a ? fma(a[p], u.c[c][p], -bvol * div[c]) : -bvol * div[c];
                const T v = b.c[c][p] - ax;
                r.c[c][p] = v;
                const unsigned long long kv = abs_key((double)v);
                key = kv > key ? kv : key;
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) *atp(out, i, j, k, c) = (double)div[c];
        }
    }
    if (MODE == 0 && norm) {
        key = block_max_key(key);
        if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) atomic_max_nonneg(norm, key_value(key) * ivol);
    }
}

// out = scale * v over whole padded arrays (FP64 -> FP32)
__global__ void k_tensor_to32(long long count, const double* __restrict__ v, double scale, float* __restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) out[t] = (float)(scale * v[t]);
}

// acc += e over whole padded arrays
__global__ void k_tensor_acc32(long long count, const float* __restrict__ e, float* __restrict__ acc)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) acc[t] += e[t];
}

// u += e / scale over whole padded arrays (FP32 correction into FP64)
__global__ void k_tensor_add(long long count, const float* __restrict__ e, double inv_scale, double* __restrict__ u)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < count) u[t] += (double)e[t] * inv_scale;
}

const dim3 kBlk(32, 4, 2);
dim3 cells_grid(const CellGeom& g)
{
    return dim3((unsigned)((g.n[0] + 31) / 32), (unsigned)((g.n[1] + 3) / 4), (unsigned)((g.n[2] + 1) / 2));
}

inline double bits_to_double(unsigned long long b)
{
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
}

}  // namespace

template <typename T>
static Fl9T<T> make_fl9(T* const fl[3][3])
{
    Fl9T<T> t{};
    for (int d = 0; d < 3; ++d)
        for (int c = 0; c < 3; ++c) t.f[d][c] = fl[d][c];
    return t;
}

// tau on every face of the three directions, once per face, in precision T
template <typename T>
static void tensor_fluxes(const CellGeom& g, T* const uu[3], T* const et[3], T* const f[3][3], cudaStream_t st)
{
    const CV3<T> uc{{uu[0], uu[1], uu[2]}};
    FaceKT<T> K;
    for (int d = 0; d < 3; ++d) {
        K.ih[d] = (T)(1.0 / g.h[d]);
        K.q[d] = (T)(0.25 / g.h[d]);
        K.n43[d] = (T)((4.0 / 3.0) / g.h[d]);
        K.t23[d] = (T)((2.0 / 3.0) * 0.25 / g.h[d]);
    }
    for (int d = 0; d < 3; ++d) {
        int fn[3] = {g.n[0], g.n[1], g.n[2]};
        fn[d] += 1;
        dim3 grid((unsigned)((fn[0] + 31) / 32), (unsigned)((fn[1] + 3) / 4), (unsigned)((fn[2] + 1) / 2));
        const V3<T> out{{f[d][0], f[d][1], f[d][2]}};
        if (d == 0)
            k_tensor_flux<0, T><<<grid, kBlk, 0, st>>>(g, uc, et[0], out, K);
        else if (d == 1)
            k_tensor_flux<1, T><<<grid, kBlk, 0, st>>>(g, uc, et[1], out, K);
        else
            k_tensor_flux<2, T><<<grid, kBlk, 0, st>>>(g, uc, et[2], out, K);
    }
}

// ghost cells of all three components, direction by direction (homog: zero boundary values)
template <typename T>
static void tensor_ghosts(const CellGeom& g, const int bclo[9], const int bchi[9], T* const uu[3],
                          const gbp_array4& vel, int homog, cudaStream_t st)
{
    for (int d = 0; d < 3; ++d) {
        const int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
        const int ne = g.n[e] + (e < d ? 2 : 0), nf = g.n[f] + (f < d ? 2 : 0);
        dim3 grid((unsigned)((ne + 31) / 32), (unsigned)((nf + 7) / 8), 2);
        k_tensor_ghost<T><<<grid, dim3(32, 8, 1), 0, st>>>(g, d, bclo[d], bclo[3 + d], bclo[6 + d], bchi[d],
                                                           bchi[3 + d], bchi[6 + d], V3<T>{{uu[0], uu[1], uu[2]}},
                                                           vel, homog);
    }
}

TensorSolver::~TensorSolver()
{
    pool.release();
    if (hnorm) cudaFreeHost(hnorm);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

int TensorSolver::init(const gbp_geometry& g, const int bc_lo[9], const int bc_hi[9], const gbp_options& o,
                       cudaStream_t stream)
{
    geom = g;
    opt = o;
    st = stream;
    for (int d = 0; d < 3; ++d) {
        const bool per = bc_lo[d] == GBP_BC_PERIODIC;
        for (int c = 0; c < 3; ++c) {
            const int lo = bc_lo[3 * c + d], hi = bc_hi[3 * c + d];
            if ((lo == GBP_BC_PERIODIC) != per || (hi == GBP_BC_PERIODIC) != per) {
                set_error("tensor: a periodic direction must be periodic on both sides for every component");
                return GBP_BAD_ARG;
            }
            for (int v : {lo, hi})
                if (v != GBP_BC_PERIODIC && v != GBP_BC_DIRICHLET && v != GBP_BC_NEUMANN && v != GBP_BC_INFLOW) {
                    set_error("tensor: boundary types must be periodic, Dirichlet (inflow) or Neumann");
                    return GBP_BAD_ARG;
                }
        }
        if (!per && g.n_cell[d] < 2) {
            set_error("tensor: a non-periodic direction needs at least 2 cells");
            return GBP_BAD_ARG;
        }
    }
    for (int q = 0; q < 9; ++q) {
        bclo[q] = bc_lo[q] == GBP_BC_INFLOW ? GBP_BC_DIRICHLET : bc_lo[q];
        bchi[q] = bc_hi[q] == GBP_BC_INFLOW ? GBP_BC_DIRICHLET : bc_hi[q];
    }
    // one V-cycle per block and step: the outer defect correction is what converges the cross terms,
    // so further inner cycles per step only sharpen the block-diagonal part
    gbp_options bo = opt;
    bo.ir_inner_cycles = 1;
    for (int c = 0; c < 3; ++c) {
        int rc = comp[c].init(g, bclo + 3 * c, bchi + 3 * c, bo, st);
        if (rc) return rc;
    }
    const CellGeom& cg = comp[0].finest();
    const size_t cnt = (size_t)cg.count;
    int rc = pool.reserve(21 * (cnt * sizeof(double) + 256) + 21 * (cnt * sizeof(float) + 256) + 4096);
    if (rc) return rc;
    for (int c = 0; c < 3; ++c) {
        u[c] = pool.take<double>(cnt);
        rhs[c] = pool.take<double>(cnt);
        r[c] = pool.take<double>(cnt);
        eta[c] = pool.take<double>(cnt);
        for (double* q : {u[c], rhs[c], r[c], eta[c]}) GBP_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * cnt, st));
    }
    for (int d = 0; d < 3; ++d)
        for (int c = 0; c < 3; ++c) {
            fl[d][c] = pool.take<double>(cnt);
            GBP_CUDA(cudaMemsetAsync(fl[d][c], 0, sizeof(double) * cnt, st));
        }
    // FP32 inner steps: correction, right-hand side, residual, face eta, fluxes
    for (int c = 0; c < 3; ++c) {
        e32[c] = pool.take<float>(cnt);
        b32[c] = pool.take<float>(cnt);
        r32[c] = pool.take<float>(cnt);
        eta32[c] = pool.take<float>(cnt);
        for (float* q : {e32[c], b32[c], r32[c], eta32[c]}) GBP_CUDA(cudaMemsetAsync(q, 0, sizeof(float) * cnt, st));
    }
    for (int d = 0; d < 3; ++d)
        for (int c = 0; c < 3; ++c) {
            fl32[d][c] = pool.take<float>(cnt);
            GBP_CUDA(cudaMemsetAsync(fl32[d][c], 0, sizeof(float) * cnt, st));
        }
    dnorm = pool.take<unsigned long long>(4);
    GBP_CUDA(cudaMallocHost(&hnorm, 4 * sizeof(unsigned long long)));
    GBP_CUDA(cudaEventCreate(&ev0));
    GBP_CUDA(cudaEventCreate(&ev1));
    return GBP_OK;
}

int TensorSolver::set_options(const gbp_options& o)
{
    gbp_options bo = o;
    bo.ir_inner_cycles = 1;
    for (int c = 0; c < 3; ++c) {
        int rc = comp[c].set_options(bo);
        if (rc) return rc;
    }
    opt = o;
    return GBP_OK;
}

size_t TensorSolver::device_bytes() const
{
    return pool.bytes + comp[0].device_bytes() + comp[1].device_bytes() + comp[2].device_bytes();
}

int TensorSolver::set_coeffs(double a_alpha, const gbp_array4* a, double a0, double a_beta, const gbp_array4* eta_cc,
                             const gbp_array4* const eta_f[3], double eta0)
{
    if (!(a_alpha > 0.0) || !(a_beta >= 0.0) || (!a && !(a0 > 0.0))) {
        set_error("tensor: need alpha > 0, beta >= 0 and a (array or a positive constant)");
        return GBP_BAD_ARG;
    }
    const bool faces = eta_f && eta_f[0] && eta_f[1] && eta_f[2];
    for (int c = 0; c < 3; ++c) {
        double sc[3] = {1.0, 1.0, 1.0};
        sc[c] = kFourThirds;
        int rc = comp[c].set_abec(a_alpha, a, a0, a_beta, faces ? eta_f : nullptr, eta0, eta_cc, sc);
        if (rc) return rc;
    }
    const CellGeom& g = comp[0].finest();
    for (int d = 0; d < 3; ++d) {
        int fn[3] = {g.n[0], g.n[1], g.n[2]};
        fn[d] += 1;
        dim3 grid((unsigned)((fn[0] + 31) / 32), (unsigned)((fn[1] + 3) / 4), (unsigned)((fn[2] + 1) / 2));
        gbp_array4 src{};
        int source = 1;
        if (eta_cc) {
            src = *eta_cc;
            source = 3;
        } else if (faces) {
            src = *eta_f[d];
            source = 0;
        }
        k_tensor_eta<<<grid, kBlk, 0, st>>>(g, d, source, src, eta0, eta[d]);
        k_tensor_to32<<<(unsigned)((g.count + 255) / 256), 256, 0, st>>>(g.count, eta[d], 1.0, eta32[d]);
    }
    GBP_CUDA(cudaGetLastError());
    alpha = a_alpha;
    beta = a_beta;
    ready = true;
    return GBP_OK;
}

int TensorSolver::check_vel(const gbp_array4& v, bool need_ghosts) const
{
    const CellGeom& g = comp[0].finest();
    if (!v.data || v.ncomp < 3 || v.jstride <= 0 || v.kstride <= 0 || v.nstride <= 0) return GBP_BAD_ARG;
    for (int d = 0; d < 3; ++d) {
        const int lo = need_ghosts && !g.per[d] ? -1 : 0;
        const int hi = need_ghosts && !g.per[d] ? g.n[d] : g.n[d] - 1;
        if (v.lo[d] > lo || v.hi[d] < hi) return GBP_BAD_ARG;
    }
    return GBP_OK;
}

void TensorSolver::load(const gbp_array4& vel)
{
    const CellGeom& g = comp[0].finest();
    k_tensor_load<<<cells_grid(g), kBlk, 0, st>>>(g, vel, U3{{u[0], u[1], u[2]}});
}

void TensorSolver::fluxes() { tensor_fluxes<double>(comp[0].finest(), u, eta, fl, st); }

void TensorSolver::fill_ghosts(const gbp_array4& vel) { tensor_ghosts<double>(comp[0].finest(), bclo, bchi, u, vel, 0, st); }

int TensorSolver::solve(const gbp_array4& rhs_in, gbp_array4& vel, gbp_stats* stats)
{
    if (!ready) {
        set_error("tensor solve: coefficients were never set");
        return GBP_BAD_ARG;
    }
    if (check_vel(vel, true)) {
        set_error("tensor solve: vel needs 3 components over the cells and one ghost layer on non-periodic sides");
        return GBP_BAD_ARG;
    }
    if (check_vel(rhs_in, false)) {
        set_error("tensor solve: rhs needs 3 components over the cells");
        return GBP_BAD_ARG;
    }
    const CellGeom& g = comp[0].finest();
    const CU3 uc{{u[0], u[1], u[2]}}, bc{{rhs[0], rhs[1], rhs[2]}};
    const U3 rr{{r[0], r[1], r[2]}};
    const Fl9 f9 = make_fl9(fl);
    GBP_CUDA(cudaEventRecord(ev0, st));
    GBP_CUDA(cudaMemsetAsync(dnorm, 0, 4 * sizeof(unsigned long long), st));
    k_tensor_rhs<<<cells_grid(g), kBlk, 0, st>>>(g, rhs_in, U3{{rhs[0], rhs[1], rhs[2]}}, dnorm);
    load(vel);
    fill_ghosts(vel);
    fluxes();
    k_tensor_div<0, double><<<cells_grid(g), kBlk, 0, st>>>(g, f9, uc, g.a64, beta * g.vol, 1.0 / g.vol, bc, rr,
                                                            dnorm + 1, gbp_array4{});
    GBP_CUDA(cudaGetLastError());
    GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    const double bnorm = bits_to_double(hnorm[0]);
    double rn = bits_to_double(hnorm[1]);
    if (!std::isfinite(bnorm) || !std::isfinite(rn)) {
        set_error("tensor solve: right-hand side or initial residual is not finite");
        if (stats) stats->status = GBP_NAN;
        return GBP_NAN;
    }
    const double r0 = rn;
    const double target = std::max(opt.rtol * (opt.always_use_bnorm ? bnorm : rn), opt.atol);
    double scale32 = 1.0;
    if (bnorm > 0.0) {
        int ex = 0;
        frexp(bnorm * g.vol, &ex);
        scale32 = ldexp(1.0, -ex);
    }
    int it = 0, status = GBP_OK, steps = 0;
    // mixed form: kInner block steps on the FP32 correction equation per FP64 residual (the residual of
    // the full operator in FP32 between them), as the single-level projections refine
    const bool inner32 = opt.precision == GBP_PREC_MIXED;
    const long long cnt = g.count;
    const unsigned nb = (unsigned)((cnt + 255) / 256);
    const Fl9T<float> f9s = make_fl9(fl32);
    const CV3<float> ce{{e32[0], e32[1], e32[2]}}, cb32{{b32[0], b32[1], b32[2]}};
    const V3<float> rr32{{r32[0], r32[1], r32[2]}};
    while (rn > target) {
        if (it >= opt.maxiter) {
            status = GBP_NOT_CONVERGED;
            set_error("tensor solve: maxiter reached before the tolerance");
            break;
        }
        if (inner32) {
            for (int c = 0; c < 3; ++c) {
                k_tensor_to32<<<nb, 256, 0, st>>>(cnt, r[c], scale32, b32[c]);
                GBP_CUDA(cudaMemsetAsync(e32[c], 0, sizeof(float) * cnt, st));
            }
            for (int q = 0; q < kInner; ++q) {
                for (int c = 0; c < 3; ++c) {
                    comp[c].vcycles32(q == 0 ? b32[c] : r32[c]);
                    k_tensor_acc32<<<nb, 256, 0, st>>>(cnt, comp[c].correction32(), e32[c]);
                }
                if (q + 1 < kInner) {
                    tensor_ghosts<float>(g, bclo, bchi, e32, vel, 1, st);
                    tensor_fluxes<float>(g, e32, eta32, fl32, st);
                    k_tensor_div<0, float><<<cells_grid(g), kBlk, 0, st>>>(g, f9s, ce, g.a32, (float)(beta * g.vol),
                                                                           0.0, cb32, rr32, nullptr, gbp_array4{});
                }
            }
            for (int c = 0; c < 3; ++c) k_tensor_add<<<nb, 256, 0, st>>>(cnt, e32[c], 1.0 / scale32, u[c]);
            steps += kInner;
        } else {
            for (int c = 0; c < 3; ++c) comp[c].add_vcycle_correction(r[c], u[c], scale32);
            ++steps;
        }
        fill_ghosts(vel);
        GBP_CUDA(cudaMemsetAsync(dnorm + 1, 0, sizeof(unsigned long long), st));
        fluxes();
        k_tensor_div<0, double><<<cells_grid(g), kBlk, 0, st>>>(g, f9, uc, g.a64, beta * g.vol, 1.0 / g.vol, bc, rr,
                                                                dnorm + 1, gbp_array4{});
        GBP_CUDA(cudaGetLastError());
        GBP_CUDA(cudaMemcpyAsync(hnorm + 1, dnorm + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        rn = bits_to_double(hnorm[1]);
        ++it;
        if (opt.verbose > 1) fprintf(stderr, "gbp tensor: iter %d rel resid %.3e\n", it, bnorm > 0 ? rn / bnorm : rn);
        if (!std::isfinite(rn)) {
            status = GBP_NAN;
            set_error("tensor solve: residual became NaN/Inf");
            break;
        }
    }
    k_tensor_store<<<cells_grid(g), kBlk, 0, st>>>(g, uc, vel);
    GBP_CUDA(cudaEventRecord(ev1, st));
    GBP_CUDA(cudaGetLastError());
    if (stats) {
        GBP_CUDA(cudaEventSynchronize(ev1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        stats->status = status;
        stats->outer_iters = it + 1;
        stats->vcycles = 3 * steps;  // one per component block and block step
        stats->rhs_norm = bnorm;
        stats->initial_rel_resid = bnorm > 0 ? r0 / bnorm : r0;
        stats->final_rel_resid = bnorm > 0 ? rn / bnorm : rn;
        stats->ms_solve = ms;
        stats->ms_total = ms;
    }
    return status;
}

int TensorSolver::apply(const gbp_array4& vel, gbp_array4& out)
{
    if (!ready) {
        set_error("tensor apply: coefficients were never set");
        return GBP_BAD_ARG;
    }
    if (check_vel(vel, true) || check_vel(out, false)) {
        set_error("tensor apply: vel (with its ghost layer) and divtau need 3 components over the cells");
        return GBP_BAD_ARG;
    }
    const CellGeom& g = comp[0].finest();
    load(vel);
    fill_ghosts(vel);
    fluxes();
    k_tensor_div<1, double><<<cells_grid(g), kBlk, 0, st>>>(g, make_fl9(fl), CU3{{u[0], u[1], u[2]}}, nullptr, 0.0,
                                                            0.0, CU3{{nullptr, nullptr, nullptr}},
                                                            U3{{nullptr, nullptr, nullptr}}, nullptr, out);
    GBP_CUDA(cudaGetLastError());
    GBP_CUDA(cudaStreamSynchronize(st));
    return GBP_OK;
}

}  // namespace gbp
