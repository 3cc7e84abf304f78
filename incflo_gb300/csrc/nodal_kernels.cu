// Nodal projection kernels: the Q1 (trilinear finite-element) variable-coefficient operator
// with cell sigma, its Jacobi smoother, residual, restriction, prolongation, single-CTA
// bottom solve, and the fused right-hand-side / correction kernels around the solve.
//
// Discretisation (the approximate projection behind Hydro::NodalProjector as used by
// incflo::ApplyNodalProjection, src/projection/incflo_apply_nodal_projection.cpp:95-267):
//   A_ij = sum over cells c of sigma_c * integral_c(grad N_i . grad N_j)   (weak form, SPD)
//   g_i  = integral(u . grad N_i) - inflow flux through the boundary        (= -V_i div u)
//   (grad phi)_c = average over the 4 cell edges of the nodal differences per direction
//   u_c -= sigma_c (grad phi)_c
// Relative residuals use the strong form |g_i - (A phi)_i| / V_i, V_i the node's control
// volume (h^3, halved per non-periodic boundary face), so they measure div(sigma grad phi) -
// div(u) like the max-norm convergence test of MLMG.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbp_internal.cuh"
#include "nodal_kernels.h"
#include "nodal_sweep.h"

namespace gbp {

// ---------------------------------------------------------------------------------------
// operator at one node
// ---------------------------------------------------------------------------------------
// Loads of the operator: plain (the level kernels), or L2-coherent ld.global.cg (kernels whose CTAs
// read what other CTAs of the same launch wrote before a cluster barrier: no stale L1 / texture line)
struct LdPlain {
    template <typename T>
    __device__ __forceinline__ static T ld(const T* p) { return *p; }
};
struct LdCg {
    __device__ __forceinline__ static float ld(const float* p) { return __ldcg(p); }
    __device__ __forceinline__ static double ld(const double* p) { return __ldcg(p); }
};

template <typename T>
struct NodalOp;

// FP64: the isotropic form sums sigma-weighted far-corner sums and subtracts the centre once
// (fewest FP64 instructions; FP64 issue rate, not HBM, bounds these kernels on GB300).
template <>
struct NodalOp<double> {
    template <bool ISO, typename LD = LdPlain>
    __device__ __forceinline__ static double apply(const double* __restrict__ x, const double* __restrict__ s,
                                                   long long c, long long sy, long long sz,
                                                   const NodalGeom& g, double& diag)
    {
        const double xc = LD::ld(x + c);
        double acc = 0.0, ssum = 0.0;
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int cx = 0; cx < 2; ++cx) {
                    const long long cell = c + (cx - 1) + (cy - 1) * sy + (cz - 1) * sz;
                    const double sg = LD::ld(s + cell);
                    const long long ox = cx ? 1 : -1, oy = cy ? sy : -sy, oz = cz ? sz : -sz;
                    ssum += sg;
                    if (ISO) {
                        double S = (LD::ld(x + c + ox + oy) + LD::ld(x + c + ox + oz)) +
                                   (LD::ld(x + c + oy + oz) + LD::ld(x + c + ox + oy + oz));
                        acc = fma(sg, S, acc);
                    } else {
                        double t = g.K[1] * (LD::ld(x + c + ox) - xc) + g.K[2] * (LD::ld(x + c + oy) - xc) +
                                   g.K[4] * (LD::ld(x + c + oz) - xc) + g.K[3] * (LD::ld(x + c + ox + oy) - xc) +
                                   g.K[5] * (LD::ld(x + c + ox + oz) - xc) + g.K[6] * (LD::ld(x + c + oy + oz) - xc) +
                                   g.K[7] * (LD::ld(x + c + ox + oy + oz) - xc);
                        acc = fma(sg, t, acc);
                    }
                }
        diag = g.K[0] * ssum;
        if (ISO) return g.K[3] * fma(-4.0 * xc, ssum, acc);
        return acc;
    }
};

// FP32: explicit differences to the centre keep the rounding error proportional to the
// local variation of x rather than to x itself.
template <>
struct NodalOp<float> {
    template <bool ISO, typename LD = LdPlain>
    __device__ __forceinline__ static float apply(const float* __restrict__ x, const float* __restrict__ s,
                                                  long long c, long long sy, long long sz,
                                                  const NodalGeom& g, float& diag)
    {
        const float xc = LD::ld(x + c);
        float acc = 0.f, ssum = 0.f;
        const float k1 = (float)g.K[1], k2 = (float)g.K[2], k4 = (float)g.K[4], k3 = (float)g.K[3],
                    k5 = (float)g.K[5], k6 = (float)g.K[6], k7 = (float)g.K[7];
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
            for (int cy = 0; cy < 2; ++cy)
#pragma unroll
                for (int cx = 0; cx < 2; ++cx) {
                    const long long cell = c + (cx - 1) + (cy - 1) * sy + (cz - 1) * sz;
                    const float sg = LD::ld(s + cell);
                    const long long ox = cx ? 1 : -1, oy = cy ? sy : -sy, oz = cz ? sz : -sz;
                    ssum += sg;
                    if (ISO) {
                        float S = ((LD::ld(x + c + ox + oy) - xc) + (LD::ld(x + c + ox + oz) - xc)) +
                                  ((LD::ld(x + c + oy + oz) - xc) + (LD::ld(x + c + ox + oy + oz) - xc));
                        acc = fmaf(sg, S, acc);
                    } else {
                        float t = k1 * (LD::ld(x + c + ox) - xc) + k2 * (LD::ld(x + c + oy) - xc) +
                                  k4 * (LD::ld(x + c + oz) - xc) + k3 * (LD::ld(x + c + ox + oy) - xc) +
                                  k5 * (LD::ld(x + c + ox + oz) - xc) + k6 * (LD::ld(x + c + oy + oz) - xc) +
                                  k7 * (LD::ld(x + c + ox + oy + oz) - xc);
                        acc = fmaf(sg, t, acc);
                    }
                }
        diag = (float)g.K[0] * ssum;
        if (ISO) return (float)g.K[3] * acc;
        return acc;
    }
};

// Smoother weight / diagonal. A Jacobi smoother only needs an approximate reciprocal, so the
// FP64 path uses the single-precision reciprocal when the diagonal is in range.
__device__ __forceinline__ double approx_recip(double d)
{
    double a = fabs(d);
    if (a > 1e-30 && a < 1e30) return (double)__frcp_rn((float)d);
    return 1.0 / d;
}
__device__ __forceinline__ float approx_recip(float d) { return __frcp_rn(d); }

__device__ __forceinline__ bool decode_node(const NodalGeom& g, long long t, int& i, int& j, int& k)
{
    const long long nxy = (long long)g.nu[0] * g.nu[1];
    if (t >= nxy * g.nu[2]) return false;
    if (t < 0x7fffffffll) {
        // 32-bit division where it fits (all levels below about 2^31 nodes): several times cheaper
        const unsigned u = (unsigned)t, uxy = (unsigned)nxy;
        k = (int)(u / uxy);
        const unsigned r = u - (unsigned)k * uxy;
        j = (int)(r / (unsigned)g.nu[0]);
        i = (int)(r - (unsigned)j * (unsigned)g.nu[0]);
        return true;
    }
    k = (int)(t / nxy);
    long long r = t - (long long)k * nxy;
    j = (int)(r / g.nu[0]);
    i = (int)(r - (long long)j * g.nu[0]);
    return true;
}

// 3-D launch over the unique nodes: block (32, 4, 2), no index division
__device__ __forceinline__ bool grid3_node(const NodalGeom& g, int& i, int& j, int& k)
{
    i = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    k = blockIdx.z * blockDim.z + threadIdx.z;
    return i < g.nu[0] && j < g.nu[1] && k < g.nu[2];
}

// ---------------------------------------------------------------------------------------
// smoother / residual / transfer
// ---------------------------------------------------------------------------------------
template <typename T, bool ISO, bool ZERO>
__global__ void __launch_bounds__(256) k_jacobi(NodalGeom g, const T* __restrict__ s, const T* __restrict__ xin,
                                                const T* __restrict__ b, T* __restrict__ xout, T omega)
{
    int i, j, k;
    if (!grid3_node(g, i, j, k)) return;
    T v = T(0);
    if (!node_is_dirichlet(g, i, j, k)) {
        const long long c = pidx(g.sy, g.sz, i, j, k);
        T diag;
        if (ZERO) {
            T ssum = T(0);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                ssum += s[c + ((q & 1) - 1) + (((q >> 1) & 1) - 1) * g.sy + (((q >> 2) & 1) - 1) * g.sz];
            diag = T(g.K[0]) * ssum;
            v = omega * b[c] * approx_recip(diag);
        } else {
            T ax = NodalOp<T>::template apply<ISO>(xin, s, c, g.sy, g.sz, g, diag);
            v = xin[c] + omega * (b[c] - ax) * approx_recip(diag);
        }
    }
    store_node(xout, g, i, j, k, v);
}

// r = b - A x, with the strong-form max norm accumulated into *norm when norm != nullptr.
// NodalOp::apply() evaluates sum_c sigma_c sum_{b != i} K(i,b) (x_b - x_i), which equals
// (A x)_i because every element row of K sums to zero.
template <typename T, bool ISO>
__global__ void __launch_bounds__(256) k_resid(NodalGeom g, const T* __restrict__ s, const T* __restrict__ x,
                                               const T* __restrict__ b, T* __restrict__ r,
                                               unsigned long long* norm)
{
    int i, j, k;
    double nv = 0.0;
    if (grid3_node(g, i, j, k)) {
        T v = T(0);
        if (!node_is_dirichlet(g, i, j, k)) {
            const long long c = pidx(g.sy, g.sz, i, j, k);
            T diag;
            T ax = NodalOp<T>::template apply<ISO>(x, s, c, g.sy, g.sz, g, diag);
            v = b[c] - ax;
            if (norm) nv = fabs((double)v) * node_inv_volume(g, i, j, k);
        }
        store_node(r, g, i, j, k, v);
    }
    if (norm) {
        nv = block_max(nv);
        if (threadIdx.x == 0) atomic_max_nonneg(norm, nv);
    }
}

// r = b - A x at the listed unique nodes only (nodes[t] = (i, j, k)); no aliases written
template <typename T, bool ISO>
__global__ void __launch_bounds__(256) k_resid_list(NodalGeom g, const T* __restrict__ s, const T* __restrict__ x,
                                                    const T* __restrict__ b, T* __restrict__ r,
                                                    const int4* __restrict__ nodes, int n)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int4 q = nodes[t];
    const long long c = pidx(g.sy, g.sz, q.x, q.y, q.z);
    T v = T(0);
    if (!node_is_dirichlet(g, q.x, q.y, q.z)) {
        T diag;
        v = b[c] - NodalOp<T>::template apply<ISO>(x, s, c, g.sy, g.sz, g, diag);
    }
    r[c] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_restrict(NodalGeom gf, NodalGeom gc, const T* __restrict__ rf,
                                                  T* __restrict__ bc)
{
    int I, J, K;
    if (!grid3_node(gc, I, J, K)) return;
    T v = T(0);
    if (!node_is_dirichlet(gc, I, J, K)) {
        const long long f = pidx(gf.sy, gf.sz, 2 * I, 2 * J, 2 * K);
        T acc = T(0);
#pragma unroll
        for (int c = -1; c <= 1; ++c) {
            T accy = T(0);
#pragma unroll
            for (int b = -1; b <= 1; ++b) {
                const long long row = f + b * gf.sy + c * gf.sz;
                T rx = T(0.5) * (rf[row - 1] + rf[row + 1]) + rf[row];
                accy += (b == 0 ? T(1) : T(0.5)) * rx;
            }
            acc += (c == 0 ? T(1) : T(0.5)) * accy;
        }
        v = acc;
    }
    bc[pidx(gc.sy, gc.sz, I, J, K)] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_prolong_add(NodalGeom gf, NodalGeom gc, const T* __restrict__ xc,
                                                     T* __restrict__ xf)
{
    int i, j, k;
    if (!grid3_node(gf, i, j, k)) return;
    if (node_is_dirichlet(gf, i, j, k)) return;
    const int I0 = i >> 1, J0 = j >> 1, K0 = k >> 1;
    const int oi = i & 1, oj = j & 1, ok = k & 1;
    const long long base = pidx(gc.sy, gc.sz, I0, J0, K0);
    T acc = T(0);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        if (c && !ok) break;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            if (b && !oj) break;
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                if (a && !oi) break;
                acc += xc[base + a + b * gc.sy + c * gc.sz];
            }
        }
    }
    const int sh = oi + oj + ok;
    const T w = sh == 0 ? T(1) : (sh == 1 ? T(0.5) : (sh == 2 ? T(0.25) : T(0.125)));
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    store_node(xf, gf, i, j, k, xf[p] + w * acc);
}

// fine += P xc with one thread per coarse node (I, J, K): it reads the 8 coarse nodes of the cell
// (I..I+1, J..J+1, K..K+1) once and updates the fine block (2I..2I+1, 2J..2J+1, 2K..2K+1), x pairs
// as one vector access. Fine nodes on Dirichlet faces lie on coarse Dirichlet faces, whose coarse
// values are 0, so they receive 0 without a test; with an overset mask every fine node is tested
// (a masked node with an odd index interpolates unmasked coarse nodes).
template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
    using type = float2;
};
template <>
struct Vec2<double> {
    using type = double2;
};

template <typename T>
__global__ void __launch_bounds__(256) k_prolong_block(NodalGeom gf, NodalGeom gc, const T* __restrict__ xc,
                                                       T* __restrict__ xf)
{
    int I, J, K;
    if (!grid3_node(gc, I, J, K)) return;
    const bool vx = 2 * I + 1 < gf.nu[0], vy = 2 * J + 1 < gf.nu[1], vz = 2 * K + 1 < gf.nu[2];
    const long long pc = pidx(gc.sy, gc.sz, I, J, K);
    T c[2][2][2];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
        for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx) {
                const bool need = (!cx || vx) && (!cy || vy) && (!cz || vz);
                c[cz][cy][cx] = need ? xc[pc + cx + cy * gc.sy + cz * gc.sz] : T(0);
            }
    const bool seam = (gf.per[0] && (2 * I <= 1 || 2 * I + 1 >= gf.n[0] - 1)) ||
                      (gf.per[1] && (2 * J <= 1 || 2 * J + 1 >= gf.n[1] - 1)) ||
                      (gf.per[2] && (2 * K <= 1 || 2 * K + 1 >= gf.n[2] - 1));
#pragma unroll
    for (int oz = 0; oz < 2; ++oz) {
        if (oz && !vz) break;
#pragma unroll
        for (int oy = 0; oy < 2; ++oy) {
            if (oy && !vy) break;
            // coarse values interpolated to (., 2J+oy, 2K+oz) at x = I and I+1
            T e0 = c[0][0][0], e1 = c[0][0][1];
            if (oy) {
                e0 = T(0.5) * (e0 + c[0][1][0]);
                e1 = T(0.5) * (e1 + c[0][1][1]);
            }
            if (oz) {
                T f0 = c[1][0][0], f1 = c[1][0][1];
                if (oy) {
                    f0 = T(0.5) * (f0 + c[1][1][0]);
                    f1 = T(0.5) * (f1 + c[1][1][1]);
                }
                e0 = T(0.5) * (e0 + f0);
                e1 = T(0.5) * (e1 + f1);
            }
            const T a0 = e0, a1 = T(0.5) * (e0 + e1);  // fine x = 2I, 2I+1
            const int i = 2 * I, j = 2 * J + oy, k = 2 * K + oz;
            const long long p = pidx(gf.sy, gf.sz, i, j, k);
            if (!seam && vx && !gf.mask) {
                using V = typename Vec2<T>::type;
                V v = *reinterpret_cast<const V*>(xf + p);
                v.x += a0;
                v.y += a1;
                *reinterpret_cast<V*>(xf + p) = v;
            } else {
                if (!(gf.mask && !gf.mask[p])) store_node(xf, gf, i, j, k, xf[p] + a0);
                if (vx && !(gf.mask && !gf.mask[p + 1])) store_node(xf, gf, i + 1, j, k, xf[p + 1] + a1);
            }
        }
    }
}

__global__ void k_mask_load(NodalGeom g, gbp_iarray4 m, unsigned char* __restrict__ out, unsigned* zeros)
{
    int i, j, k;
    if (!grid3_node(g, i, j, k)) return;
    const int v = m.data[(long long)(i - m.lo[0]) + (long long)(j - m.lo[1]) * m.jstride +
                         (long long)(k - m.lo[2]) * m.kstride];
    store_node(out, g, i, j, k, (unsigned char)(v != 0));
    if (!v) atomicAdd(zeros, 1u);
}

// A coarse node is free only where every fine node of its support (2I-1 .. 2I+1 per direction, inside
// the domain) is free. Injection alone moves the held region's edge outwards by up to one coarse spacing
// per level; the coarse correction then overshoots next to it and the V-cycle can diverge (measured at
// 128^3 with masks that vary within the planes).
__global__ void k_mask_coarsen(NodalGeom gf, NodalGeom gc, const unsigned char* __restrict__ mf,
                               unsigned char* __restrict__ mc)
{
    int I, J, K;
    if (!grid3_node(gc, I, J, K)) return;
    const int C[3] = {I, J, K};
    unsigned char v = 1;
    for (int q = 0; q < 27 && v; ++q) {
        int f[3];
        bool in = true;
        for (int d = 0; d < 3; ++d) {
            f[d] = 2 * C[d] + (d == 0 ? q % 3 : (d == 1 ? (q / 3) % 3 : q / 9)) - 1;
            if (gf.per[d]) {
                if (f[d] < 0) f[d] += gf.n[d];
                if (f[d] >= gf.n[d]) f[d] -= gf.n[d];
            } else if (f[d] < 0 || f[d] > gf.n[d]) {
                in = false;
            }
        }
        if (in && !mf[pidx(gf.sy, gf.sz, f[0], f[1], f[2])]) v = 0;
    }
    store_node(mc, gc, I, J, K, v);
}

// ---------------------------------------------------------------------------------------
// bottom solve: Jacobi-preconditioned CG in FP64 inside one CTA
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double v, double*) { return block_sum_all(v); }

template <typename T>
__global__ void __launch_bounds__(1024) k_bottom_cg(NodalGeom g, const double* __restrict__ s,
                                                    const T* __restrict__ bin, T* __restrict__ xout,
                                                    double* __restrict__ scr, int maxiter, double rtol,
                                                    double atol, int* info, int singular)
{
    __shared__ double red[32];
    const long long P = g.count;
    double* x = scr;
    double* r = scr + P;
    double* p = scr + 2 * P;
    double* q = scr + 3 * P;
    double* dg = scr + 4 * P;
    const long long N = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    // singular: no Dirichlet side and no pinning mask (the caller knows whether the level's mask pins phi
    // or only takes out nodes that touch no fluid)

    // clear the scratch (padding must hold zeros for the stencil)
    for (long long t = threadIdx.x; t < 5 * P; t += blockDim.x) scr[t] = 0.0;
    __syncthreads();

    double bs = 0.0;
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        const long long c = pidx(g.sy, g.sz, i, j, k);
        double bv = node_is_dirichlet(g, i, j, k) ? 0.0 : (double)bin[c];
        r[c] = bv;
        bs += bv;
        double d;
        double zero_unused = NodalOp<double>::apply<false>(x, s, c, g.sy, g.sz, g, d);
        (void)zero_unused;
        dg[c] = d;
    }
    if (singular) {
        // make the right-hand side consistent: remove its component along the null space
        double tot = block_sum(bs, red);
        double vtot = 0.0;
        for (long long t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_node(g, t, i, j, k);
            if (!node_is_dirichlet(g, i, j, k)) vtot += node_volume(g, i, j, k);
        }
        vtot = block_sum(vtot, red);
        double cfac = vtot > 0.0 ? tot / vtot : 0.0;
        for (long long t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_node(g, t, i, j, k);
            if (!node_is_dirichlet(g, i, j, k)) r[pidx(g.sy, g.sz, i, j, k)] -= cfac * node_volume(g, i, j, k);
        }
    }
    __syncthreads();

    // z = r / diag, p = z (with periodic aliases)
    double rz = 0.0, rr = 0.0;
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        const long long c = pidx(g.sy, g.sz, i, j, k);
        double z = node_is_dirichlet(g, i, j, k) ? 0.0 : r[c] / dg[c];
        store_node(p, g, i, j, k, z);
        rz += r[c] * z;
        rr += r[c] * r[c];
    }
    rz = block_sum(rz, red);
    rr = block_sum(rr, red);
    const double r0 = sqrt(rr);
    const double target = fmax(rtol * r0, atol > 0 ? atol : 0.0);
    int it = 0;
    if (r0 > 0.0) {
        for (it = 1; it <= maxiter; ++it) {
            __syncthreads();
            double pq = 0.0;
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_node(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                double d, v = 0.0;
                if (!node_is_dirichlet(g, i, j, k)) v = NodalOp<double>::apply<false>(p, s, c, g.sy, g.sz, g, d);
                q[c] = v;
                pq += p[c] * v;
            }
            pq = block_sum(pq, red);
            if (!(pq > 0.0)) break;
            const double alpha = rz / pq;
            double rz2 = 0.0;
            rr = 0.0;
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_node(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                x[c] += alpha * p[c];
                r[c] -= alpha * q[c];
                double z = node_is_dirichlet(g, i, j, k) ? 0.0 : r[c] / dg[c];
                q[c] = z;  // reuse q for z
                rz2 += r[c] * z;
                rr += r[c] * r[c];
            }
            rz2 = block_sum(rz2, red);
            rr = block_sum(rr, red);
            if (sqrt(rr) <= target) break;
            const double beta = rz2 / rz;
            rz = rz2;
            __syncthreads();
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_node(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                store_node(p, g, i, j, k, q[c] + beta * p[c]);
            }
        }
    }
    __syncthreads();
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        store_node(xout, g, i, j, k, (T)x[pidx(g.sy, g.sz, i, j, k)]);
    }
    if (threadIdx.x == 0 && info) {
        int used = it > maxiter ? maxiter : it;
        if (used > info[0]) info[0] = used;
    }
}

// Dense bottom solve: x = M b with M the precomputed FP64 inverse of the coarsest operator
// (singular systems: the inverse of A + c 1 1^T, exact for consistent b). M is symmetric and
// stored so that step v of the product reads a contiguous row across the threads.
template <typename T>
__global__ void __launch_bounds__(256) k_bottom_dense(NodalGeom g, const double* __restrict__ M,
                                                      const T* __restrict__ bin, T* __restrict__ xout, int singular)
{
    extern __shared__ double bb[];
    const int N = g.nu[0] * g.nu[1] * g.nu[2];
    double part = 0.0, vpart = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        const bool held = node_is_dirichlet(g, i, j, k);
        const double v = held ? 0.0 : (double)bin[pidx(g.sy, g.sz, i, j, k)];
        bb[t] = v;
        part += v;
        if (!held) vpart += node_volume(g, i, j, k);
    }
    if (singular) {
        // consistent right-hand side: remove the component along the constants of the free nodes
        // (masked nodes that touch no fluid are outside the system and keep 0)
        const double s = block_sum_all(part);
        const double vs = block_sum_all(vpart);
        const double c = vs > 0.0 ? s / vs : 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_node(g, t, i, j, k);
            if (!node_is_dirichlet(g, i, j, k)) bb[t] -= c * node_volume(g, i, j, k);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        double a0 = 0.0, a1 = 0.0;
        int v = 0;
        for (; v + 1 < N; v += 2) {
            a0 = fma(M[(size_t)v * N + t], bb[v], a0);
            a1 = fma(M[(size_t)(v + 1) * N + t], bb[v + 1], a1);
        }
        if (v < N) a0 = fma(M[(size_t)v * N + t], bb[v], a0);
        int i, j, k;
        decode_node(g, t, i, j, k);
        store_node(xout, g, i, j, k, (T)(a0 + a1));
    }
}

template <typename T>
void nodal_bottom_dense(const NodalGeom& g, const double* M, const T* b, T* x, int singular, cudaStream_t st)
{
    const int N = g.nu[0] * g.nu[1] * g.nu[2];
    k_bottom_dense<T><<<1, 256, N * sizeof(double), st>>>(g, M, b, x, singular);
}
template void nodal_bottom_dense<double>(const NodalGeom&, const double*, const double*, double*, int, cudaStream_t);
template void nodal_bottom_dense<float>(const NodalGeom&, const double*, const float*, float*, int, cudaStream_t);

// ---------------------------------------------------------------------------------------
// coarse V-cycle in one cluster
// ---------------------------------------------------------------------------------------
// one Jacobi sweep xout = xin + omega D^-1 (b - A xin) (zero: xin = 0) over the level's unique nodes
template <typename T>
__device__ __forceinline__ void cc_jacobi(const NodalGeom& g, const T* s, const T* xin, const T* b, T* xout, T omega,
                                          bool zero, long long t0, long long dt)
{
    const long long N = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    for (long long t = t0; t < N; t += dt) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        T v = T(0);
        if (!node_is_dirichlet(g, i, j, k)) {
            const long long c = pidx(g.sy, g.sz, i, j, k);
            T diag;
            if (zero) {
                T ssum = T(0);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    ssum += __ldcg(s + c + ((q & 1) - 1) + (((q >> 1) & 1) - 1) * g.sy + (((q >> 2) & 1) - 1) * g.sz);
                diag = T(g.K[0]) * ssum;
                v = omega * __ldcg(b + c) * approx_recip(diag);
            } else {
                const T ax = g.iso ? NodalOp<T>::template apply<true, LdCg>(xin, s, c, g.sy, g.sz, g, diag)
                                   : NodalOp<T>::template apply<false, LdCg>(xin, s, c, g.sy, g.sz, g, diag);
                v = __ldcg(xin + c) + omega * (__ldcg(b + c) - ax) * approx_recip(diag);
            }
        }
        store_node_unrolled(xout, g, i, j, k, v);
    }
}

template <typename T>
__device__ __forceinline__ void cc_resid(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, long long t0,
                                         long long dt)
{
    const long long N = (long long)g.nu[0] * g.nu[1] * g.nu[2];
    for (long long t = t0; t < N; t += dt) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        T v = T(0);
        if (!node_is_dirichlet(g, i, j, k)) {
            const long long c = pidx(g.sy, g.sz, i, j, k);
            T diag;
            const T ax = g.iso ? NodalOp<T>::template apply<true, LdCg>(x, s, c, g.sy, g.sz, g, diag)
                               : NodalOp<T>::template apply<false, LdCg>(x, s, c, g.sy, g.sz, g, diag);
            v = __ldcg(b + c) - ax;
        }
        store_node_unrolled(r, g, i, j, k, v);
    }
}

// full-weighting restriction (the transpose of trilinear prolongation), as k_restrict
template <typename T>
__device__ __forceinline__ void cc_restrict(const NodalGeom& gf, const NodalGeom& gc, const T* rf, T* bc, long long t0,
                                            long long dt)
{
    const long long N = (long long)gc.nu[0] * gc.nu[1] * gc.nu[2];
    for (long long t = t0; t < N; t += dt) {
        int I, J, K;
        decode_node(gc, t, I, J, K);
        T v = T(0);
        if (!node_is_dirichlet(gc, I, J, K)) {
            const long long f = pidx(gf.sy, gf.sz, 2 * I, 2 * J, 2 * K);
            T acc = T(0);
#pragma unroll
            for (int c = -1; c <= 1; ++c) {
                T accy = T(0);
#pragma unroll
                for (int b = -1; b <= 1; ++b) {
                    const long long row = f + b * gf.sy + c * gf.sz;
                    const T rx = T(0.5) * (__ldcg(rf + row - 1) + __ldcg(rf + row + 1)) + __ldcg(rf + row);
                    accy += (b == 0 ? T(1) : T(0.5)) * rx;
                }
                acc += (c == 0 ? T(1) : T(0.5)) * accy;
            }
            v = acc;
        }
        store_node_unrolled(bc, gc, I, J, K, v);
    }
}

// xf += P xc over the fine unique nodes (trilinear; Dirichlet and masked fine nodes keep their value)
template <typename T>
__device__ __forceinline__ void cc_prolong(const NodalGeom& gf, const NodalGeom& gc, const T* xc, T* xf, long long t0,
                                           long long dt)
{
    const long long N = (long long)gf.nu[0] * gf.nu[1] * gf.nu[2];
    for (long long t = t0; t < N; t += dt) {
        int i, j, k;
        decode_node(gf, t, i, j, k);
        if (node_is_dirichlet(gf, i, j, k)) continue;
        const int oi = i & 1, oj = j & 1, ok = k & 1;
        const long long base = pidx(gc.sy, gc.sz, i >> 1, j >> 1, k >> 1);
        T acc = T(0);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            if (c && !ok) break;
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                if (b && !oj) break;
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    if (a && !oi) break;
                    acc += __ldcg(xc + base + a + b * gc.sy + c * gc.sz);
                }
            }
        }
        const int sh = oi + oj + ok;
        const T w = sh == 0 ? T(1) : (sh == 1 ? T(0.5) : (sh == 2 ? T(0.25) : T(0.125)));
        const long long p = pidx(gf.sy, gf.sz, i, j, k);
        store_node_unrolled(xf, gf, i, j, k, __ldcg(xf + p) + w * acc);
    }
}

// x = M b on the bottom level by one CTA (the dense inverse; singular: b made consistent first), as
// k_bottom_dense
template <typename T>
__device__ __forceinline__ void cc_bottom(const NodalGeom& g, const double* M, const T* bin, T* xout, int singular,
                                          double* bb)
{
    const int N = g.nu[0] * g.nu[1] * g.nu[2];
    double part = 0.0, vpart = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_node(g, t, i, j, k);
        const bool held = node_is_dirichlet(g, i, j, k);
        const double v = held ? 0.0 : (double)__ldcg(bin + pidx(g.sy, g.sz, i, j, k));
        bb[t] = v;
        part += v;
        if (!held) vpart += node_volume(g, i, j, k);
    }
    if (singular) {
        const double sum = block_sum_all(part);
        const double vs = block_sum_all(vpart);
        const double c = vs > 0.0 ? sum / vs : 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_node(g, t, i, j, k);
            if (!node_is_dirichlet(g, i, j, k)) bb[t] -= c * node_volume(g, i, j, k);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        double a0 = 0.0, a1 = 0.0;
        int v = 0;
        for (; v + 1 < N; v += 2) {
            a0 = fma(M[(size_t)v * N + t], bb[v], a0);
            a1 = fma(M[(size_t)(v + 1) * N + t], bb[v + 1], a1);
        }
        if (v < N) a0 = fma(M[(size_t)v * N + t], bb[v], a0);
        int i, j, k;
        decode_node(g, t, i, j, k);
        store_node_unrolled(xout, g, i, j, k, (T)(a0 + a1));
    }
}

// Every thread runs the same phase sequence (no early exit: each must reach every cluster barrier).
template <typename T>
__global__ void __launch_bounds__(kCoarseThreads) k_coarse_vcycle(CoarseCycle<T> a)
{
    extern __shared__ double bb[];
    const long long t0 = (long long)cluster_rank() * blockDim.x + threadIdx.x;
    const long long dt = (long long)cluster_nctas() * blockDim.x;
    const int L = a.nl;
    int slot[kCoarseMaxLevels];  // 0: the level's x holds its iterate, 1: its t
    for (int q = 0; q + 1 < L; ++q) {
        const NodalGeom& g = a.g[q];
        T* buf[2] = {a.x[q], a.t[q]};
        int cur = 0;
        if (a.nu1 > 0) {
            cc_jacobi<T>(g, a.s[q], nullptr, a.b[q], buf[0], a.wpre[0], true, t0, dt);
            cluster_barrier();
            for (int p = 1; p < a.nu1; ++p) {
                cc_jacobi<T>(g, a.s[q], buf[cur], a.b[q], buf[cur ^ 1], a.wpre[p % kSweepWeights], false, t0, dt);
                cluster_barrier();
                cur ^= 1;
            }
        } else {
            for (long long t = t0; t < g.count; t += dt) buf[0][t] = T(0);
            cluster_barrier();
        }
        slot[q] = cur;
        cc_resid<T>(g, a.s[q], buf[cur], a.b[q], a.r[q], t0, dt);
        cluster_barrier();
        cc_restrict<T>(g, a.g[q + 1], a.r[q], a.b[q + 1], t0, dt);
        cluster_barrier();
    }
    if (cluster_rank() == 0) cc_bottom<T>(a.g[L - 1], a.M, a.b[L - 1], a.x[L - 1], a.singular, bb);
    slot[L - 1] = 0;
    cluster_barrier();
    for (int q = L - 2; q >= 0; --q) {
        const NodalGeom& g = a.g[q];
        T* buf[2] = {a.x[q], a.t[q]};
        int cur = slot[q];
        cc_prolong<T>(g, a.g[q + 1], slot[q + 1] ? a.t[q + 1] : a.x[q + 1], buf[cur], t0, dt);
        cluster_barrier();
        for (int p = 0; p < a.nu2; ++p) {
            cc_jacobi<T>(g, a.s[q], buf[cur], a.b[q], buf[cur ^ 1], a.wpost[p % kSweepWeights], false, t0, dt);
            cluster_barrier();
            cur ^= 1;
        }
        slot[q] = cur;
    }
}

int coarse_result_slot(int nu1, int nu2)
{
    const int pre = nu1 > 0 ? (nu1 - 1) & 1 : 0;
    return (pre + nu2) & 1;
}

int nodal_coarse_cluster_size()
{
    static int cached = -1;
    if (cached > 0) return cached;
    int best = 8;
    if (cudaFuncSetAttribute(k_coarse_vcycle<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(k_coarse_vcycle<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(kCoarseThreads);
        cfg.dynamicSmemBytes = 216 * sizeof(double);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n32 = 0, n64 = 0;
        if (cudaOccupancyMaxActiveClusters(&n32, k_coarse_vcycle<float>, &cfg) == cudaSuccess &&
            cudaOccupancyMaxActiveClusters(&n64, k_coarse_vcycle<double>, &cfg) == cudaSuccess && n32 > 0 && n64 > 0)
            best = 16;
    }
    cudaGetLastError();  // a refused attribute or query leaves no sticky error behind
    cached = best;
    return best;
}

template <typename T>
int nodal_coarse_vcycle(const CoarseCycle<T>& c, int cluster, cudaStream_t st)
{
    const NodalGeom& gb = c.g[c.nl - 1];
    const int nb = gb.nu[0] * gb.nu[1] * gb.nu[2];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(kCoarseThreads);
    cfg.dynamicSmemBytes = (size_t)nb * sizeof(double);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_coarse_vcycle<T>, c);
    return e == cudaSuccess ? GBP_OK : cuda_fail(e, "k_coarse_vcycle launch");
}
template int nodal_coarse_vcycle<float>(const CoarseCycle<float>&, int, cudaStream_t);
template int nodal_coarse_vcycle<double>(const CoarseCycle<double>&, int, cudaStream_t);

// ---------------------------------------------------------------------------------------
// level-0 set-up and the fused kernels around the solve
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double a4(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data[(long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride +
                  (long long)(k - a.lo[2]) * a.kstride + (long long)n * a.nstride];
}
__device__ __forceinline__ double* a4p(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride +
           (long long)(k - a.lo[2]) * a.kstride + (long long)n * a.nstride;
}

// cells away from a periodic seam have no alias: one store
__device__ __forceinline__ bool cell_alias_free(const NodalGeom& g, int i, int j, int k)
{
    return !((g.per[0] && (i == 0 || i == g.n[0] - 1)) || (g.per[1] && (j == 0 || j == g.n[1] - 1)) ||
             (g.per[2] && (k == 0 || k == g.n[2] - 1)));
}

template <typename T>
__device__ __forceinline__ void put_sigma_cell(T* a, const NodalGeom& g, int i, int j, int k, T v)
{
    if (cell_alias_free(g, i, j, k))
        a[pidx(g.sy, g.sz, i, j, k)] = v;
    else
        store_sigma_cell(a, g, i, j, k, v);
}

// 3-D launch over the cells (block 32 x 4 x 2): no index division
__global__ void __launch_bounds__(256) k_sigma_from_rho(NodalGeom g, gbp_array4 rho, int have_rho, double scale,
                                                        double rho0, double* __restrict__ s64, float* __restrict__ s32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= g.n[0] || j >= g.n[1] || k >= g.n[2]) return;
    const double v = have_rho ? scale / a4(rho, i, j, k, 0) : scale / rho0;
    put_sigma_cell(s64, g, i, j, k, v);
    if (s32) put_sigma_cell(s32, g, i, j, k, (float)v);
}

__global__ void __launch_bounds__(256) k_sigma_copy(NodalGeom g, gbp_array4 sig, int have_sig, double cval,
                                                    double* __restrict__ s64, float* __restrict__ s32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= g.n[0] || j >= g.n[1] || k >= g.n[2]) return;
    const double v = have_sig ? a4(sig, i, j, k, 0) : cval;
    put_sigma_cell(s64, g, i, j, k, v);
    if (s32) put_sigma_cell(s32, g, i, j, k, (float)v);
}

__global__ void k_sigma_coarsen(NodalGeom gf, NodalGeom gc, const double* __restrict__ sf,
                                double* __restrict__ sc64, float* __restrict__ sc32)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nxy = (long long)gc.n[0] * gc.n[1];
    if (t >= nxy * gc.n[2]) return;
    int i, j, k;
    split3(t, gc.n[0], gc.n[1], nxy * gc.n[2], i, j, k);
    const long long f = pidx(gf.sy, gf.sz, 2 * i, 2 * j, 2 * k);
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) acc += sf[f + (q & 1) + ((q >> 1) & 1) * gf.sy + ((q >> 2) & 1) * gf.sz];
    const double v = 0.125 * acc;
    store_sigma_cell(sc64, gc, i, j, k, v);
    if (sc32) store_sigma_cell(sc32, gc, i, j, k, (float)v);
}

// Tiles of the z-marching FP64 kernels: a CTA of 33 x 9 threads covers 32 x 8 node columns; thread
// (tx, ty) owns cell column and node column (x0 - 1 + tx, y0 - 1 + ty) (a cell is named by its low
// node), the threads with tx, ty >= 1 own nodes, and the CTA walks a z range one layer at a time.
constexpr int ZX = 32, ZY = 8, ZTX = ZX + 1, ZTY = ZY + 1;

// z chunk length for a bx x by tile grid over nz planes: about 4 waves of CTAs
static int zchunk(int bx, int by, int nz)
{
    const int want = std::max(1, 4 * sm_count_cached() * 6 / std::max(1, bx * by));
    return std::max(4, (nz + want - 1) / want);
}

// g = -(weak divergence) of u' = u + (add_gp ? sigma*gp : 0) - (sub_old ? u_old : 0), for the nodes.
// Each cell of a layer computes its weak fluxes F_d = (h_e h_f / 4) u'_d once (ghost cells carry F
// only across an inflow face, and only the normal component; other ghosts carry 0); a node sums +-F
// over its 8 cells in separable form: per layer the x difference of y-pair sums of F_x, the y
// difference of x-pair sums of F_y and the 4-cell sum of F_z, then layers k-1 and k.
// part: per-CTA sums of g (consistency correction of singular systems).
__global__ void __launch_bounds__(ZTX* ZTY) k_nodal_rhs(NodalGeom g, RhsArgs a, const double* __restrict__ s64,
                                                        double* __restrict__ b, double* __restrict__ part, int kchunk,
                                                        int zb0, int nzb)
{
    __shared__ double F[2][3][ZTY][ZTX];
    const int tx = threadIdx.x % ZTX, ty = threadIdx.x / ZTX;
    const int ci = blockIdx.x * ZX - 1 + tx, cj = blockIdx.y * ZY - 1 + ty;
    const int zb = zb0 + blockIdx.z;  // z chunk (a launch may cover a subset of them)
    const int kbeg = zb * kchunk;
    const int kend = min(kbeg + kchunk, g.nu[2]);
    const bool owner = tx >= 1 && ty >= 1 && ci < g.nu[0] && cj < g.nu[1];
    // cells beyond the last node column are never read by an owner
    const bool used = ci < g.nu[0] && cj < g.nu[1];
    // x / y part of this cell column: periodic wrap, or out of the domain (ghost)
    int c0 = ci, c1 = cj, nout_xy = 0, dout_xy = -1;
    if (g.per[0]) {
        if (c0 < 0) c0 += g.n[0];
        if (c0 >= g.n[0]) c0 -= g.n[0];
    } else if (c0 < 0 || c0 >= g.n[0]) {
        ++nout_xy;
        dout_xy = 0;
    }
    if (g.per[1]) {
        if (c1 < 0) c1 += g.n[1];
        if (c1 >= g.n[1]) c1 -= g.n[1];
    } else if (c1 < 0 || c1 >= g.n[1]) {
        ++nout_xy;
        dout_xy = 1;
    }
    double A0p = 0.0, A1p = 0.0, Q2p = 0.0, acc = 0.0;
    for (int L = kbeg - 1; L < kend; ++L) {
        const int buf = (L - kbeg + 1) & 1;
        double f0 = 0.0, f1 = 0.0, f2 = 0.0;
        if (used) {
            int c2 = L, nout = nout_xy, dout = dout_xy;
            if (g.per[2]) {
                if (c2 < 0) c2 += g.n[2];
                if (c2 >= g.n[2]) c2 -= g.n[2];
            } else if (c2 < 0 || c2 >= g.n[2]) {
                ++nout;
                dout = 2;
            }
            if (nout == 0 && a.cmask && !a.cmask[pidx(g.sy, g.sz, c0, c1, c2)]) {
                // not a leaf cell of this level: no flux
            } else if (nout == 0) {
                const long long off = (long long)(c0 - a.vel.lo[0]) + (long long)(c1 - a.vel.lo[1]) * a.vel.jstride +
                                      (long long)(c2 - a.vel.lo[2]) * a.vel.kstride;
                double u0 = a.vel.data[off], u1 = a.vel.data[off + a.vel.nstride],
                       u2 = a.vel.data[off + 2 * a.vel.nstride];
                if (a.add_gp) {
                    const double sg = s64[pidx(g.sy, g.sz, c0, c1, c2)];
                    const long long og = (long long)(c0 - a.gp.lo[0]) + (long long)(c1 - a.gp.lo[1]) * a.gp.jstride +
                                         (long long)(c2 - a.gp.lo[2]) * a.gp.kstride;
                    u0 = fma(a.gp.data[og], sg, u0);
                    u1 = fma(a.gp.data[og + a.gp.nstride], sg, u1);
                    u2 = fma(a.gp.data[og + 2 * a.gp.nstride], sg, u2);
                }
                if (a.sub_old) {
                    const long long oo = (long long)(c0 - a.vel_old.lo[0]) +
                                         (long long)(c1 - a.vel_old.lo[1]) * a.vel_old.jstride +
                                         (long long)(c2 - a.vel_old.lo[2]) * a.vel_old.kstride;
                    u0 -= a.vel_old.data[oo];
                    u1 -= a.vel_old.data[oo + a.vel_old.nstride];
                    u2 -= a.vel_old.data[oo + 2 * a.vel_old.nstride];
                }
                f0 = a.cf[0] * u0;
                f1 = a.cf[1] * u1;
                f2 = a.cf[2] * u2;
            } else if (nout == 1) {
                // the ghost cell across one face: its raw (unwrapped) index in that direction
                int q[3] = {c0, c1, c2};
                q[dout] = dout == 0 ? ci : (dout == 1 ? cj : L);
                const int inflow = q[dout] < 0 ? a.inflow_lo[dout] : a.inflow_hi[dout];
                if (inflow) {
                    const double fv = a.cf[dout] * a4(a.vel, q[0], q[1], q[2], dout);
                    if (dout == 0) f0 = fv;
                    else if (dout == 1) f1 = fv;
                    else f2 = fv;
                }
            }
        }
        F[buf][0][ty][tx] = f0;
        F[buf][1][ty][tx] = f1;
        F[buf][2][ty][tx] = f2;
        __syncthreads();
        if (owner) {
            const double(*F0)[ZTX] = F[buf][0];
            const double(*F1)[ZTX] = F[buf][1];
            const double(*F2)[ZTX] = F[buf][2];
            const double A0 = (F0[ty - 1][tx] + F0[ty][tx]) - (F0[ty - 1][tx - 1] + F0[ty][tx - 1]);
            const double A1 = (F1[ty][tx - 1] + F1[ty][tx]) - (F1[ty - 1][tx - 1] + F1[ty - 1][tx]);
            const double Q2 = (F2[ty - 1][tx - 1] + F2[ty - 1][tx]) + (F2[ty][tx - 1] + F2[ty][tx]);
            if (L >= kbeg) {
                // node (ci, cj, L): layers L-1 and L
                double gv = 0.0;
                if (!node_is_dirichlet(g, ci, cj, L)) gv = -(((A0p + A0) + (A1p + A1)) + (Q2 - Q2p));
                b[pidx(g.sy, g.sz, ci, cj, L)] = gv;
                acc += gv;
            }
            A0p = A0;
            A1p = A1;
            Q2p = Q2;
        }
    }
    if (part) {
        const double t = block_sum_all(acc);
        if (threadIdx.x == 0) part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * zb)] = t;
    }
    (void)nzb;
}

// strong-form max norm max_i |v_i| / V_i over the unique non-Dirichlet nodes
__global__ void __launch_bounds__(256) k_node_norm(NodalGeom g, const double* __restrict__ v, unsigned long long* norm)
{
    double nv = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (!decode_node(g, t, i, j, k)) break;
        if (!node_is_dirichlet(g, i, j, k))
            nv = nanmax(nv, fabs(v[pidx(g.sy, g.sz, i, j, k)]) * node_inv_volume(g, i, j, k));
    }
    nv = block_max(nv);
    if (threadIdx.x == 0) atomic_max_nonneg(norm, nv);
}

// Per-block partial sums (weighted: sum V_i v_i), grid-stride over the unique nodes.
// Tiled launches over the unique nodes without index division: block (32, 8), each thread walks
// a z chunk of its node column.
__global__ void __launch_bounds__(256) k_node_sums(NodalGeom g, const double* __restrict__ v, int weighted,
                                                   double* __restrict__ part, int kchunk)
{
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    const int kbeg = blockIdx.z * kchunk, kend = min(kbeg + kchunk, g.nu[2]);
    double acc = 0.0;
    if (i < g.nu[0] && j < g.nu[1])
        for (int k = kbeg; k < kend; ++k) {
            const double x = v[pidx(g.sy, g.sz, i, j, k)];
            acc += weighted ? x * node_volume(g, i, j, k) : x;
        }
    acc = block_sum_all(acc);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = acc;
}

// One block folds the partials in a fixed order: scal = sum / vtot.
__global__ void __launch_bounds__(1024) k_fold(const double* __restrict__ part, int nparts, double vtot,
                                               double* __restrict__ scal)
{
    double acc = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x) acc += part[t];
    acc = block_sum_all(acc);
    if (threadIdx.x == 0) *scal = acc / vtot;
}

// mode 0: b_i -= V_i c (consistent right-hand side of a singular system), and the strong-form
//         max norm of the corrected b into *norm
// mode 1: x_i -= c (gauge: volume-weighted mean zero), with periodic aliases
__global__ void __launch_bounds__(256) k_remove_mean(NodalGeom g, double* __restrict__ v, const double* __restrict__ scal,
                                                     int mode, unsigned long long* norm, int kchunk)
{
    const double c = *scal;
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    const int kbeg = blockIdx.z * kchunk, kend = min(kbeg + kchunk, g.nu[2]);
    // node volume = V / 2^(boundary count): the x / y part is fixed along the column; the norm keeps
    // the max of |b| 2^e as an integer key and multiplies by 1/V once (FP64 instructions are the
    // bound of this kernel on GB300)
    const int exy = (!g.per[0] && (i == 0 || i == g.n[0])) + (!g.per[1] && (j == 0 || j == g.n[1]));
    const double cv = c * (exy == 0 ? g.vol : (exy == 1 ? 0.5 * g.vol : 0.25 * g.vol));
    const double cvz = 0.5 * cv;  // on a z boundary plane
    unsigned long long key = 0;
    if (i < g.nu[0] && j < g.nu[1])
        for (int k = kbeg; k < kend; ++k) {
            const long long p = pidx(g.sy, g.sz, i, j, k);
            if (mode == 0) {
                const int e = exy + (!g.per[2] && (k == 0 || k == g.n[2]));
                const double bv = v[p] - (e == exy ? cv : cvz);
                v[p] = bv;
                const unsigned long long kb = e == 0 ? abs_key(bv) : abs_key(bv * (double)(1 << e));
                key = kb > key ? kb : key;
            } else {
                store_node(v, g, i, j, k, v[p] - c);
            }
        }
    if (mode == 0 && norm) {
        key = block_max_key(key);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(norm, key_value(key) * g.ivol);
    }
}

template <typename TE>
__global__ void __launch_bounds__(256) k_add_correction(NodalGeom g, double* __restrict__ x, const TE* __restrict__ e,
                                                        double inv_scale)
{
    int i, j, k;
    if (!grid3_node(g, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    store_node(x, g, i, j, k, x[p] + (double)e[p] * inv_scale);
}

__global__ void __launch_bounds__(256) k_to_f32(NodalGeom g, const double* __restrict__ r, float* __restrict__ r32,
                                                double scale)
{
    int i, j, k;
    if (!grid3_node(g, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    r32[p] = (float)(r[p] * scale);
}

// u <- u + (add_gp ? sigma*gp : 0) - sigma*G phi; gradphi <- G phi; gp <- G phi (+= if incremental).
// z-marching tile (33 x 9 node columns for 32 x 8 cell columns): each node column forms the z-pair sum
// S and difference D of its two planes once; a cell's gradient is then
//   4h G_x = (S10 + S11) - (S00 + S01), 4h G_y = (S01 + S11) - (S00 + S10), 4h G_z = (D00 + D10) + (D01 + D11)
// (Sab = node column (i+a, j+b)), 9 additions instead of 21.
__global__ void __launch_bounds__(ZTX* ZTY) k_nodal_correct(NodalGeom g, CorrArgs a, const double* __restrict__ s64,
                                                            const double* __restrict__ phi, int kchunk, int k0, int k1)
{
    __shared__ double S[2][ZTY][ZTX], D[2][ZTY][ZTX];
    const int tx = threadIdx.x % ZTX, ty = threadIdx.x / ZTX;
    const int ni = blockIdx.x * ZX + tx, nj = blockIdx.y * ZY + ty;  // node column; cell column = same
    const int kbeg = k0 + blockIdx.z * kchunk;
    const int kend = min(kbeg + kchunk, k1);
    // node columns 0..n (index n: the periodic alias or the high boundary node)
    const bool has_node = ni <= g.n[0] && nj <= g.n[1];
    const bool cell = tx < ZX && ty < ZY && ni < g.n[0] && nj < g.n[1];
    const long long pc = pidx(g.sy, g.sz, ni, nj, kbeg);
    double plo = has_node ? phi[pc] : 0.0;
    for (int k = kbeg; k < kend; ++k) {
        const int buf = (k - kbeg) & 1;
        const long long pk = pc + (long long)(k - kbeg) * g.sz;
        const double phi_hi = has_node ? phi[pk + g.sz] : 0.0;
        S[buf][ty][tx] = plo + phi_hi;
        D[buf][ty][tx] = phi_hi - plo;
        plo = phi_hi;
        __syncthreads();
        if (cell && (!a.cmask || a.cmask[pk])) {
            const double S00 = S[buf][ty][tx], S10 = S[buf][ty][tx + 1], S01 = S[buf][ty + 1][tx],
                         S11 = S[buf][ty + 1][tx + 1];
            const double D00 = D[buf][ty][tx], D10 = D[buf][ty][tx + 1], D01 = D[buf][ty + 1][tx],
                         D11 = D[buf][ty + 1][tx + 1];
            double G[3];
            G[0] = ((S10 + S11) - (S00 + S01)) * a.inv4h[0];
            G[1] = ((S01 + S11) - (S00 + S10)) * a.inv4h[1];
            G[2] = ((D00 + D10) + (D01 + D11)) * a.inv4h[2];
            const double sg = s64[pk];
            const long long ov = (long long)(ni - a.vel.lo[0]) + (long long)(nj - a.vel.lo[1]) * a.vel.jstride +
                                 (long long)(k - a.vel.lo[2]) * a.vel.kstride;
            long long og = 0;
            if (a.gp.data)
                og = (long long)(ni - a.gp.lo[0]) + (long long)(nj - a.gp.lo[1]) * a.gp.jstride +
                     (long long)(k - a.gp.lo[2]) * a.gp.kstride;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double* up = a.vel.data + ov + d * a.vel.nstride;
                double u = *up;
                double gpo = 0.0;
                if (a.gp.data) gpo = a.gp.data[og + d * a.gp.nstride];
                if (a.add_gp) u = fma(gpo, sg, u);
                *up = fma(-sg, G[d], u);
                if (a.gradphi.data) *a4p(a.gradphi, ni, nj, k, d) = G[d];
                if (a.gp.data) a.gp.data[og + d * a.gp.nstride] = a.incremental ? gpo + G[d] : G[d];
            }
        }
    }
}

// p_nd (nodal, all nodes 0..n) <- phi (+= if incremental)
__global__ void __launch_bounds__(256) k_nodal_store_phi(NodalGeom g, gbp_array4 out, const double* __restrict__ phi,
                                                         int accumulate)
{
    // 3-D launch over all nodes 0..n (block 32 x 4 x 2)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i > g.n[0] || j > g.n[1] || k > g.n[2]) return;
    const double v = phi[pidx(g.sy, g.sz, i, j, k)];
    double* p = a4p(out, i, j, k, 0);
    *p = accumulate ? *p + v : v;
}

// div(i,j,k) = -g_i / V_i (strong-form nodal divergence) on all nodes 0..n; the periodic duplicate
// node n reads its unique node 0
__global__ void k_nodal_store_div(NodalGeom g, gbp_array4 out, const double* __restrict__ b)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int n0 = g.n[0] + 1, n1 = g.n[1] + 1, n2 = g.n[2] + 1;
    const long long nxy = (long long)n0 * n1;
    if (t >= nxy * n2) return;
    int i, j, k;
    split3(t, n0, n1, nxy * n2, i, j, k);
    const int iu = (g.per[0] && i == g.n[0]) ? 0 : i;
    const int ju = (g.per[1] && j == g.n[1]) ? 0 : j;
    const int ku = (g.per[2] && k == g.n[2]) ? 0 : k;
    *a4p(out, i, j, k, 0) = -b[pidx(g.sy, g.sz, iu, ju, ku)] * node_inv_volume(g, iu, ju, ku);
}

void nodal_store_div(const NodalGeom& g, const gbp_array4& out, const double* b, cudaStream_t st)
{
    const long long n = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
    k_nodal_store_div<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, out, b);
}

__global__ void k_nodal_load_phi(NodalGeom g, gbp_array4 in, double* __restrict__ phi)
{
    int i, j, k;
    if (!grid3_node(g, i, j, k)) return;
    const double v = node_is_dirichlet(g, i, j, k) ? 0.0 : a4(in, i, j, k, 0);
    store_node(phi, g, i, j, k, v);
}

// Streaming reference for the sweep rooflines: out = a + b + c over whole padded arrays (three reads,
// one write, perfectly coalesced float4) -- the best any level sweep of the same arrays can do.
__global__ void __launch_bounds__(256) k_stream_triad(const float4* __restrict__ a, const float4* __restrict__ b,
                                                      const float4* __restrict__ c, float4* __restrict__ out, long long n4)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n4; t += (long long)gridDim.x * blockDim.x) {
        const float4 x = __ldg(a + t), y = __ldg(b + t), z = __ldg(c + t);
        out[t] = make_float4(x.x + y.x + z.x, x.y + y.y + z.y, x.z + y.z + z.z, x.w + y.w + z.w);
    }
}

void stream_triad(const float* a, const float* b, const float* c, float* out, long long n, cudaStream_t st)
{
    const long long n4 = n / 4;
    k_stream_triad<<<152 * 8, 256, 0, st>>>(reinterpret_cast<const float4*>(a), reinterpret_cast<const float4*>(b),
                                            reinterpret_cast<const float4*>(c), reinterpret_cast<float4*>(out), n4);
}

// ---------------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------------
static inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }
static inline long long nunique(const NodalGeom& g) { return (long long)g.nu[0] * g.nu[1] * g.nu[2]; }
static inline long long ncells(const NodalGeom& g) { return (long long)g.n[0] * g.n[1] * g.n[2]; }

static const dim3 kBlock3(32, 4, 2);
static inline dim3 grid3c(const NodalGeom& g)
{
    return dim3((g.n[0] + 31) / 32, (g.n[1] + 3) / 4, (g.n[2] + 1) / 2);
}
static inline dim3 grid3(const NodalGeom& g)
{
    return dim3((g.nu[0] + 31) / 32, (g.nu[1] + 3) / 4, (g.nu[2] + 1) / 2);
}

template <typename T>
void nodal_jacobi(const NodalGeom& g, const T* s, const T* xin, const T* b, T* xout, double omega, bool zero,
                  cudaStream_t st)
{
    if (zero) {
        k_jacobi<T, true, true><<<grid3(g), kBlock3, 0, st>>>(g, s, xin, b, xout, (T)omega);
    } else if (g.iso) {
        k_jacobi<T, true, false><<<grid3(g), kBlock3, 0, st>>>(g, s, xin, b, xout, (T)omega);
    } else {
        k_jacobi<T, false, false><<<grid3(g), kBlock3, 0, st>>>(g, s, xin, b, xout, (T)omega);
    }
}

template <typename T>
void nodal_resid(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, unsigned long long* norm,
                 cudaStream_t st)
{
    if (g.iso)
        k_resid<T, true><<<grid3(g), kBlock3, 0, st>>>(g, s, x, b, r, norm);
    else
        k_resid<T, false><<<grid3(g), kBlock3, 0, st>>>(g, s, x, b, r, norm);
}

template <typename T>
void nodal_resid_list(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, const int4* nodes, int n,
                      cudaStream_t st)
{
    if (n <= 0) return;
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (g.iso)
        k_resid_list<T, true><<<nb, 256, 0, st>>>(g, s, x, b, r, nodes, n);
    else
        k_resid_list<T, false><<<nb, 256, 0, st>>>(g, s, x, b, r, nodes, n);
}
template void nodal_resid_list<float>(const NodalGeom&, const float*, const float*, const float*, float*, const int4*,
                                      int, cudaStream_t);

template <typename T>
void nodal_restrict(const NodalGeom& gf, const NodalGeom& gc, const T* rf, T* bc, cudaStream_t st)
{
    k_restrict<T><<<grid3(gc), kBlock3, 0, st>>>(gf, gc, rf, bc);
}

template <typename T>
void nodal_prolong_add(const NodalGeom& gf, const NodalGeom& gc, const T* xc, T* xf, cudaStream_t st)
{
    k_prolong_block<T><<<grid3(gc), kBlock3, 0, st>>>(gf, gc, xc, xf);
}

template <typename T>
void nodal_bottom(const NodalGeom& g, const double* s64, const T* b, T* x, double* scratch, int maxiter,
                  double rtol, double atol, int* info, int singular, cudaStream_t st)
{
    k_bottom_cg<T><<<1, 1024, 0, st>>>(g, s64, b, x, scratch, maxiter, rtol, atol, info, singular);
}

template void nodal_jacobi<double>(const NodalGeom&, const double*, const double*, const double*, double*, double,
                                   bool, cudaStream_t);
template void nodal_jacobi<float>(const NodalGeom&, const float*, const float*, const float*, float*, double, bool,
                                  cudaStream_t);
template void nodal_resid<double>(const NodalGeom&, const double*, const double*, const double*, double*,
                                  unsigned long long*, cudaStream_t);
template void nodal_resid<float>(const NodalGeom&, const float*, const float*, const float*, float*,
                                 unsigned long long*, cudaStream_t);
template void nodal_restrict<double>(const NodalGeom&, const NodalGeom&, const double*, double*, cudaStream_t);
template void nodal_restrict<float>(const NodalGeom&, const NodalGeom&, const float*, float*, cudaStream_t);
template void nodal_prolong_add<double>(const NodalGeom&, const NodalGeom&, const double*, double*, cudaStream_t);
template void nodal_prolong_add<float>(const NodalGeom&, const NodalGeom&, const float*, float*, cudaStream_t);
template void nodal_bottom<double>(const NodalGeom&, const double*, const double*, double*, double*, int, double,
                                   double, int*, int, cudaStream_t);
template void nodal_bottom<float>(const NodalGeom&, const double*, const float*, float*, double*, int, double,
                                  double, int*, int, cudaStream_t);

void nodal_sigma_from_rho(const NodalGeom& g, const gbp_array4* rho, double scale, double rho0, double* s64,
                          float* s32, cudaStream_t st)
{
    gbp_array4 r{};
    if (rho) r = *rho;
    k_sigma_from_rho<<<grid3c(g), kBlock3, 0, st>>>(g, r, rho != nullptr, scale, rho0, s64, s32);
}

void nodal_sigma_copy(const NodalGeom& g, const gbp_array4* sig, double cval, double* s64, float* s32,
                      cudaStream_t st)
{
    gbp_array4 r{};
    if (sig) r = *sig;
    k_sigma_copy<<<grid3c(g), kBlock3, 0, st>>>(g, r, sig != nullptr, cval, s64, s32);
}

void nodal_sigma_coarsen(const NodalGeom& gf, const NodalGeom& gc, const double* sf, double* sc64, float* sc32,
                         cudaStream_t st)
{
    k_sigma_coarsen<<<nblocks(ncells(gc), 256), 256, 0, st>>>(gf, gc, sf, sc64, sc32);
}

static dim3 rhs_grid(const NodalGeom& g, int& kchunk)
{
    const int bx = (g.nu[0] + ZX - 1) / ZX, by = (g.nu[1] + ZY - 1) / ZY;
    kchunk = zchunk(bx, by, g.nu[2]);
    return dim3(bx, by, (g.nu[2] + kchunk - 1) / kchunk);
}

void nodal_rhs(const NodalGeom& g, const RhsArgs& a, const double* s64, double* b, double* part, cudaStream_t st,
               int zb0, int zb1)
{
    int kchunk;
    const dim3 grid = rhs_grid(g, kchunk);
    if (zb1 < 0) zb1 = (int)grid.z;
    if (zb1 <= zb0) return;
    k_nodal_rhs<<<dim3(grid.x, grid.y, zb1 - zb0), ZTX * ZTY, 0, st>>>(g, a, s64, b, part, kchunk, zb0, (int)grid.z);
}

int nodal_rhs_zchunks(const NodalGeom& g, int* kchunk)
{
    int kc;
    const dim3 grid = rhs_grid(g, kc);
    if (kchunk) *kchunk = kc;
    return (int)grid.z;
}

int nodal_rhs_partials(const NodalGeom& g)
{
    int kchunk;
    const dim3 grid = rhs_grid(g, kchunk);
    return (int)(grid.x * grid.y * grid.z);
}

// node-column launches (block 32 x 8, z chunks) with at most `cap` blocks
static dim3 column_grid(const NodalGeom& g, int cap, int& kchunk)
{
    const int bx = (g.nu[0] + 31) / 32, by = (g.nu[1] + 7) / 8;
    int gz = std::max(1, std::min(cap / std::max(1, bx * by), (g.nu[2] + 7) / 8));
    kchunk = (g.nu[2] + gz - 1) / gz;
    gz = (g.nu[2] + kchunk - 1) / kchunk;
    return dim3(bx, by, gz);
}

static inline unsigned stride_blocks(long long n) { return (unsigned)std::min<long long>(nblocks(n, 256), 1184); }

static double domain_volume(const NodalGeom& g)
{
    return (double)g.n[0] * g.h[0] * (double)g.n[1] * g.h[1] * (double)g.n[2] * g.h[2];
}

// fold `nparts` partial sums into scal = sum / domain volume
void nodal_fold(const NodalGeom& g, const double* part, int nparts, double* scal, cudaStream_t st)
{
    k_fold<<<1, 1024, 0, st>>>(part, nparts, domain_volume(g), scal);
}

void nodal_remove_mean(const NodalGeom& g, double* v, double* partials, double* scal, int mode, int have_partials,
                       int nparts, unsigned long long* norm, cudaStream_t st)
{
    const int cap = nodal_partials_needed(g);
    int kchunk;
    const dim3 grid = column_grid(g, cap, kchunk);
    if (!have_partials) {
        k_node_sums<<<grid, dim3(32, 8), 0, st>>>(g, v, mode == 1, partials, kchunk);
        nparts = (int)(grid.x * grid.y * grid.z);
    }
    k_fold<<<1, 1024, 0, st>>>(partials, nparts, domain_volume(g), scal);
    k_remove_mean<<<grid, dim3(32, 8), 0, st>>>(g, v, scal, mode, norm, kchunk);
}

void nodal_norm(const NodalGeom& g, const double* v, unsigned long long* norm, cudaStream_t st)
{
    k_node_norm<<<stride_blocks(nunique(g)), 256, 0, st>>>(g, v, norm);
}

int nodal_partials_needed(const NodalGeom& g) { return std::max(nodal_rhs_partials(g), 1184); }

template <typename TE>
void nodal_add_correction(const NodalGeom& g, double* x, const TE* e, double inv_scale, cudaStream_t st)
{
    k_add_correction<TE><<<grid3(g), kBlock3, 0, st>>>(g, x, e, inv_scale);
}
template void nodal_add_correction<double>(const NodalGeom&, double*, const double*, double, cudaStream_t);
template void nodal_add_correction<float>(const NodalGeom&, double*, const float*, double, cudaStream_t);

void nodal_to_f32(const NodalGeom& g, const double* r, float* r32, double scale, cudaStream_t st)
{
    k_to_f32<<<grid3(g), kBlock3, 0, st>>>(g, r, r32, scale);
}

void nodal_correct(const NodalGeom& g, const CorrArgs& a, const double* s64, const double* phi, cudaStream_t st,
                   int k0, int k1)
{
    if (k1 < 0) k1 = g.n[2];
    if (k1 <= k0) return;
    const int bx = (g.n[0] + ZX - 1) / ZX, by = (g.n[1] + ZY - 1) / ZY;
    const int kchunk = zchunk(bx, by, k1 - k0);
    k_nodal_correct<<<dim3(bx, by, (k1 - k0 + kchunk - 1) / kchunk), ZTX * ZTY, 0, st>>>(g, a, s64, phi, kchunk, k0,
                                                                                         k1);
}

void nodal_store_phi(const NodalGeom& g, const gbp_array4& out, const double* phi, int accumulate, cudaStream_t st)
{
    k_nodal_store_phi<<<dim3((g.n[0] + 32) / 32, (g.n[1] + 4) / 4, (g.n[2] + 2) / 2), kBlock3, 0, st>>>(g, out, phi,
                                                                                                   accumulate);
}

void nodal_load_phi(const NodalGeom& g, const gbp_array4& in, double* phi, cudaStream_t st)
{
    k_nodal_load_phi<<<grid3(g), kBlock3, 0, st>>>(g, in, phi);
}

void nodal_mask_load(const NodalGeom& g, const gbp_iarray4& m, unsigned char* out, unsigned* zeros, cudaStream_t st)
{
    k_mask_load<<<grid3(g), kBlock3, 0, st>>>(g, m, out, zeros);
}

void nodal_mask_coarsen(const NodalGeom& gf, const NodalGeom& gc, const unsigned char* mf, unsigned char* mc,
                        cudaStream_t st)
{
    k_mask_coarsen<<<grid3(gc), kBlock3, 0, st>>>(gf, gc, mf, mc);
}

}  // namespace gbp
