// MAC (cell-centred) projection kernels: the 7-point flux-form operator div(beta grad phi) with
// face beta, red-black Gauss-Seidel smoother, residual, restriction (sum of the 8 fine weak-form
// residuals), piecewise-constant prolongation, single-CTA bottom CG, and the right-hand side /
// correction kernels of Hydro::MacProjector as driven by incflo
// (src/convection/incflo_compute_MAC_projected_velocities.cpp:69-133, 272-299).
//
// Weak form per cell (volume V): (A phi)_c = sum_faces w_d beta_f (phi_c - phi_nbr), w_d = V/h_d^2.
// Boundary faces carry an effective beta: 0 on Neumann/inflow faces (no flux), 2*beta on
// Dirichlet faces with a zero ghost (phi = 0 on the face, linear through the first cell).
// The right-hand side is g = -V div(umac), the correction umac -= beta_eff grad phi.
#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "mac_kernels.h"

namespace gbp {

__device__ __forceinline__ bool decode_cell(const CellGeom& g, long long t, int& i, int& j, int& k)
{
    const long long nxy = (long long)g.n[0] * g.n[1];
    const long long n = nxy * g.n[2];
    if (t >= n) return false;
    if (n <= 0xffffffffll) {
        // 32-bit unsigned division (a 64-bit one is emulated in far more instructions)
        const unsigned u = (unsigned)t, nx = (unsigned)g.n[0], nxy32 = (unsigned)nxy;
        const unsigned kk = u / nxy32, r = u - kk * nxy32, jj = r / nx;
        k = (int)kk;
        j = (int)jj;
        i = (int)(r - jj * nx);
        return true;
    }
    k = (int)(t / nxy);
    long long r = t - (long long)k * nxy;
    j = (int)(r / g.n[0]);
    i = (int)(r - (long long)j * g.n[0]);
    return true;
}

// face (f0, f1, f2) of linear index t over extents fn (faces of one direction), as decode_cell
__device__ __forceinline__ bool decode_face(const int fn[3], long long t, int f[3])
{
    const long long nxy = (long long)fn[0] * fn[1];
    const long long n = nxy * fn[2];
    if (t >= n) return false;
    if (n <= 0xffffffffll) {
        const unsigned u = (unsigned)t, nx = (unsigned)fn[0], nxy32 = (unsigned)nxy;
        const unsigned kk = u / nxy32, r = u - kk * nxy32, jj = r / nx;
        f[2] = (int)kk;
        f[1] = (int)jj;
        f[0] = (int)(r - jj * nx);
        return true;
    }
    f[2] = (int)(t / nxy);
    const long long rem = t - (long long)f[2] * nxy;
    f[1] = (int)(rem / fn[0]);
    f[0] = (int)(rem - (long long)f[1] * fn[0]);
    return true;
}

template <typename T>
__device__ __forceinline__ const T* mac_acoef(const CellGeom& g);
template <>
__device__ __forceinline__ const double* mac_acoef<double>(const CellGeom& g) { return g.a64; }
template <>
__device__ __forceinline__ const float* mac_acoef<float>(const CellGeom& g) { return g.a32; }

// Loads of the operator: plain (the per-level kernels) or L2-coherent (the cluster kernel, whose CTAs read
// what other CTAs wrote before a cluster barrier)
struct MacLdPlain {
    template <typename T>
    __device__ __forceinline__ static T ld(const T* p) { return *p; }
};
struct MacLdCg {
    __device__ __forceinline__ static float ld(const float* p) { return __ldcg(p); }
    __device__ __forceinline__ static double ld(const double* p) { return __ldcg(p); }
};

// (A x)_p = sum over faces of w beta (x_p - x_nb) [+ alpha a V x_p]; diag and the neighbour sum for
// the Gauss-Seidel update x_p = (b_p + offsum) / diag
template <typename T, typename LD = MacLdPlain>
__device__ __forceinline__ T mac_Ax(const CellGeom& g, const T* __restrict__ x, const T* __restrict__ bx,
                                    const T* __restrict__ by, const T* __restrict__ bz, long long p, T& diag,
                                    T& offsum)
{
    const T xc = LD::ld(x + p);
    const T wx = (T)g.w[0], wy = (T)g.w[1], wz = (T)g.w[2];
    const T b0 = bx[p] * wx, b1 = bx[p + 1] * wx;
    const T b2 = by[p] * wy, b3 = by[p + g.sy] * wy;
    const T b4 = bz[p] * wz, b5 = bz[p + g.sz] * wz;
    const T xw = LD::ld(x + p - 1), xe = LD::ld(x + p + 1), xs = LD::ld(x + p - g.sy), xn = LD::ld(x + p + g.sy);
    const T xb = LD::ld(x + p - g.sz), xt = LD::ld(x + p + g.sz);
    diag = ((b0 + b1) + (b2 + b3)) + (b4 + b5);
    offsum = ((b0 * xw + b1 * xe) + (b2 * xs + b3 * xn)) + (b4 * xb + b5 * xt);
    T ax = ((b0 * (xc - xw) + b1 * (xc - xe)) + (b2 * (xc - xs) + b3 * (xc - xn))) + (b4 * (xc - xb) + b5 * (xc - xt));
    const T* ac = mac_acoef<T>(g);
    if (ac) {
        diag += ac[p];
        ax += ac[p] * xc;
    }
    return ax;
}

template <typename T>
__global__ void __launch_bounds__(256) k_mac_rbgs(CellGeom g, const T* __restrict__ bx, const T* __restrict__ by,
                                                  const T* __restrict__ bz, const T* __restrict__ b, T* x, int color)
{
    // thread t handles the t-th cell of this colour along x
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int hx = (g.n[0] + 1) / 2;
    const long long rows = (long long)g.n[1] * g.n[2];
    if (t >= rows * hx) return;
    int i, j, k;
    if (rows * hx <= 0xffffffffll) {
        // 32-bit unsigned division (a 64-bit one is emulated in far more instructions)
        const unsigned u = (unsigned)t, row = u / (unsigned)hx, kk = row / (unsigned)g.n[1];
        k = (int)kk;
        j = (int)(row - kk * (unsigned)g.n[1]);
        i = 2 * (int)(u - row * (unsigned)hx) + ((j + k + color) & 1);
    } else {
        const long long row = t / hx;
        k = (int)(row / g.n[1]);
        j = (int)(row - (long long)k * g.n[1]);
        i = 2 * (int)(t - row * hx) + ((j + k + color) & 1);
    }
    if (i >= g.n[0]) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    T diag, off;
    (void)mac_Ax<T>(g, x, bx, by, bz, p, diag, off);
    const T v = diag != T(0) ? (b[p] + off) / diag : T(0);
    store_cell(x, g, i, j, k, v);
}

template <typename T>
__global__ void __launch_bounds__(256) k_mac_resid(CellGeom g, const T* __restrict__ bx, const T* __restrict__ by,
                                                   const T* __restrict__ bz, const T* __restrict__ x,
                                                   const T* __restrict__ b, T* __restrict__ r,
                                                   unsigned long long* norm)
{
    int i, j, k;
    double nv = 0.0;
    if (decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
        T diag, off;
        const T v = b[p] - mac_Ax<T>(g, x, bx, by, bz, p, diag, off);
        r[p] = v;
        if (norm) nv = fabs((double)v) / g.vol;
    }
    if (norm) {
        nv = block_max(nv);
        if (threadIdx.x == 0) atomic_max_nonneg(norm, nv);
    }
}

// The FP64 residual (outer refinement steps, plain-form V-cycles): one face weight multiplication per
// direction instead of per face, and the max norm as an integer key of |r| scaled by 1 / V once per
// block (no FP64 division per cell). FP64 instructions bound it.
template <>
__global__ void __launch_bounds__(256) k_mac_resid<double>(CellGeom g, const double* __restrict__ bx,
                                                           const double* __restrict__ by, const double* __restrict__ bz,
                                                           const double* __restrict__ x, const double* __restrict__ b,
                                                           double* __restrict__ r, unsigned long long* norm)
{
    int i, j, k;
    unsigned long long key = 0;
    if (decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
        const double xc = x[p];
        const double dx = fma(bx[p], xc - x[p - 1], bx[p + 1] * (xc - x[p + 1]));
        const double dy = fma(by[p], xc - x[p - g.sy], by[p + g.sy] * (xc - x[p + g.sy]));
        const double dz = fma(bz[p], xc - x[p - g.sz], bz[p + g.sz] * (xc - x[p + g.sz]));
        double ax = fma(g.w[0], dx, fma(g.w[1], dy, g.w[2] * dz));
        if (g.a64) ax = fma(g.a64[p], xc, ax);
        const double v = b[p] - ax;
        r[p] = v;
        key = abs_key(v);
    }
    if (norm) {
        key = block_max_key(key);
        if (threadIdx.x == 0) atomic_max_nonneg(norm, key_value(key) * (1.0 / g.vol));
    }
}

template <typename T>
__global__ void k_mac_restrict(CellGeom gf, CellGeom gc, const T* __restrict__ rf, T* __restrict__ bc)
{
    int I, J, K;
    if (!decode_cell(gc, blockIdx.x * (long long)blockDim.x + threadIdx.x, I, J, K)) return;
    const long long f = pidx(gf.sy, gf.sz, 2 * I, 2 * J, 2 * K);
    const T v = ((rf[f] + rf[f + 1]) + (rf[f + gf.sy] + rf[f + 1 + gf.sy])) +
                ((rf[f + gf.sz] + rf[f + 1 + gf.sz]) + (rf[f + gf.sy + gf.sz] + rf[f + 1 + gf.sy + gf.sz]));
    bc[pidx(gc.sy, gc.sz, I, J, K)] = v;
}

template <typename T>
__global__ void k_mac_prolong_add(CellGeom gf, CellGeom gc, const T* __restrict__ xc, T* __restrict__ xf)
{
    int i, j, k;
    if (!decode_cell(gf, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const long long p = pidx(gf.sy, gf.sz, i, j, k);
    store_cell(xf, gf, i, j, k, xf[p] + xc[pidx(gc.sy, gc.sz, i >> 1, j >> 1, k >> 1)]);
}

__device__ __forceinline__ double mac_block_sum(double v, double*) { return block_sum_all(v); }

// Jacobi-preconditioned CG in FP64 on the coarsest level, one CTA.
template <typename T>
__global__ void __launch_bounds__(1024) k_mac_bottom(CellGeom g, const double* __restrict__ bx,
                                                     const double* __restrict__ by, const double* __restrict__ bz,
                                                     const T* __restrict__ bin, T* __restrict__ xout,
                                                     double* __restrict__ scr, int maxiter, double rtol,
                                                     double atol, int singular)
{
    __shared__ double red[32];
    const long long P = g.count;
    double* x = scr;
    double* r = scr + P;
    double* p = scr + 2 * P;
    double* q = scr + 3 * P;
    double* dg = scr + 4 * P;
    const long long N = (long long)g.n[0] * g.n[1] * g.n[2];
    for (long long t = threadIdx.x; t < 5 * P; t += blockDim.x) scr[t] = 0.0;
    __syncthreads();
    double bs = 0.0, nf = 0.0;
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_cell(g, t, i, j, k);
        const long long c = pidx(g.sy, g.sz, i, j, k);
        const double bv = (double)bin[c];
        r[c] = bv;
        double d, off;
        (void)mac_Ax<double>(g, x, bx, by, bz, c, d, off);
        dg[c] = d;
        if (d != 0.0) {  // cells fully covered by an embedded boundary have no equation
            bs += bv;
            nf += 1.0;
        }
    }
    if (singular) {
        bs = mac_block_sum(bs, red);
        nf = mac_block_sum(nf, red);
        const double mean = nf > 0.0 ? bs / nf : 0.0;
        __syncthreads();
        for (long long t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_cell(g, t, i, j, k);
            const long long c = pidx(g.sy, g.sz, i, j, k);
            r[c] = dg[c] != 0.0 ? r[c] - mean : 0.0;
        }
    }
    __syncthreads();
    double rz = 0.0, rr = 0.0;
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_cell(g, t, i, j, k);
        const long long c = pidx(g.sy, g.sz, i, j, k);
        const double z = dg[c] != 0.0 ? r[c] / dg[c] : 0.0;
        store_cell(p, g, i, j, k, z);
        rz += r[c] * z;
        rr += r[c] * r[c];
    }
    rz = mac_block_sum(rz, red);
    rr = mac_block_sum(rr, red);
    const double r0 = sqrt(rr);
    const double target = fmax(rtol * r0, atol > 0 ? atol : 0.0);
    if (r0 > 0.0) {
        for (int it = 1; it <= maxiter; ++it) {
            __syncthreads();
            double pq = 0.0;
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_cell(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                double d, off;
                const double v = mac_Ax<double>(g, p, bx, by, bz, c, d, off);
                q[c] = v;
                pq += p[c] * v;
            }
            pq = mac_block_sum(pq, red);
            if (!(pq > 0.0)) break;
            const double alpha = rz / pq;
            double rz2 = 0.0;
            rr = 0.0;
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_cell(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                x[c] += alpha * p[c];
                r[c] -= alpha * q[c];
                const double z = dg[c] != 0.0 ? r[c] / dg[c] : 0.0;
                q[c] = z;
                rz2 += r[c] * z;
                rr += r[c] * r[c];
            }
            rz2 = mac_block_sum(rz2, red);
            rr = mac_block_sum(rr, red);
            if (sqrt(rr) <= target) break;
            const double beta = rz2 / rz;
            rz = rz2;
            __syncthreads();
            for (long long t = threadIdx.x; t < N; t += blockDim.x) {
                int i, j, k;
                decode_cell(g, t, i, j, k);
                const long long c = pidx(g.sy, g.sz, i, j, k);
                store_cell(p, g, i, j, k, q[c] + beta * p[c]);
            }
        }
    }
    __syncthreads();
    for (long long t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_cell(g, t, i, j, k);
        store_cell(xout, g, i, j, k, (T)x[pidx(g.sy, g.sz, i, j, k)]);
    }
}

// ------------------------------------------------------------------ level-0 set-up kernels
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

// Effective face beta of direction d for faces 0..n[d]: source 0 = array, 1 = constant,
// 2 = dt / (0.5 (rho_lo + rho_hi)) (incflo: average_cellcenter_to_face then invert(dt)).
__global__ void k_mac_beta(CellGeom g, int d, int source, gbp_array4 src, double cval, int bclo, int bchi,
                           double* __restrict__ b64, float* __restrict__ b32, RobinFaces rb,
                           const double* __restrict__ ap, double mult)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    fn[d] += 1;
    int f[3];
    if (!decode_face(fn, t, f)) return;
    const int fd = f[d];
    const bool per = g.per[d];
    const long long p = pidx(g.sy, g.sz, f[0], f[1], f[2]);
    const int bside = fd == 0 ? bclo : bchi;
    if (!per && (fd == 0 || fd == g.n[d]) && bside != GBP_BC_DIRICHLET && bside != GBP_BC_ROBIN) {
        // wall / inflow face: no flux through it, and no ghost value is read
        b64[p] = 0.0;
        b32[p] = 0.f;
        return;
    }
    double beta;
    int q[3] = {f[0], f[1], f[2]};
    if (per && fd == g.n[d]) q[d] = 0;  // face n is face 0
    if (source == 0) {
        beta = a4(src, q[0], q[1], q[2], 0);
    } else if (source == 1) {
        beta = cval;
    } else if (source == 3) {
        // face average of a cell field (amrex::average_cellcenter_to_face), the adjacent cell on a
        // non-periodic domain side (incflo::fixup_eta_on_domain_faces)
        int lo[3] = {q[0], q[1], q[2]};
        lo[d] -= 1;
        if (per && lo[d] < 0) lo[d] += g.n[d];
        if (!per && fd == 0)
            beta = a4(src, q[0], q[1], q[2], 0);
        else if (!per && fd == g.n[d])
            beta = a4(src, lo[0], lo[1], lo[2], 0);
        else
            beta = 0.5 * (a4(src, lo[0], lo[1], lo[2], 0) + a4(src, q[0], q[1], q[2], 0));
    } else {
        int lo[3] = {q[0], q[1], q[2]};
        lo[d] -= 1;
        if (per && lo[d] < 0) lo[d] += g.n[d];
        beta = cval / (0.5 * (a4(src, lo[0], lo[1], lo[2], 0) + a4(src, q[0], q[1], q[2], 0)));
    }
    beta *= mult;  // the ABecLaplacian's beta scalar times b (1 for the projections)
    // Dirichlet face: the ghost value sits half a cell out, so the face weight doubles; Robin face
    // (a phi + b dphi/dn = 0): weight beta a h / (a h / 2 + b), with the raw beta kept for later factors
    double eff = beta;
    if (!per && (fd == 0 || fd == g.n[d])) {
        if (bside == GBP_BC_ROBIN) {
            const int q = 2 * d + (fd == 0 ? 0 : 1);
            const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
            const long long fi = f[d1] + (long long)g.n[d1] * f[d2];
            rb.braw[q][fi] = beta;
            eff = beta * rb.rfac[q][fi];
        } else {
            eff = 2.0 * beta;
        }
    }
    if (ap) eff = ap[p] > 0.0 ? eff * ap[p] : 0.0;  // cut cells: the open fraction scales the flux
    b64[p] = eff;
    b32[p] = (float)eff;
}

__global__ void k_mac_beta_coarsen(CellGeom gf, CellGeom gc, int d, const double* __restrict__ bf,
                                   double* __restrict__ bc64, float* __restrict__ bc32)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {gc.n[0], gc.n[1], gc.n[2]};
    fn[d] += 1;
    int f[3];
    if (!decode_face(fn, t, f)) return;
    const long long base = pidx(gf.sy, gf.sz, 2 * f[0], 2 * f[1], 2 * f[2]);
    const long long s1 = d == 0 ? gf.sy : 1;
    const long long s2 = d == 2 ? gf.sy : gf.sz;
    const double v = 0.25 * ((bf[base] + bf[base + s1]) + (bf[base + s2] + bf[base + s1 + s2]));
    const long long p = pidx(gc.sy, gc.sz, f[0], f[1], f[2]);
    bc64[p] = v;
    bc32[p] = (float)v;
}

__global__ void __launch_bounds__(256) k_mac_rhs(CellGeom g, gbp_array4 ux, gbp_array4 uy, gbp_array4 uz,
                                                 double* __restrict__ b, MacEB eb)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const int ip = (g.per[0] && i + 1 == g.n[0]) ? 0 : i + 1;
    const int jp = (g.per[1] && j + 1 == g.n[1]) ? 0 : j + 1;
    const int kp = (g.per[2] && k + 1 == g.n[2]) ? 0 : k + 1;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    double fx0 = a4(ux, i, j, k, 0), fx1 = a4(ux, ip, j, k, 0);
    double fy0 = a4(uy, i, j, k, 0), fy1 = a4(uy, i, jp, k, 0);
    double fz0 = a4(uz, i, j, k, 0), fz1 = a4(uz, i, j, kp, 0);
    if (eb.ap[0]) {
        // cut cells: fluxes through the open part of each face only (no flow through the EB)
        fx0 *= eb.ap[0][p];
        fx1 *= eb.ap[0][p + 1];
        fy0 *= eb.ap[1][p];
        fy1 *= eb.ap[1][p + g.sy];
        fz0 *= eb.ap[2][p];
        fz1 *= eb.ap[2][p + g.sz];
    }
    const double dv = (fx1 - fx0) * g.ih[0] + (fy1 - fy0) * g.ih[1] + (fz1 - fz0) * g.ih[2];
    b[p] = -g.vol * dv - (eb.ebflux ? eb.ebflux[p] : 0.0);
}

__global__ void __launch_bounds__(256) k_mac_eb_inflow_flux(CellGeom g, gbp_array4 ev, MacEB eb,
                                                            double* __restrict__ flux)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    double f = 0.0;
    if (eb.kap[p] > 0.0) {
        f = a4(ev, i, j, k, 0) * (eb.ap[0][p] - eb.ap[0][p + 1]) * (g.vol / g.h[0]) +
            a4(ev, i, j, k, 1) * (eb.ap[1][p] - eb.ap[1][p + g.sy]) * (g.vol / g.h[1]) +
            a4(ev, i, j, k, 2) * (eb.ap[2][p] - eb.ap[2][p + g.sz]) * (g.vol / g.h[2]);
    }
    flux[p] = f;
}

__global__ void __launch_bounds__(256) k_mac_correct(CellGeom g, int d, gbp_array4 u, const double* __restrict__ beta,
                                                     const double* __restrict__ phi, const double* __restrict__ ap)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    fn[d] += 1;
    int f[3];
    if (!decode_face(fn, t, f)) return;
    const long long p = pidx(g.sy, g.sz, f[0], f[1], f[2]);
    const long long s = d == 0 ? 1 : (d == 1 ? g.sy : g.sz);
    double be = beta[p];
    if (be == 0.0) return;
    if (ap) be /= ap[p];  // beta here is ap x beta (be != 0 implies ap > 0)
    double* up = a4p(u, f[0], f[1], f[2], 0);
    *up -= be * (phi[p] - phi[p - s]) * g.ih[d];
}

// zero the faces 0..n (direction d) of a caller face array
__global__ void __launch_bounds__(256) k_mac_zero_faces(CellGeom g, int d, gbp_array4 u)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    fn[d] += 1;
    const long long nxy = (long long)fn[0] * fn[1];
    if (t >= nxy * fn[2]) return;
    const int k = (int)(t / nxy);
    const long long rem = t - (long long)k * nxy;
    const int j = (int)(rem / fn[0]);
    const int i = (int)(rem - (long long)j * fn[0]);
    *a4p(u, i, j, k, 0) = 0.0;
}

__global__ void k_mac_load_phi(CellGeom g, gbp_array4 in, double* __restrict__ phi)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    store_cell(phi, g, i, j, k, a4(in, i, j, k, 0));
}

__global__ void k_mac_store_phi(CellGeom g, gbp_array4 out, const double* __restrict__ phi)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    *a4p(out, i, j, k, 0) = phi[pidx(g.sy, g.sz, i, j, k)];
}

__global__ void __launch_bounds__(256) k_mac_norm(CellGeom g, const double* __restrict__ v, unsigned long long* norm,
                                                  const double* __restrict__ kap)
{
    int i, j, k;
    if (!kap) {
        // max |v| / V: an integer key of |v| per cell, one multiplication by 1 / V per block
        unsigned long long key = 0;
        if (decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k))
            key = abs_key(v[pidx(g.sy, g.sz, i, j, k)]);
        key = block_max_key(key);
        if (threadIdx.x == 0) atomic_max_nonneg(norm, key_value(key) * (1.0 / g.vol));
        return;
    }
    double nv = 0.0;
    if (decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) {
        const long long p = pidx(g.sy, g.sz, i, j, k);
        if (kap[p] > 0.0) nv = fabs(v[p]) / (kap[p] * g.vol);  // the cut-cell operator divides by the volume fraction
    }
    nv = block_max(nv);
    if (threadIdx.x == 0) atomic_max_nonneg(norm, nv);
}

// per-block sums of v (kap != null and weighted: of kap * v): each thread sums its cells of a grid-stride
// walk in a fixed order, then a fixed block tree (the grid size is fixed by the host: deterministic)
__global__ void k_mac_sums(CellGeom g, const double* __restrict__ v, double* __restrict__ part,
                           const double* __restrict__ kap, int weighted)
{
    __shared__ double red[32];
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (!decode_cell(g, t, i, j, k)) break;
        const long long p = pidx(g.sy, g.sz, i, j, k);
        acc += (kap && weighted) ? kap[p] * v[p] : v[p];
    }
    acc = mac_block_sum(acc, red);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// part[nparts] = (sum of the nparts block sums) / nfluid, by one block in a fixed order
__global__ void k_mac_fold(double* __restrict__ part, int nparts, double nfluid)
{
    __shared__ double red[32];
    double acc = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x) acc += part[t];
    acc = mac_block_sum(acc, red);
    if (threadIdx.x == 0) part[nparts] = acc / nfluid;
}

// mode 0: b_c -= kappa_c sum(b) / sum(kappa), so that sum(b) = 0 (the range of the operator);
// mode 1: x -= its volume-weighted mean, with periodic aliases, and 0 in covered cells. Without cut
// cells kappa = 1 and nfluid = the cell count.
__global__ void k_mac_remove_mean(CellGeom g, double* __restrict__ v, const double* __restrict__ part, int nparts,
                                  int mode, const double* __restrict__ kap)
{
    const double c = part[nparts];  // the mean (k_mac_fold)
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;; t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (!decode_cell(g, t, i, j, k)) break;
        const long long p = pidx(g.sy, g.sz, i, j, k);
        const double kc = kap ? kap[p] : 1.0;
        if (mode == 0)
            v[p] -= c * kc;
        else
            store_cell(v, g, i, j, k, kc > 0.0 ? v[p] - c : 0.0);
    }
}

template <typename TE>
__global__ void k_mac_add_correction(CellGeom g, double* __restrict__ x, const TE* __restrict__ e, double inv_scale)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    store_cell(x, g, i, j, k, x[p] + (double)e[p] * inv_scale);
}

__global__ void k_mac_to_f32(CellGeom g, const double* __restrict__ r, float* __restrict__ r32, double scale)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    r32[p] = (float)(r[p] * scale);
}

// ------------------------------------------------------------------------------ launchers
static inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }
static inline long long ncell(const CellGeom& g) { return (long long)g.n[0] * g.n[1] * g.n[2]; }
static inline long long nface(const CellGeom& g, int d)
{
    long long v = 1;
    for (int e = 0; e < 3; ++e) v *= g.n[e] + (e == d);
    return v;
}

template <typename T>
void mac_rbgs(const CellGeom& g, const T* bx, const T* by, const T* bz, const T* b, T* x, int color, cudaStream_t st)
{
    const long long n = (long long)g.n[1] * g.n[2] * ((g.n[0] + 1) / 2);
    k_mac_rbgs<T><<<nblk(n, 256), 256, 0, st>>>(g, bx, by, bz, b, x, color);
}
template <typename T>
void mac_resid(const CellGeom& g, const T* bx, const T* by, const T* bz, const T* x, const T* b, T* r,
               unsigned long long* norm, cudaStream_t st)
{
    k_mac_resid<T><<<nblk(ncell(g), 256), 256, 0, st>>>(g, bx, by, bz, x, b, r, norm);
}
template <typename T>
void mac_restrict(const CellGeom& gf, const CellGeom& gc, const T* rf, T* bc, cudaStream_t st)
{
    k_mac_restrict<T><<<nblk(ncell(gc), 256), 256, 0, st>>>(gf, gc, rf, bc);
}
template <typename T>
void mac_prolong_add(const CellGeom& gf, const CellGeom& gc, const T* xc, T* xf, cudaStream_t st)
{
    k_mac_prolong_add<T><<<nblk(ncell(gf), 256), 256, 0, st>>>(gf, gc, xc, xf);
}
template <typename T>
void mac_bottom(const CellGeom& g, const double* bx, const double* by, const double* bz, const T* b, T* x,
                double* scratch, int maxiter, double rtol, double atol, int singular, cudaStream_t st)
{
    k_mac_bottom<T><<<1, 1024, 0, st>>>(g, bx, by, bz, b, x, scratch, maxiter, rtol, atol, singular);
}

#define GBP_MAC_INST(T)                                                                                        \
    template void mac_rbgs<T>(const CellGeom&, const T*, const T*, const T*, const T*, T*, int, cudaStream_t); \
    template void mac_resid<T>(const CellGeom&, const T*, const T*, const T*, const T*, const T*, T*,          \
                               unsigned long long*, cudaStream_t);                                            \
    template void mac_restrict<T>(const CellGeom&, const CellGeom&, const T*, T*, cudaStream_t);              \
    template void mac_prolong_add<T>(const CellGeom&, const CellGeom&, const T*, T*, cudaStream_t);           \
    template void mac_bottom<T>(const CellGeom&, const double*, const double*, const double*, const T*, T*,   \
                                double*, int, double, double, int, cudaStream_t);
GBP_MAC_INST(double)
GBP_MAC_INST(float)

// Dense bottom solve: x = M b with M the FP64 inverse of the coarsest operator, precomputed on the host
// whenever the face coefficients change (singular systems: the inverse of A + c 1 1^T over the cells
// that carry an equation, exact for a right-hand side of zero mean over them). One CTA; N <= 128.
template <typename T>
__global__ void __launch_bounds__(128) k_mac_bottom_dense(CellGeom g, const double* __restrict__ M,
                                                          const unsigned char* __restrict__ act,
                                                          const T* __restrict__ bin, T* __restrict__ xout, int singular)
{
    __shared__ double bb[128];
    __shared__ double red[32];
    const int N = g.n[0] * g.n[1] * g.n[2];
    double s = 0.0, na = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        int i, j, k;
        decode_cell(g, t, i, j, k);
        const double v = act[t] ? (double)bin[pidx(g.sy, g.sz, i, j, k)] : 0.0;
        bb[t] = v;
        s += v;
        na += act[t] ? 1.0 : 0.0;
    }
    if (singular) {
        s = mac_block_sum(s, red);
        na = mac_block_sum(na, red);
        const double mean = na > 0.0 ? s / na : 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x)
            if (act[t]) bb[t] -= mean;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        double a0 = 0.0;
        for (int v = 0; v < N; ++v) a0 = fma(M[(size_t)v * N + t], bb[v], a0);
        int i, j, k;
        decode_cell(g, t, i, j, k);
        store_cell(xout, g, i, j, k, (T)a0);
    }
}

template <typename T>
void mac_bottom_dense(const CellGeom& g, const double* M, const unsigned char* act, const T* b, T* x, int singular,
                      cudaStream_t st)
{
    k_mac_bottom_dense<T><<<1, 128, 0, st>>>(g, M, act, b, x, singular);
}
template void mac_bottom_dense<double>(const CellGeom&, const double*, const unsigned char*, const double*, double*,
                                       int, cudaStream_t);
template void mac_bottom_dense<float>(const CellGeom&, const double*, const unsigned char*, const float*, float*, int,
                                      cudaStream_t);

// ------------------------------------------------------------------------------------------------
// coarse V-cycle in one cluster (the small levels of the MAC / ABecLaplacian hierarchy)
template <typename T>
__device__ __forceinline__ void mc_rbgs(const CellGeom& g, const T* bx, const T* by, const T* bz, const T* b, T* x,
                                        int color, long long t0, long long dt)
{
    const int hx = (g.n[0] + 1) / 2;
    const long long n = (long long)g.n[1] * g.n[2] * hx;
    for (long long t = t0; t < n; t += dt) {
        const long long row = t / hx;
        const int k = (int)(row / g.n[1]);
        const int j = (int)(row - (long long)k * g.n[1]);
        const int i = 2 * (int)(t - row * hx) + ((j + k + color) & 1);
        if (i >= g.n[0]) continue;
        const long long p = pidx(g.sy, g.sz, i, j, k);
        T diag, off;
        (void)mac_Ax<T, MacLdCg>(g, x, bx, by, bz, p, diag, off);
        const T v = diag != T(0) ? (__ldcg(b + p) + off) / diag : T(0);
        store_cell(x, g, i, j, k, v);
    }
}

template <typename T>
__global__ void __launch_bounds__(kMacCoarseThreads) k_mac_coarse_vcycle(MacCoarseCycle<T> a)
{
    extern __shared__ double bb[];
    const long long t0 = (long long)cluster_rank() * blockDim.x + threadIdx.x;
    const long long dt = (long long)cluster_nctas() * blockDim.x;
    const int L = a.nl;
    for (int q = 0; q + 1 < L; ++q) {
        const CellGeom& g = a.g[q];
        for (long long t = t0; t < g.count; t += dt) a.x[q][t] = T(0);
        cluster_barrier();
        for (int p = 0; p < a.nu1; ++p) {
            mc_rbgs<T>(g, a.bx[q], a.by[q], a.bz[q], a.b[q], a.x[q], 0, t0, dt);
            cluster_barrier();
            mc_rbgs<T>(g, a.bx[q], a.by[q], a.bz[q], a.b[q], a.x[q], 1, t0, dt);
            cluster_barrier();
        }
        const long long nc = (long long)g.n[0] * g.n[1] * g.n[2];
        for (long long t = t0; t < nc; t += dt) {
            int i, j, k;
            decode_cell(g, t, i, j, k);
            const long long p = pidx(g.sy, g.sz, i, j, k);
            T diag, off;
            a.r[q][p] = __ldcg(a.b[q] + p) - mac_Ax<T, MacLdCg>(g, a.x[q], a.bx[q], a.by[q], a.bz[q], p, diag, off);
        }
        cluster_barrier();
        const CellGeom& gc = a.g[q + 1];
        const long long ncc = (long long)gc.n[0] * gc.n[1] * gc.n[2];
        const T* rf = a.r[q];
        for (long long t = t0; t < ncc; t += dt) {
            int I, J, K;
            decode_cell(gc, t, I, J, K);
            const long long f = pidx(g.sy, g.sz, 2 * I, 2 * J, 2 * K);
            const T v = ((__ldcg(rf + f) + __ldcg(rf + f + 1)) + (__ldcg(rf + f + g.sy) + __ldcg(rf + f + 1 + g.sy))) +
                        ((__ldcg(rf + f + g.sz) + __ldcg(rf + f + 1 + g.sz)) +
                         (__ldcg(rf + f + g.sy + g.sz) + __ldcg(rf + f + 1 + g.sy + g.sz)));
            a.b[q + 1][pidx(gc.sy, gc.sz, I, J, K)] = v;
        }
        cluster_barrier();
    }
    if (cluster_rank() == 0) {
        // x = M b on the bottom (as k_mac_bottom_dense)
        const CellGeom& g = a.g[L - 1];
        const int N = g.n[0] * g.n[1] * g.n[2];
        double sm = 0.0, na = 0.0;
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            int i, j, k;
            decode_cell(g, t, i, j, k);
            const double v = a.act[t] ? (double)__ldcg(a.b[L - 1] + pidx(g.sy, g.sz, i, j, k)) : 0.0;
            bb[t] = v;
            sm += v;
            na += a.act[t] ? 1.0 : 0.0;
        }
        if (a.singular) {
            sm = block_sum_all(sm);
            na = block_sum_all(na);
            const double mean = na > 0.0 ? sm / na : 0.0;
            for (int t = threadIdx.x; t < N; t += blockDim.x)
                if (a.act[t]) bb[t] -= mean;
        }
        __syncthreads();
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            double a0 = 0.0;
            for (int v = 0; v < N; ++v) a0 = fma(a.M[(size_t)v * N + t], bb[v], a0);
            int i, j, k;
            decode_cell(g, t, i, j, k);
            store_cell(a.x[L - 1], g, i, j, k, (T)a0);
        }
    }
    cluster_barrier();
    for (int q = L - 2; q >= 0; --q) {
        const CellGeom& g = a.g[q];
        const CellGeom& gc = a.g[q + 1];
        const long long nc = (long long)g.n[0] * g.n[1] * g.n[2];
        for (long long t = t0; t < nc; t += dt) {
            int i, j, k;
            decode_cell(g, t, i, j, k);
            const long long p = pidx(g.sy, g.sz, i, j, k);
            store_cell(a.x[q], g, i, j, k,
                       __ldcg(a.x[q] + p) + __ldcg(a.x[q + 1] + pidx(gc.sy, gc.sz, i >> 1, j >> 1, k >> 1)));
        }
        cluster_barrier();
        for (int p = 0; p < a.nu2; ++p) {
            mc_rbgs<T>(g, a.bx[q], a.by[q], a.bz[q], a.b[q], a.x[q], 1, t0, dt);
            cluster_barrier();
            mc_rbgs<T>(g, a.bx[q], a.by[q], a.bz[q], a.b[q], a.x[q], 0, t0, dt);
            cluster_barrier();
        }
    }
}

int mac_coarse_cluster_size()
{
    static int cached = -1;
    if (cached > 0) return cached;
    int best = 8;
    if (cudaFuncSetAttribute(k_mac_coarse_vcycle<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(k_mac_coarse_vcycle<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(kMacCoarseThreads);
        cfg.dynamicSmemBytes = kMacDenseBottomMax * sizeof(double);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n32 = 0, n64 = 0;
        if (cudaOccupancyMaxActiveClusters(&n32, k_mac_coarse_vcycle<float>, &cfg) == cudaSuccess &&
            cudaOccupancyMaxActiveClusters(&n64, k_mac_coarse_vcycle<double>, &cfg) == cudaSuccess && n32 > 0 &&
            n64 > 0)
            best = 16;
    }
    cudaGetLastError();
    cached = best;
    return best;
}

template <typename T>
int mac_coarse_vcycle(const MacCoarseCycle<T>& c, int cluster, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(kMacCoarseThreads);
    cfg.dynamicSmemBytes = kMacDenseBottomMax * sizeof(double);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k_mac_coarse_vcycle<T>, c);
    return e == cudaSuccess ? GBP_OK : cuda_fail(e, "k_mac_coarse_vcycle launch");
}
template int mac_coarse_vcycle<float>(const MacCoarseCycle<float>&, int, cudaStream_t);
template int mac_coarse_vcycle<double>(const MacCoarseCycle<double>&, int, cudaStream_t);

void mac_set_beta(const CellGeom& g, int d, int source, const gbp_array4* src, double cval, int bclo, int bchi,
                  double* b64, float* b32, cudaStream_t st, const RobinFaces* rb, const double* ap, double mult)
{
    gbp_array4 a{};
    if (src) a = *src;
    RobinFaces r{};
    if (rb) r = *rb;
    k_mac_beta<<<nblk(nface(g, d), 256), 256, 0, st>>>(g, d, source, a, cval, bclo, bchi, b64, b32, r, ap, mult);
}

// ------------------------------------------------------------------------------------------------
// ABecLaplacian extras: the diagonal alpha a V per cell on every level, the right-hand side V rhs with
// the Dirichlet boundary values moved onto it
__global__ void k_abec_acoef(CellGeom g, gbp_array4 a, int have_a, double alpha, double a0, double* __restrict__ a64,
                             float* __restrict__ a32)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    const double v = alpha * (have_a ? a4(a, i, j, k, 0) : a0) * g.vol;
    const long long p = pidx(g.sy, g.sz, i, j, k);
    a64[p] = v;
    a32[p] = (float)v;
}

__global__ void k_abec_acoarsen(CellGeom gf, CellGeom gc, const double* __restrict__ af, double* __restrict__ ac64,
                                float* __restrict__ ac32)
{
    int I, J, K;
    if (!decode_cell(gc, blockIdx.x * (long long)blockDim.x + threadIdx.x, I, J, K)) return;
    const long long f = pidx(gf.sy, gf.sz, 2 * I, 2 * J, 2 * K);
    const double v = ((af[f] + af[f + 1]) + (af[f + gf.sy] + af[f + 1 + gf.sy])) +
                     ((af[f + gf.sz] + af[f + 1 + gf.sz]) + (af[f + gf.sy + gf.sz] + af[f + 1 + gf.sy + gf.sz]));
    const long long p = pidx(gc.sy, gc.sz, I, J, K);
    ac64[p] = v;
    ac32[p] = (float)v;
}

__global__ void k_abec_rhs(CellGeom g, gbp_array4 rhs, double* __restrict__ b)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    b[pidx(g.sy, g.sz, i, j, k)] = g.vol * a4(rhs, i, j, k, 0);
}

// b += w eff_face phi_b on the cells next to a Dirichlet side (phi_b: the ghost cell of phi, which holds
// the value on the face)
__global__ void k_abec_dirichlet(CellGeom g, int d, int hi, const double* __restrict__ beta, gbp_array4 phi,
                                 double* __restrict__ b)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.n[d1] * g.n[d2]) return;
    int c[3], f[3];
    c[d1] = f[d1] = (int)(t % g.n[d1]);
    c[d2] = f[d2] = (int)(t / g.n[d1]);
    c[d] = hi ? g.n[d] - 1 : 0;
    f[d] = hi ? g.n[d] : 0;
    int gh[3] = {c[0], c[1], c[2]};
    gh[d] = hi ? g.n[d] : -1;
    const double eff = beta[pidx(g.sy, g.sz, f[0], f[1], f[2])];
    b[pidx(g.sy, g.sz, c[0], c[1], c[2])] += g.w[d] * eff * a4(phi, gh[0], gh[1], gh[2], 0);
}

void abec_acoef(const CellGeom& g, const gbp_array4* a, double alpha, double a0, double* a64, float* a32,
                cudaStream_t st)
{
    gbp_array4 aa{};
    if (a) aa = *a;
    k_abec_acoef<<<nblk(ncell(g), 256), 256, 0, st>>>(g, aa, a != nullptr, alpha, a0, a64, a32);
}
void abec_acoarsen(const CellGeom& gf, const CellGeom& gc, const double* af, double* ac64, float* ac32,
                   cudaStream_t st)
{
    k_abec_acoarsen<<<nblk(ncell(gc), 256), 256, 0, st>>>(gf, gc, af, ac64, ac32);
}
void abec_rhs(const CellGeom& g, const gbp_array4& rhs, double* b, cudaStream_t st)
{
    k_abec_rhs<<<nblk(ncell(g), 256), 256, 0, st>>>(g, rhs, b);
}
void abec_dirichlet(const CellGeom& g, int d, int hi, const double* beta, const gbp_array4& phi, double* b,
                    cudaStream_t st)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    k_abec_dirichlet<<<nblk((long long)g.n[d1] * g.n[d2], 256), 256, 0, st>>>(g, d, hi, beta, phi, b);
}

__global__ void k_mac_load_kappa(CellGeom g, gbp_array4 in, double* __restrict__ kap)
{
    int i, j, k;
    if (decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k))
        store_cell(kap, g, i, j, k, a4(in, i, j, k, 0));
}

__global__ void k_mac_load_aperture(CellGeom g, int d, gbp_array4 in, double* __restrict__ ap)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    fn[d] += 1;
    if (t >= (long long)fn[0] * fn[1] * fn[2]) return;
    int f[3];
    f[0] = (int)(t % fn[0]);
    f[1] = (int)((t / fn[0]) % fn[1]);
    f[2] = (int)(t / ((long long)fn[0] * fn[1]));
    ap[pidx(g.sy, g.sz, f[0], f[1], f[2])] = a4(in, f[0], f[1], f[2], 0);
}

void mac_load_eb(const CellGeom& g, const gbp_array4& vfrac, const gbp_array4* const apf[3], const MacEB& eb,
                 cudaStream_t st)
{
    cudaMemsetAsync(eb.kap, 0, sizeof(double) * g.count, st);
    k_mac_load_kappa<<<nblk(ncell(g), 256), 256, 0, st>>>(g, vfrac, eb.kap);
    for (int d = 0; d < 3; ++d) {
        cudaMemsetAsync(eb.ap[d], 0, sizeof(double) * g.count, st);
        k_mac_load_aperture<<<nblk(nface(g, d), 256), 256, 0, st>>>(g, d, *apf[d], eb.ap[d]);
    }
}

__global__ void k_mac_robin_factors(CellGeom g, int d, int hi, gbp_array4 a, gbp_array4 b, gbp_array4 f, int has_f,
                                    double* __restrict__ rfac, unsigned* flags)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.n[d1] * g.n[d2]) return;
    int c[3];
    c[d1] = (int)(t % g.n[d1]);
    c[d2] = (int)(t / g.n[d1]);
    c[d] = hi ? g.n[d] : -1;  // the ghost cell next to the face holds the Robin data
    const double av = a4(a, c[0], c[1], c[2], 0), bv = a4(b, c[0], c[1], c[2], 0);
    const double fv = has_f ? a4(f, c[0], c[1], c[2], 0) : 0.0;
    const double den = av * 0.5 * g.h[d] + bv;
    unsigned fl = 0;
    if (!(av >= 0.0) || !(bv >= 0.0) || !(den > 0.0) || fv != 0.0) fl |= 2u;
    if (av > 0.0) fl |= 1u;
    rfac[t] = den > 0.0 ? av * g.h[d] / den : 0.0;
    if (fl) atomicOr(flags, fl);
}

void mac_robin_factors(const CellGeom& g, int d, int hi, const gbp_array4& a, const gbp_array4& b,
                       const gbp_array4* f, double* rfac, unsigned* flags, cudaStream_t st)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const long long n = (long long)g.n[d1] * g.n[d2];
    gbp_array4 fz{};
    if (f) fz = *f;
    k_mac_robin_factors<<<nblk(n, 256), 256, 0, st>>>(g, d, hi, a, b, fz, f ? 1 : 0, rfac, flags);
}

__global__ void k_mac_robin_apply(CellGeom g, int d, int hi, const double* __restrict__ braw,
                                  const double* __restrict__ rfac, double* __restrict__ b64, float* __restrict__ b32,
                                  const double* __restrict__ ap)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)g.n[d1] * g.n[d2]) return;
    int f[3];
    f[d1] = (int)(t % g.n[d1]);
    f[d2] = (int)(t / g.n[d1]);
    f[d] = hi ? g.n[d] : 0;
    const long long p = pidx(g.sy, g.sz, f[0], f[1], f[2]);
    double eff = braw[t] * rfac[t];
    if (ap) eff = ap[p] > 0.0 ? eff * ap[p] : 0.0;
    b64[p] = eff;
    b32[p] = (float)eff;
}

void mac_robin_apply(const CellGeom& g, int d, int hi, const double* braw, const double* rfac, double* b64,
                     float* b32, cudaStream_t st, const double* ap)
{
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const long long n = (long long)g.n[d1] * g.n[d2];
    k_mac_robin_apply<<<nblk(n, 256), 256, 0, st>>>(g, d, hi, braw, rfac, b64, b32, ap);
}
void mac_coarsen_beta(const CellGeom& gf, const CellGeom& gc, int d, const double* bf, double* bc64, float* bc32,
                      cudaStream_t st)
{
    k_mac_beta_coarsen<<<nblk(nface(gc, d), 256), 256, 0, st>>>(gf, gc, d, bf, bc64, bc32);
}
void mac_rhs(const CellGeom& g, const gbp_array4& ux, const gbp_array4& uy, const gbp_array4& uz, double* b,
             cudaStream_t st, const MacEB* eb)
{
    MacEB e{};
    if (eb) e = *eb;
    k_mac_rhs<<<nblk(ncell(g), 256), 256, 0, st>>>(g, ux, uy, uz, b, e);
}
void mac_eb_inflow_flux(const CellGeom& g, const gbp_array4& eb_vel, const MacEB& eb, double* ebflux,
                        cudaStream_t st)
{
    k_mac_eb_inflow_flux<<<nblk(ncell(g), 256), 256, 0, st>>>(g, eb_vel, eb, ebflux);
}
void mac_zero_faces(const CellGeom& g, int d, const gbp_array4& u, cudaStream_t st)
{
    k_mac_zero_faces<<<nblk(nface(g, d), 256), 256, 0, st>>>(g, d, u);
}

void mac_correct(const CellGeom& g, int d, const gbp_array4& u, const double* beta, const double* phi,
                 cudaStream_t st, const double* ap)
{
    k_mac_correct<<<nblk(nface(g, d), 256), 256, 0, st>>>(g, d, u, beta, phi, ap);
}
void mac_load_phi(const CellGeom& g, const gbp_array4& in, double* phi, cudaStream_t st)
{
    k_mac_load_phi<<<nblk(ncell(g), 256), 256, 0, st>>>(g, in, phi);
}
void mac_store_phi(const CellGeom& g, const gbp_array4& out, const double* phi, cudaStream_t st)
{
    k_mac_store_phi<<<nblk(ncell(g), 256), 256, 0, st>>>(g, out, phi);
}
void mac_norm(const CellGeom& g, const double* v, unsigned long long* norm, cudaStream_t st, const double* kap)
{
    k_mac_norm<<<nblk(ncell(g), 256), 256, 0, st>>>(g, v, norm, kap);
}
// the sums' grid: at most 1184 blocks (8 per SM of a 148-SM part and more than enough on 152), each
// thread walking its cells; partials holds one sum per block and the folded mean after them
static unsigned mac_sum_blocks(const CellGeom& g)
{
    const unsigned nb = nblk(ncell(g), 256);
    return nb < 1184 ? nb : 1184;
}
int mac_partials_needed(const CellGeom& g) { return (int)mac_sum_blocks(g) + 1; }
void mac_remove_mean(const CellGeom& g, double* v, double* partials, int mode, cudaStream_t st, const double* kap,
                     double nfluid)
{
    const unsigned nb = mac_sum_blocks(g);
    if (!kap) nfluid = (double)g.n[0] * g.n[1] * g.n[2];
    k_mac_sums<<<nb, 256, 0, st>>>(g, v, partials, kap, mode);
    k_mac_fold<<<1, 1024, 0, st>>>(partials, (int)nb, nfluid);
    const unsigned na = nblk(ncell(g), 256);
    k_mac_remove_mean<<<na < 2368 ? na : 2368, 256, 0, st>>>(g, v, partials, (int)nb, mode, kap);
}

// ------------------------------------------------------------------------------------------------
// Cut cells (embedded boundary) on the finest level. The 7-point part of the operator carries the
// apertures in its face betas; the kernels below add the difference between the centroid and the
// face-centre normal derivative on the few cut faces, from a table built once per geometry.
__global__ void k_mac_pack_faces(CellGeom g, int d, gbp_array4 in, int c, double* __restrict__ out)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    if (d >= 0) fn[d] += 1;
    if (t >= (long long)fn[0] * fn[1] * fn[2]) return;
    const int i = (int)(t % fn[0]);
    const int j = (int)((t / fn[0]) % fn[1]);
    const int k = (int)(t / ((long long)fn[0] * fn[1]));
    out[t] = a4(in, i, j, k, c);
}

void mac_pack_faces(const CellGeom& g, int d, const gbp_array4& in, int c, double* out, cudaStream_t st)
{
    k_mac_pack_faces<<<nblk(d >= 0 ? nface(g, d) : ncell(g), 256), 256, 0, st>>>(g, d, in, c, out);
}

struct EbPtrs {
    const double* b[3];
    const double* ap[3];
};

__global__ void k_eb_table_beta(const EbFace* __restrict__ F, int nf, EbPtrs P, double* __restrict__ cb64,
                                float* __restrict__ cb32)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nf) return;
    const EbFace& f = F[e];
    for (int m = 0; m < 4; ++m) {
        double v = 0.0;
        if (m < f.nm) {
            const long long q = f.pf[m];
            v = f.coef[m] * (P.b[f.d][q] / P.ap[f.d][q]);
        }
        cb64[4 * e + m] = v;
        cb32[4 * e + m] = (float)v;
    }
}

void eb_table_beta(const EbFace* F, int nf, const double* const b64[3], const double* const ap[3], double* cb64,
                   float* cb32, cudaStream_t st)
{
    if (nf <= 0) return;
    EbPtrs P;
    for (int d = 0; d < 3; ++d) {
        P.b[d] = b64[d];
        P.ap[d] = ap[d];
    }
    k_eb_table_beta<<<nblk(nf, 128), 128, 0, st>>>(F, nf, P, cb64, cb32);
}

template <typename T>
__device__ __forceinline__ T eb_dflux(const EbFace& f, const T* __restrict__ cb, int e, const T* __restrict__ x,
                                      long long sd)
{
    T acc = T(0);
    for (int m = 0; m < f.nm; ++m) acc += cb[4 * e + m] * (x[f.pf[m]] - x[f.pf[m] - sd]);
    return acc;
}

template <typename T>
__global__ void k_eb_cells(CellGeom g, const EbCell* __restrict__ C, int nc, const EbFace* __restrict__ F,
                           const T* __restrict__ cb, const T* __restrict__ x, const T* in, T* out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nc) return;
    const EbCell c = C[e];
    const long long sd[3] = {1, g.sy, g.sz};
    T corr = T(0);
    for (int s = 0; s < 6; ++s) {
        const int q = c.slot[s];
        if (q < 0) continue;
        const EbFace& f = F[q];
        const T df = eb_dflux<T>(f, cb, q, x, sd[f.d]);
        // (A phi)_c = -(F_high - F_low) summed over the directions
        corr += (s & 1) ? -df : df;
    }
    out[c.p] = in[c.p] - corr;
}

template <typename T>
void eb_cells(const CellGeom& g, const EbCell* C, int nc, const EbFace* F, const T* cb, const T* x, const T* in,
              T* out, cudaStream_t st)
{
    if (nc <= 0) return;
    k_eb_cells<T><<<nblk(nc, 128), 128, 0, st>>>(g, C, nc, F, cb, x, in, out);
}
template void eb_cells<double>(const CellGeom&, const EbCell*, int, const EbFace*, const double*, const double*,
                               const double*, double*, cudaStream_t);
template void eb_cells<float>(const CellGeom&, const EbCell*, int, const EbFace*, const float*, const float*,
                              const float*, float*, cudaStream_t);

struct EbU {
    gbp_array4 u[3];
};

__global__ void k_eb_correct_u(CellGeom g, const EbFace* __restrict__ F, int nf, EbPtrs P,
                               const double* __restrict__ phi, EbU U)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nf) return;
    const EbFace& f = F[e];
    const long long sd = f.d == 0 ? 1 : (f.d == 1 ? g.sy : g.sz);
    double acc = 0.0;
    for (int m = 0; m < f.nm; ++m) {
        const long long q = f.pf[m];
        acc += f.vcoef[m] * (P.b[f.d][q] / P.ap[f.d][q]) * (phi[q] - phi[q - sd]);
    }
    *a4p(U.u[f.d], f.f[0], f.f[1], f.f[2], 0) -= acc;
}

void eb_correct_u(const CellGeom& g, const EbFace* F, int nf, const double* const b64[3], const double* const ap[3],
                  const double* phi, gbp_array4* const u[3], cudaStream_t st)
{
    if (nf <= 0) return;
    EbPtrs P;
    EbU U;
    for (int d = 0; d < 3; ++d) {
        P.b[d] = b64[d];
        P.ap[d] = ap[d];
        U.u[d] = *u[d];
    }
    k_eb_correct_u<<<nblk(nf, 128), 128, 0, st>>>(g, F, nf, P, phi, U);
}

__global__ void k_eb_zero_covered(CellGeom g, const double* __restrict__ kap, double* phi)
{
    int i, j, k;
    if (!decode_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, i, j, k)) return;
    if (!(kap[pidx(g.sy, g.sz, i, j, k)] > 0.0)) store_cell(phi, g, i, j, k, 0.0);
}

void eb_zero_covered(const CellGeom& g, const double* kap, double* phi, cudaStream_t st)
{
    k_eb_zero_covered<<<nblk(ncell(g), 256), 256, 0, st>>>(g, kap, phi);
}
template <typename TE>
void mac_add_correction(const CellGeom& g, double* x, const TE* e, double inv_scale, cudaStream_t st)
{
    k_mac_add_correction<TE><<<nblk(ncell(g), 256), 256, 0, st>>>(g, x, e, inv_scale);
}
template void mac_add_correction<double>(const CellGeom&, double*, const double*, double, cudaStream_t);
template void mac_add_correction<float>(const CellGeom&, double*, const float*, double, cudaStream_t);
void mac_to_f32(const CellGeom& g, const double* r, float* r32, double scale, cudaStream_t st)
{
    k_mac_to_f32<<<nblk(ncell(g), 256), 256, 0, st>>>(g, r, r32, scale);
}

}  // namespace gbp
