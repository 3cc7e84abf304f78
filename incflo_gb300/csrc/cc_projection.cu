// incflo::ApplyCCProjection for one single-box level, non-EB
// (src/projection/incflo_apply_cc_projection.cpp:199-487): the cell-centred ("MAC-type") projection of
// the cell velocity. Kernels around the MAC multigrid solve:
//   k_cc_prep    u += s gp / rho (non-incremental, :214-238); u -= U^n (incremental / small dt, :241-249)
//   k_mol_faces  normal velocity on faces by method-of-lines extrapolation (MOL::ExtrapVelToFaces,
//                AMReX-Hydro, :350-353): monotonised-central slopes, upwinding by the average of the
//                two face states; it also keeps a copy of the unprojected face velocity
//   (MAC solve)  beta = s / rho_face (arithmetic mean of the two cells, :276-323), project (:366)
//   k_cc_final   fluxes -beta grad phi = (projected - unprojected) face velocity, averaged to cells
//                (getFluxes + average_mac_to_ccvel, :383-399); u += gphi, p_cc = phi (+=), gp = -gphi rho / s
//                (-=) (:401-463); u += U^n (:471-477)
#include <cuda_runtime.h>

#include "cc_projection.h"
#include "gbp_internal.cuh"

namespace gbp {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ double& A(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data[(long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
                  (long long)n * a.nstride];
}

struct CcGeom {
    int n[3];
    int per[3];
    int bclo[3], bchi[3];
};

__global__ void k_cc_prep(CcGeom g, CcArgs a)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    split3(t, g.n[0], g.n[1], (long long)g.n[0] * g.n[1] * g.n[2], i, j, k);
    const double rho = a.rho.data ? A(a.rho, i, j, k, 0) : a.rho0;
    for (int d = 0; d < 3; ++d) {
        double u = A(a.vel, i, j, k, d);
        if (a.add_gp) u += A(a.gp, i, j, k, d) * (a.s / rho);
        if (a.sub_old) u -= A(a.vel_old, i, j, k, d);
        A(a.vel, i, j, k, d) = u;
    }
}

// value of component d of the cell at index c along d (other indices fixed); periodic wrap
__device__ __forceinline__ double qd(const CcArgs& a, int d, const int base[3], int c, int n)
{
    int q[3] = {base[0], base[1], base[2]};
    q[d] = c < 0 ? c + n : (c >= n ? c - n : c);
    return A(a.vel, q[0], q[1], q[2], d);
}

__device__ __forceinline__ double mc_slope(double qm, double q, double qp)
{
    const double dl = 2.0 * (q - qm), dr = 2.0 * (qp - q), dc = 0.5 * (qp - qm);
    double s = fmin(fmin(fabs(dl), fabs(dr)), fabs(dc));
    s = dl * dr > 0.0 ? s : 0.0;
    return dc > 0.0 ? s : -s;
}

__device__ __forceinline__ double upwind(double um, double up)
{
    constexpr double small = 1e-10;
    if (um < 0.0 && up > 0.0) return 0.0;
    const double avg = 0.5 * (um + up);
    return avg >= small ? um : (avg <= -small ? up : 0.0);
}

__global__ void k_mol_faces(CcGeom g, CcArgs a, int d, gbp_array4 uf, double* __restrict__ u0)
{
    int fn[3] = {g.n[0], g.n[1], g.n[2]};
    fn[d] += 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)fn[0] * fn[1] * fn[2]) return;
    int f[3];
    split3(t, fn[0], fn[1], (long long)fn[0] * fn[1] * fn[2], f[0], f[1], f[2]);
    const int n = g.n[d], fi = f[d];
    double val;
    if (!g.per[d] && (fi == 0 || fi == n)) {
        const int bc = fi == 0 ? g.bclo[d] : g.bchi[d];
        int c[3] = {f[0], f[1], f[2]};
        if (bc == GBP_BC_DIRICHLET) {
            c[d] = fi == 0 ? 0 : n - 1;  // outflow: the adjacent interior value
            val = A(a.vel, c[0], c[1], c[2], d);
        } else if (bc == GBP_BC_INFLOW && a.use_inflow) {
            c[d] = fi == 0 ? -1 : n;     // the ghost cell holds the inflow value
            val = A(a.vel, c[0], c[1], c[2], d);
        } else {
            val = 0.0;
        }
    } else {
        // cells L = fi-1 and R = fi (periodic wrap); zero slope next to a non-periodic boundary
        const int cl = fi - 1, cr = fi;
        const double ql = qd(a, d, f, cl, n), qr = qd(a, d, f, cr, n);
        double sl = 0.0, sr = 0.0;
        if (g.per[d] || (cl >= 1 && cl <= n - 2)) sl = mc_slope(qd(a, d, f, cl - 1, n), ql, qd(a, d, f, cl + 1, n));
        if (g.per[d] || (cr >= 1 && cr <= n - 2)) sr = mc_slope(qd(a, d, f, cr - 1, n), qr, qd(a, d, f, cr + 1, n));
        val = upwind(ql + 0.5 * sl, qr - 0.5 * sr);
    }
    A(uf, f[0], f[1], f[2], 0) = val;
    u0[t] = val;
}

__global__ void k_cc_final(CcGeom g, CcArgs a, gbp_array4 ux, gbp_array4 uy, gbp_array4 uz,
                           const double* __restrict__ u0x, const double* __restrict__ u0y,
                           const double* __restrict__ u0z, const double* __restrict__ phi)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    split3(t, g.n[0], g.n[1], (long long)g.n[0] * g.n[1] * g.n[2], i, j, k);
    const long long nx1 = g.n[0] + 1, ny1 = g.n[1] + 1;
    // unprojected copies are dense face arrays in x-fastest order
    const long long fx = i + nx1 * (j + (long long)g.n[1] * k);
    const long long fy = i + (long long)g.n[0] * (j + ny1 * k);
    const long long fz = i + (long long)g.n[0] * (j + (long long)g.n[1] * k);
    const long long sx = 1, sy = g.n[0], sz = (long long)g.n[0] * g.n[1];
    double gphi[3];
    gphi[0] = 0.5 * ((A(ux, i, j, k, 0) - u0x[fx]) + (A(ux, i + 1, j, k, 0) - u0x[fx + sx]));
    gphi[1] = 0.5 * ((A(uy, i, j, k, 0) - u0y[fy]) + (A(uy, i, j + 1, k, 0) - u0y[fy + sy]));
    gphi[2] = 0.5 * ((A(uz, i, j, k, 0) - u0z[fz]) + (A(uz, i, j, k + 1, 0) - u0z[fz + sz]));
    const double rho = a.rho.data ? A(a.rho, i, j, k, 0) : a.rho0;
    const double p = phi[t];
    for (int d = 0; d < 3; ++d) {
        double u = A(a.vel, i, j, k, d) + gphi[d];
        if (a.sub_old) u += A(a.vel_old, i, j, k, d);
        A(a.vel, i, j, k, d) = u;
        if (a.gp.data) {
            if (a.incremental) A(a.gp, i, j, k, d) -= gphi[d] * rho / a.s;
            else A(a.gp, i, j, k, d) = -gphi[d] * rho / a.s;
        }
    }
    if (a.p_cc.data) {
        if (a.incremental) A(a.p_cc, i, j, k, 0) += p;
        else A(a.p_cc, i, j, k, 0) = p;
    }
}

}  // namespace

int cc_projection(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const CcArgs& a,
                  gbp_array4* umac[3], double* scratch, MacSolver& mac, gbp_stats* stats, cudaStream_t st)
{
    CcGeom g{};
    for (int d = 0; d < 3; ++d) {
        g.n[d] = geom.n_cell[d];
        g.per[d] = bc_lo[d] == GBP_BC_PERIODIC;
        g.bclo[d] = bc_lo[d];
        g.bchi[d] = bc_hi[d];
    }
    const long long nc = (long long)g.n[0] * g.n[1] * g.n[2];
    const unsigned nbc = (unsigned)((nc + kT - 1) / kT);
    k_cc_prep<<<nbc, kT, 0, st>>>(g, a);
    double* u0[3];
    double* p = scratch;
    for (int d = 0; d < 3; ++d) {
        long long nf = nc / g.n[d] * (g.n[d] + 1);
        u0[d] = p;
        p += nf;
        k_mol_faces<<<(unsigned)((nf + kT - 1) / kT), kT, 0, st>>>(g, a, d, *umac[d], u0[d]);
    }
    double* phi = p;
    GBP_CUDA(cudaGetLastError());
    // beta = s / rho_face (or s / rho0), then the MAC solve from phi = 0
    int rc;
    if (a.rho.data) {
        const gbp_array4* src[3] = {&a.rho, nullptr, nullptr};
        rc = mac.set_beta(2, src, a.s);
    } else {
        const gbp_array4* src[3] = {nullptr, nullptr, nullptr};
        rc = mac.set_beta(1, src, a.s / a.rho0);
    }
    if (rc) return rc;
    gbp_array4 ph{};
    ph.data = phi;
    ph.hi[0] = g.n[0] - 1;
    ph.hi[1] = g.n[1] - 1;
    ph.hi[2] = g.n[2] - 1;
    ph.ncomp = 1;
    ph.jstride = g.n[0];
    ph.kstride = (long long)g.n[0] * g.n[1];
    rc = mac.project(umac, &ph, 0, stats);
    if (rc && rc != GBP_NOT_CONVERGED) return rc;
    k_cc_final<<<nbc, kT, 0, st>>>(g, a, *umac[0], *umac[1], *umac[2], u0[0], u0[1], u0[2], phi);
    GBP_CUDA(cudaGetLastError());
    return rc;
}

size_t cc_scratch_doubles(const gbp_geometry& geom)
{
    const size_t nx = geom.n_cell[0], ny = geom.n_cell[1], nz = geom.n_cell[2];
    return (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1) + nx * ny * nz;
}

}  // namespace gbp
