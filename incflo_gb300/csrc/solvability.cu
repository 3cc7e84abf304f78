// Inflow/outflow solvability: scale the outflow part of the normal velocity on the
// direction-dependent boundary faces so that the net boundary flux is zero. This is what
// HydroUtils::enforceInOutSolvability (AMReX-Hydro, not vendored) does for incflo before the nodal
// projection (src/projection/incflo_apply_nodal_projection.cpp:166-179, on the cell-centred
// velocity whose ghost cells hold the boundary values) and before the MAC projection
// (src/convection/incflo_compute_MAC_projected_velocities.cpp:266-270, on the boundary faces).
//
// Two kernels, no host synchronisation: a reduction of the inflow and outflow fluxes (face area x
// normal velocity) over the marked faces into two device doubles, then a pass that multiplies every
// outflow normal velocity by influx / outflux (left unchanged when there is no outflow).
#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "incflo_gb300.h"
#include "solvability.h"

namespace gbp {

namespace {

constexpr int kT = 256;

__device__ __forceinline__ double* at(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride +
           (long long)(k - a.lo[2]) * a.kstride + (long long)n * a.nstride;
}

struct Faces {
    gbp_array4 u[3];   // normal-velocity array of each direction (component comp[d])
    int comp[3];
    int n[3];          // cells
    int face_hi[3];    // index of the high boundary position in u[d] along d
    int face_lo[3];    // index of the low boundary position
    int mark[6];       // face 2*d + side takes part
    double area[3];
    long long nf[6];   // positions on each face
};

// face f = 2d + side; position q on that face -> (i, j, k) in u[d]'s index space
__device__ __forceinline__ void face_pos(const Faces& F, int f, long long q, int& i, int& j, int& k)
{
    const int d = f >> 1, side = f & 1;
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    int c[3];
    c[d1] = (int)(q % F.n[d1]);
    c[d2] = (int)(q / F.n[d1]);
    c[d] = side ? F.face_hi[d] : F.face_lo[d];
    i = c[0];
    j = c[1];
    k = c[2];
}

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// flux[0] += inflow, flux[1] += outflow (both positive), over all marked faces
__global__ void k_inout_flux(Faces F, long long total, double* flux)
{
    double in = 0.0, out = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long q = t;
        int f = 0;
        while (f < 6 && q >= F.nf[f]) q -= F.nf[f++];
        if (f >= 6 || !F.mark[f]) continue;
        int i, j, k;
        face_pos(F, f, q, i, j, k);
        const int d = f >> 1;
        const double un = *at(F.u[d], i, j, k, F.comp[d]);
        // flux into the domain: +u on the low side, -u on the high side
        const double into = (f & 1) ? -un : un;
        if (into > 0.0) in += into * F.area[d];
        else out -= into * F.area[d];
    }
    in = block_sum(in);
    out = block_sum(out);
    if (threadIdx.x == 0) {
        atomicAdd(flux, in);
        atomicAdd(flux + 1, out);
    }
}

__global__ void k_inout_scale(Faces F, long long total, const double* flux)
{
    const double out = flux[1];
    if (!(out > 0.0)) return;
    const double alpha = flux[0] / out;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long q = t;
        int f = 0;
        while (f < 6 && q >= F.nf[f]) q -= F.nf[f++];
        if (f >= 6 || !F.mark[f]) continue;
        int i, j, k;
        face_pos(F, f, q, i, j, k);
        const int d = f >> 1;
        double* p = at(F.u[d], i, j, k, F.comp[d]);
        const double into = (f & 1) ? -*p : *p;
        if (into < 0.0) *p *= alpha;
    }
}

int launch(const Faces& F, double* flux, cudaStream_t st)
{
    long long total = 0;
    for (int f = 0; f < 6; ++f) total += F.nf[f];
    if (total == 0) return GBP_OK;
    GBP_CUDA(cudaMemsetAsync(flux, 0, 2 * sizeof(double), st));
    const unsigned nb = (unsigned)std::min<long long>(1024, (total + kT - 1) / kT);
    k_inout_flux<<<nb, kT, 0, st>>>(F, total, flux);
    k_inout_scale<<<nb, kT, 0, st>>>(F, total, flux);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

Faces base_faces(const gbp_geometry& geom, const int dd_lo[3], const int dd_hi[3])
{
    Faces F{};
    for (int d = 0; d < 3; ++d) F.n[d] = geom.n_cell[d];
    double h[3];
    for (int d = 0; d < 3; ++d) h[d] = (geom.prob_hi[d] - geom.prob_lo[d]) / geom.n_cell[d];
    for (int d = 0; d < 3; ++d) {
        const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
        F.area[d] = h[d1] * h[d2];
        F.mark[2 * d] = dd_lo[d] != 0;
        F.mark[2 * d + 1] = dd_hi[d] != 0;
        const long long nf = (long long)F.n[d1] * F.n[d2];
        F.nf[2 * d] = F.mark[2 * d] ? nf : 0;
        F.nf[2 * d + 1] = F.mark[2 * d + 1] ? nf : 0;
    }
    return F;
}

}  // namespace

int enforce_inout_cell(const gbp_geometry& geom, const int dd_lo[3], const int dd_hi[3], const gbp_array4& vel,
                       double* flux, cudaStream_t st)
{
    Faces F = base_faces(geom, dd_lo, dd_hi);
    for (int d = 0; d < 3; ++d) {
        F.u[d] = vel;
        F.comp[d] = d;
        F.face_lo[d] = -1;          // ghost cell holding the boundary value
        F.face_hi[d] = geom.n_cell[d];
    }
    return launch(F, flux, st);
}

int enforce_inout_faces(const gbp_geometry& geom, const int dd_lo[3], const int dd_hi[3], const gbp_array4* u,
                        double* flux, cudaStream_t st)
{
    Faces F = base_faces(geom, dd_lo, dd_hi);
    for (int d = 0; d < 3; ++d) {
        F.u[d] = u[d];
        F.comp[d] = 0;
        F.face_lo[d] = 0;           // boundary face
        F.face_hi[d] = geom.n_cell[d];
    }
    return launch(F, flux, st);
}

}  // namespace gbp

// ------------------------------------------------------------------------------------------------
// amrex::average_down of a cell field (incflo_apply_nodal_projection.cpp:258-266 for gp): each coarse
// cell of the region the fine level covers takes the mean of its ratio[0] x ratio[1] x ratio[2] fine
// cells, component by component.
namespace gbp {
namespace {
__global__ void k_average_down(gbp_array4 f, gbp_array4 c, int r0, int r1, int r2, int ncomp, int lo0, int lo1,
                               int lo2, int nx, int ny, int nz)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * ny * nz * ncomp) return;
    const int i = lo0 + (int)(t % nx);
    const int j = lo1 + (int)((t / nx) % ny);
    const long long r = t / ((long long)nx * ny);
    const int k = lo2 + (int)(r % nz);
    const int n = (int)(r / nz);
    double acc = 0.0;
    for (int c2 = 0; c2 < r2; ++c2)
        for (int c1 = 0; c1 < r1; ++c1)
            for (int c0 = 0; c0 < r0; ++c0) acc += *at(f, i * r0 + c0, j * r1 + c1, k * r2 + c2, n);
    *at(c, i, j, k, n) = acc / (double)(r0 * r1 * r2);
}
}  // namespace

int average_down(const gbp_array4& fine, const gbp_array4& crse, const int ratio[3], int ncomp, const int lo[3],
                 const int hi[3], cudaStream_t st)
{
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const long long n = (long long)nx * ny * nz * ncomp;
    if (n <= 0) return GBP_OK;
    k_average_down<<<(unsigned)((n + kT - 1) / kT), kT, 0, st>>>(fine, crse, ratio[0], ratio[1], ratio[2], ncomp,
                                                                 lo[0], lo[1], lo[2], nx, ny, nz);
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}
}  // namespace gbp
