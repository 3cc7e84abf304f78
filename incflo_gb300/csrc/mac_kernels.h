// Host-side launchers of the MAC projection kernels (mac_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

template <typename T>
void mac_rbgs(const CellGeom& g, const T* bx, const T* by, const T* bz, const T* b, T* x, int color, cudaStream_t st);
template <typename T>
void mac_resid(const CellGeom& g, const T* bx, const T* by, const T* bz, const T* x, const T* b, T* r,
               unsigned long long* norm, cudaStream_t st);
template <typename T>
void mac_restrict(const CellGeom& gf, const CellGeom& gc, const T* rf, T* bc, cudaStream_t st);
template <typename T>
void mac_prolong_add(const CellGeom& gf, const CellGeom& gc, const T* xc, T* xf, cudaStream_t st);
template <typename T>
void mac_bottom(const CellGeom& g, const double* bx, const double* by, const double* bz, const T* b, T* x,
                double* scratch, int maxiter, double rtol, double atol, int singular, cudaStream_t st);

// source: 0 = face array, 1 = constant, 2 = dt / face average of rho (src = rho, cval = dt)
// Robin boundary faces of the finest level (side q = 2 d + hi): rfac = a h / (a h / 2 + b) per face,
// braw = the face beta before that factor; nullptr for the other sides
struct RobinFaces {
    const double* rfac[6];
    double* braw[6];
};
// rfac of one Robin side from the ghost cells of robin_a / robin_b / robin_f (cell arrays with one
// ghost layer); flags: bit 0 = some a > 0, bit 1 = invalid (a < 0, b < 0, a h / 2 + b <= 0, f != 0)
void mac_robin_factors(const CellGeom& g, int d, int hi, const gbp_array4& a, const gbp_array4& b,
                       const gbp_array4* f, double* rfac, unsigned* flags, cudaStream_t st);
// eff beta = braw * rfac on the faces of one Robin side of the finest level
void mac_robin_apply(const CellGeom& g, int d, int hi, const double* braw, const double* rfac, double* b64,
                     float* b32, cudaStream_t st);
void mac_set_beta(const CellGeom& g, int d, int source, const gbp_array4* src, double cval, int bclo, int bchi,
                  double* b64, float* b32, cudaStream_t st, const RobinFaces* rb = nullptr);
void mac_coarsen_beta(const CellGeom& gf, const CellGeom& gc, int d, const double* bf, double* bc64, float* bc32,
                      cudaStream_t st);
void mac_rhs(const CellGeom& g, const gbp_array4& ux, const gbp_array4& uy, const gbp_array4& uz, double* b,
             cudaStream_t st);
void mac_correct(const CellGeom& g, int d, const gbp_array4& u, const double* beta, const double* phi,
                 cudaStream_t st);
void mac_load_phi(const CellGeom& g, const gbp_array4& in, double* phi, cudaStream_t st);
void mac_store_phi(const CellGeom& g, const gbp_array4& out, const double* phi, cudaStream_t st);
void mac_norm(const CellGeom& g, const double* v, unsigned long long* norm, cudaStream_t st);
int mac_partials_needed(const CellGeom& g);
void mac_remove_mean(const CellGeom& g, double* v, double* partials, int mode, cudaStream_t st);
template <typename TE>
void mac_add_correction(const CellGeom& g, double* x, const TE* e, double inv_scale, cudaStream_t st);
void mac_to_f32(const CellGeom& g, const double* r, float* r32, double scale, cudaStream_t st);

}  // namespace gbp
