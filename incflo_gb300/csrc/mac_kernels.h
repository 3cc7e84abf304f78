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
// x = M b on the coarsest level (M: the precomputed dense inverse, act: cells with an equation)
constexpr int kMacDenseBottomMax = 128;
template <typename T>
void mac_bottom_dense(const CellGeom& g, const double* M, const unsigned char* act, const T* b, T* x, int singular,
                      cudaStream_t st);

// The coarse end of a MAC / ABecLaplacian V-cycle in one launch: levels 0 .. nl-1 of this struct (a tail of
// the hierarchy ending at the dense bottom) cycled from a zero start by one thread-block cluster, its CTAs
// meeting at cluster barriers between the phases (each colour of each red-black sweep, residual,
// restriction, bottom, prolongation); loads of data written inside the launch are L2-coherent.
constexpr int kMacCoarseMaxLevels = 10;
constexpr int kMacCoarseThreads = 1024;
template <typename T>
struct MacCoarseCycle {
    int nl;  // >= 2
    CellGeom g[kMacCoarseMaxLevels];
    const T* bx[kMacCoarseMaxLevels];
    const T* by[kMacCoarseMaxLevels];
    const T* bz[kMacCoarseMaxLevels];
    T* x[kMacCoarseMaxLevels];  // the result is x[0]
    T* b[kMacCoarseMaxLevels];  // b[0]: the first level's right-hand side (caller); b[q > 0]: restricted
    T* r[kMacCoarseMaxLevels];
    const double* M;            // dense inverse of the bottom operator
    const unsigned char* act;   // bottom cells that carry an equation
    int singular;
    int nu1, nu2;
};
int mac_coarse_cluster_size();
template <typename T>
int mac_coarse_vcycle(const MacCoarseCycle<T>& c, int cluster, cudaStream_t st);

// Cut cells of an embedded boundary on the finest level (all nullptr: no EB). Padded layouts: kap like a
// cell array, ap[d] like the face array of direction d (face (i,j,k) at pidx(i,j,k)).
struct MacEB {
    double* kap;
    double* ap[3];
    // flux of the EB inflow velocity out of each cell's fluid through its embedded boundary (padded cell
    // layout), subtracted from the right-hand side; nullptr: no EB inflow
    const double* ebflux;
};

// One cut face (0 < aperture < 1, not on a non-periodic domain side) whose flux uses the normal
// derivative at the face centroid: the bilinear blend of the face-centre differences of nm faces of
// direction d (m = 0 the face itself, then its open neighbours towards the centroid). pf[m] = padded
// index of face m (its high cell; the low cell is pf[m] - stride of d). coef[m] = ap w_d wt'_m and
// vcoef[m] = wt'_m / h_d, with wt'_0 = blend weight - 1 (the face-centre term is in the 7-point part).
struct EbFace {
    long long pf[4];
    double coef[4];
    double vcoef[4];
    int d, nm;
    int f[3];
};
// A cell with at least one cut face: slot[2d] = its low face of direction d, slot[2d+1] its high face
// (index into the EbFace table, -1 if that face is not cut).
struct EbCell {
    long long p;
    int slot[6];
};

// source: 0 = face array, 1 = constant, 2 = dt / face average of rho (src = rho, cval = dt),
// 3 = face average of a cell field (the adjacent cell on non-periodic sides); mult scales the result
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
                     float* b32, cudaStream_t st, const double* ap = nullptr);
// ap (cut cells): the face's aperture multiplies its beta
void mac_set_beta(const CellGeom& g, int d, int source, const gbp_array4* src, double cval, int bclo, int bchi,
                  double* b64, float* b32, cudaStream_t st, const RobinFaces* rb = nullptr,
                  const double* ap = nullptr, double mult = 1.0);
// ABecLaplacian (alpha a phi - beta div(b grad phi) = rhs on the same levels): a64 / a32 = alpha a V per
// cell (a == nullptr: the constant a0), coarse levels the sum of their 8 fine cells; b = V rhs; the
// Dirichlet boundary values (ghost cells of phi) moved onto b
void abec_acoef(const CellGeom& g, const gbp_array4* a, double alpha, double a0, double* a64, float* a32,
                cudaStream_t st);
void abec_acoarsen(const CellGeom& gf, const CellGeom& gc, const double* af, double* ac64, float* ac32,
                   cudaStream_t st);
void abec_rhs(const CellGeom& g, const gbp_array4& rhs, double* b, cudaStream_t st);
void abec_dirichlet(const CellGeom& g, int d, int hi, const double* beta, const gbp_array4& phi, double* b,
                    cudaStream_t st);
// copy the EB arrays into the padded layouts of eb (other padded positions 0)
void mac_load_eb(const CellGeom& g, const gbp_array4& vfrac, const gbp_array4* const apf[3], const MacEB& eb,
                 cudaStream_t st);
// dense copy of component c of a face array of direction d (d = -1: a cell array), x fastest
void mac_pack_faces(const CellGeom& g, int d, const gbp_array4& in, int c, double* out, cudaStream_t st);
// cb[4 e + m] = coef[m] * beta of face m (beta = b64 / ap of direction d), for every cut face e
void eb_table_beta(const EbFace* F, int nf, const double* const b64[3], const double* const ap[3], double* cb64,
                   float* cb32, cudaStream_t st);
// out[p] = in[p] - ((A_full - A_7point) x)_p over the cut cells (in == out allowed)
template <typename T>
void eb_cells(const CellGeom& g, const EbCell* C, int nc, const EbFace* F, const T* cb, const T* x, const T* in,
              T* out, cudaStream_t st);
// u -= (centroid - centre) part of beta dphi/dn on the cut faces
void eb_correct_u(const CellGeom& g, const EbFace* F, int nf, const double* const b64[3], const double* const ap[3],
                  const double* phi, gbp_array4* const u[3], cudaStream_t st);
// phi = 0 in covered cells (kap == 0), with periodic aliases
void eb_zero_covered(const CellGeom& g, const double* kap, double* phi, cudaStream_t st);
void mac_coarsen_beta(const CellGeom& gf, const CellGeom& gc, int d, const double* bf, double* bc64, float* bc32,
                      cudaStream_t st);
void mac_rhs(const CellGeom& g, const gbp_array4& ux, const gbp_array4& uy, const gbp_array4& uz, double* b,
             cudaStream_t st, const MacEB* eb = nullptr);
// ebflux = sum_d u_eb,d (ap_d(low face) - ap_d(high face)) V / h_d on the cells 0..n-1 (0 on covered
// cells): the EB inflow velocity's outflow through each cut cell's boundary, whose area vector the
// divergence theorem gives from the apertures
void mac_eb_inflow_flux(const CellGeom& g, const gbp_array4& eb_vel, const MacEB& eb, double* ebflux,
                        cudaStream_t st);
// ap (cut cells): beta / ap is the raw face beta; faces with ap == 0 are left alone
void mac_correct(const CellGeom& g, int d, const gbp_array4& u, const double* beta, const double* phi,
                 cudaStream_t st, const double* ap = nullptr);
void mac_load_phi(const CellGeom& g, const gbp_array4& in, double* phi, cudaStream_t st);
void mac_zero_faces(const CellGeom& g, int d, const gbp_array4& u, cudaStream_t st);
void mac_store_phi(const CellGeom& g, const gbp_array4& out, const double* phi, cudaStream_t st);
// max |v| / (kap V) over the cells (kap == nullptr: kap = 1; cells with kap == 0 skipped)
void mac_norm(const CellGeom& g, const double* v, unsigned long long* norm, cudaStream_t st,
              const double* kap = nullptr);
int mac_partials_needed(const CellGeom& g);
// mode 0: v -= kap sum(v) / sum(kap); mode 1: v -= sum(kap v) / sum(kap) on fluid cells, 0 on covered ones.
// nfluid = sum(kap) (the cell count without cut cells)
void mac_remove_mean(const CellGeom& g, double* v, double* partials, int mode, cudaStream_t st,
                     const double* kap = nullptr, double nfluid = 0.0);
template <typename TE>
void mac_add_correction(const CellGeom& g, double* x, const TE* e, double inv_scale, cudaStream_t st);
void mac_to_f32(const CellGeom& g, const double* r, float* r32, double scale, cudaStream_t st);

}  // namespace gbp
