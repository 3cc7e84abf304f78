// MAC multigrid solver: the replacement of Hydro::MacProjector + MLPoisson/MLABecLaplacian + MLMG for one
// single-box level (incflo::compute_MAC_projected_velocities,
// src/convection/incflo_compute_MAC_projected_velocities.cpp:93-133, 272-299).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gbp_internal.cuh"
#include "mac_kernels.h"
#include "nodal_solver.h"

namespace gbp {

struct MacLevel {
    CellGeom g;
    double *b64[3] = {}, *x64 = nullptr, *rhs64 = nullptr, *r64 = nullptr;
    float *b32[3] = {}, *x32 = nullptr, *rhs32 = nullptr, *r32 = nullptr;
};

class MacSolver {
public:
    int init(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const gbp_options& opt,
             cudaStream_t stream);
    void destroy();
    ~MacSolver() { destroy(); }
    int set_options(const gbp_options& opt);
    // source: 0 = arrays, 1 = constant, 2 = dt / face average of rho
    int set_beta(int source, const gbp_array4* src[3], double cval);
    // Robin data of the ROBIN sides (MacProjector::setLevelBC(lev, nullptr, robin_a, robin_b,
    // robin_f)): cell arrays with one ghost layer, read in the ghost cells next to the Robin faces
    int set_robin(const gbp_array4* a, const gbp_array4* b, const gbp_array4* f);
    // cut cells of an embedded boundary (vfrac == nullptr removes them): volume fractions, area
    // fractions and face centroids (2 components, AMReX's fcx / fcy / fcz) of the finest level. The
    // face betas must be set again afterwards.
    int set_eb(const gbp_array4* vfrac, const gbp_array4* const area[3], const gbp_array4* const fcent[3]);
    bool has_eb() const { return eb.on; }
    // test hook: one FP32 V-cycle from the first cluster-cycled level on a seeded right-hand side through
    // the per-level launches and through the cluster kernel; *diff = max |difference| / max |result|
    int check_coarse_cycle(double* diff);
    // MacProjector::setEBInflowVelocity: the velocity on the embedded boundary of every cell (3
    // components, cells 0..n-1); its flux out of each cut cell enters the divergence of the next
    // projections. nullptr removes it; set_eb drops it.
    int set_eb_inflow(const gbp_array4* eb_vel);
    // ABecLaplacian on the same levels (MLABecLaplacian::setScalars / setACoeffs / setBCoeffs):
    // alpha a phi - beta div(b grad phi) = rhs; a == nullptr: the constant a0; b == nullptr: the
    // constant b0. alpha = 0 gives back the plain Poisson operator of the projections.
    // eta_cc (instead of b): b = the face average of this cell field (incflo's
    // average_scalar_eta_to_faces)
    // bscale (optional): a factor on b per face direction (the tensor solve's 4/3 on the normal faces)
    int set_abec(double alpha, const gbp_array4* a, double a0, double beta, const gbp_array4* const b[3], double b0,
                 const gbp_array4* eta_cc = nullptr, const double* bscale = nullptr);
    // MLMG::solve(phi, rhs, rtol, atol) with setLevelBC(0, &phi): phi (cells, one ghost layer on the
    // Dirichlet sides, whose ghost cells hold the boundary values) is the initial guess and the result
    int abec_solve(const gbp_array4* rhs, gbp_array4* phi, gbp_stats* stats);
    int project(gbp_array4* u[3], gbp_array4* phi_io, int phi_guess, gbp_stats* stats);
    // MacProjector::getFluxes: flux[d] = -beta grad phi on the faces 0..n of direction d, the correction
    // project() subtracts from umac (face centroids on cut faces), for a given phi (cells)
    int get_fluxes(const gbp_array4& phi_in, gbp_array4* flux[3]);
    // for a solver that uses this operator as one block of a preconditioner (the tensor solve): the
    // finest level, and e += the inner V-cycles of A e = r from zero (r in the finest padded layout,
    // homogeneous boundaries; FP32 V-cycles on r * scale32 in the mixed form)
    const CellGeom& finest() const { return L[0].g; }
    const gbp_options& options() const { return opt; }
    void add_vcycle_correction(const double* r, double* e, double scale32_);
    // its FP32 V-cycles on an FP32 right-hand side already scaled (mixed form); the correction stays in
    // correction32() until the next V-cycle of this solver
    void vcycles32(const float* b32);
    const float* correction32() const { return L[0].x32; }
    size_t device_bytes() const { return pool.bytes; }

private:
    template <typename T>
    void vcycle(int l, const T* b, bool zero);
    // r = b - A x on the finest level in FP64 (with the cut-face terms), norm = max |r| / (kap V)
    void resid64(const double* x, const double* b, double* r, unsigned long long* norm, cudaStream_t s);
    void eb_refresh_beta();
    int build_dense_bottom();
    void record_iteration(int m);  // m V-cycles per refinement step
    int run_iteration(int m);
    int solve(bool have_guess, gbp_stats* stats);

    gbp_options opt{};
    cudaStream_t st = nullptr, cap = nullptr, cap_or_st = nullptr;
    int bclo[3] = {}, bchi[3] = {};
    std::vector<MacLevel> L;
    DevicePool pool;
    double *phi = nullptr, *rhs0 = nullptr, *res = nullptr, *partials = nullptr, *bscr = nullptr;
    unsigned long long* dnorm = nullptr;
    unsigned long long* hnorm = nullptr;
    bool singular = false;
    bool beta_ready = false;
    double scale32 = 1.0;
    cudaGraphExec_t gexec = nullptr;
    int gexec_prec = -1;
    double gexec_scale = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    RobinFaces rb{};             // finest-level Robin faces (sides with GBP_BC_ROBIN)
    bool any_dirichlet = false;  // a Dirichlet side exists (the system is nonsingular)
    bool robin_ready = false;
    unsigned* dflags = nullptr;
    DevicePool apool;  // alpha a V per level (ABecLaplacian)
    // dense inverse of the coarsest operator (at most kMacDenseBottomMax cells), rebuilt with the face
    // coefficients; the single-CTA CG otherwise
    DevicePool dpool;
    double* dmat = nullptr;
    unsigned char* dact = nullptr;
    bool dense_bottom = false;
    // the FP32 levels with at most this many cells (below the finest) run as one cluster launch per V-cycle
    // (measured on the 256^3 MAC projection: 24.55 ms against 24.95 with per-level launches)
    static constexpr long long kCoarseCells = 40000;
    bool use_coarse = true;
    int coarse_first() const;
    int launch_rc = 0;  // first failure while issuing a launch (recorded during capture)
    bool abec = false;
    struct EbState {
        DevicePool pool;
        MacEB m{};
        EbFace* faces = nullptr;
        EbCell* cells = nullptr;
        int nfaces = 0, ncells = 0;
        double* cb64 = nullptr;
        float* cb32 = nullptr;
        double* flux = nullptr;    // EB inflow flux per cell (eb_inflow_flux), when m.ebflux is set
        double* beff64 = nullptr;  // finest-level right-hand side with the lagged cut-face terms
        float* beff32 = nullptr;
        double kap_sum = 0.0;
        bool on = false;
    } eb;
};

}  // namespace gbp
