// Two-level (AMR) composite nodal projection: incflo::ApplyNodalProjection over finest_level = 1
// (src/projection/incflo_apply_nodal_projection.cpp:95-267) with one NodalProjector over both levels
// (:187-192) and MLNodeLaplacian's composite solve (:215).
//
// Discretisation: conforming Q1 elements on the composite mesh. Leaf cells are the fine cells of the
// fine boxes (ratio 2) and the coarse cells they do not cover; unknowns are the uncovered coarse nodes
// and the fine nodes strictly inside the fine region; fine nodes on the coarse-fine interface at coarse
// positions are those coarse nodes, the others hang (linear / bilinear interpolation along the coarse
// face). A = P^T (sum over leaf cells) P, b = P^T (sum over leaf cells of int u . grad N).
//
// Data: the coarse level as one box (a NodalSolver over the domain); the fine level on the bounding box
// of its boxes (a second NodalSolver, sigma zero outside the fine cells, its overset mask holding every
// node but the fine unknowns). Solver: FP64 composite residual (fine residual with the interface values
// filled from the coarse level, coarse residual with sigma zero on covered cells, plus the fine interface
// residuals restricted to their coarse nodes), then one two-level correction per step: coarse V-cycles
// on the restricted composite residual (prolonged trilinearly to the fine unknowns), a fresh fine
// residual, fine V-cycles on the fine unknowns with the interface held. In the mixed form the FP64
// composite residual is the right-hand side of a correction equation that several such steps solve in
// FP32 arithmetic before the next FP64 residual (iterative refinement, as in the single-level solve).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "incflo_gb300.h"
#include "nodal_solver.h"
#include "nodal_sweep.h"

namespace gbp {

struct AmrBox {
    int lo[3], hi[3];  // fine cells, inclusive, in the fine index space of the whole domain
};

struct AmrFields {
    gbp_array4* vel_c;
    const gbp_array4* vel_old_c;
    const gbp_array4* rho_c;
    gbp_array4* gp_c;
    gbp_array4* p_c;
    gbp_array4* const* vel_f;       // nbox entries each; NULL arrays allowed where optional
    const gbp_array4* const* vel_old_f;
    const gbp_array4* const* rho_f;
    gbp_array4* const* gp_f;
    gbp_array4* const* p_f;
    double rho0, scale;
    int incremental;
};

class CompositeNodal {
public:
    int init(const gbp_geometry& coarse, const int bc_lo[3], const int bc_hi[3], const int* boxes, int nbox,
             const gbp_options& opt, cudaStream_t stream);
    ~CompositeNodal();
    int project(const AmrFields& f, gbp_stats* stats);
    size_t device_bytes() const;
    int set_options(const gbp_options& o);

private:
    int check_fields(const AmrFields& f);
    void composite_residual(const double* bc, const double* bf, unsigned long long* norm);
    void sync(double* vc, const double* vf);
    void resid_f(const double* x, const double* b, double* r);
    void resid_c(const double* x, const double* b, double* r);

    gbp_options opt{};
    cudaStream_t st = nullptr;
    gbp_geometry geom_c{};
    int bclo[3] = {}, bchi[3] = {};
    std::vector<AmrBox> boxes;
    int off[3] = {};   // fine bounding box origin (fine cells)
    int nfb[3] = {};   // fine bounding box extent (fine cells)
    NodalSolver crs, fin;
    NodalGeom gc{}, gf{}, gf_nomask{};
    bool singular = false;
    DevicePool pool;
    unsigned char *cmask_c = nullptr, *cmask_f = nullptr, *ccls = nullptr, *fcls = nullptr;
    double *sc_m = nullptr;                                       // coarse sigma, covered cells 0
    double *sc_t = nullptr;                                       // coarse sigma s / rho on every cell
    double *phi_c = nullptr, *b_c = nullptr, *r_c = nullptr, *rc_full = nullptr, *e_c = nullptr;
    double *phi_f = nullptr, *b_f = nullptr, *r_f = nullptr;
    double *vel_f = nullptr, *gp_f = nullptr, *rho_f = nullptr, *velo_f = nullptr, *sig_f = nullptr;
    double *p_fb = nullptr;                                       // fine phi on all bbox nodes 0..n
    double *scal = nullptr, *part = nullptr;
    int nparts = 0;
    unsigned long long *dnorm = nullptr, *hnorm = nullptr;
    bool qsw = false;      // shared-sum FP64 residuals (isotropic cells)
    bool have_last = false;  // phi_c / phi_f hold the last converged solution (initial_guess = previous)
    QWeights qwf{}, qwc{};  // their edge weights, fine and coarse
    void* dboxes = nullptr;  // device table for the batched box kernels
    size_t dboxes_bytes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // one refinement step (restriction, coarse V-cycles, prolongation, fine V-cycles, composite residual
    // and its norm read-back) captured as a CUDA graph and replayed; recaptured when the FP32 scale or
    // the options change
    void issue_step(double scale32);
    // the mixed form's step: kInner FP32 two-level steps on the correction equation per FP64 composite
    // residual
    void issue_outer32(double scale32);
    template <typename T>
    void restrict_to_coarse(const T* rc, const T* rf, T* out);
#ifndef GBP_AMR_INNER
#define GBP_AMR_INNER 8
#endif
    static constexpr int kInner = GBP_AMR_INNER;
#ifndef GBP_AMR_FINE_SWEEPS
#define GBP_AMR_FINE_SWEEPS 2
#endif
    // the fine correction of a mixed-form two-level step: 0 = one V-cycle of the fine hierarchy, n > 0 = n
    // Jacobi sweeps on the fine level only (the coarse V-cycle already corrects every scale above the fine
    // spacing; measured on the 256^3 tagged workload: V-cycle 102.1 ms, 2 sweeps 75.9 ms, 4 sweeps 86.4 ms,
    // each in 2 refinement steps of 8 two-level steps)
    static constexpr int kFineSweeps = GBP_AMR_FINE_SWEEPS;
    float *bc32 = nullptr, *rc32 = nullptr, *ec32 = nullptr, *rcf32 = nullptr, *scm32 = nullptr;  // coarse
    float *bf32 = nullptr, *rf32 = nullptr, *ef32 = nullptr;                                       // fine
    // FP32 residual of one composite part: the whole-row sweep where it applies
    void resid32(const NodalGeom& g, const float* s, const float* x, const float* b, float* r);
    // the inner steps' transfers through the fine box coarsened by 2 (the fine solver's level 1, g1n
    // without its mask): the standard full weighting / trilinear kernels plus a gather and a combine
    bool xfer1 = false;
    NodalGeom g1n{};
    float *rm32 = nullptr, *x1_32 = nullptr;  // rm32: the fine interface nodes' FP32 residuals
    // the fine interface nodes (aligned and hanging), (i, j, k) each: their values and residuals of the
    // inner steps are computed over this list instead of the whole bounding box
    int4* iface = nullptr;
    int niface = 0;
    unsigned* derr = nullptr;  // device error word of the whole-row sweeps issued here
    int launch_rc = 0;         // first launch error of a step (tensor-map set-up)
    int sweep_status();
    cudaStream_t capst = nullptr;
    cudaGraphExec_t gstep = nullptr;
    double gstep_scale = 0.0;
    int gstep_prec = -1;
};

}  // namespace gbp
