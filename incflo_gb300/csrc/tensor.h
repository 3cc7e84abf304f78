// Tensor (velocity) diffusion: DiffusionTensorOp::diffuse_velocity and compute_divtau
// (src/diffusion/DiffusionTensorOp.cpp:104-317), the work incflo hands to AMReX's MLTensorOp.
//
//   alpha a u - beta div tau = rhs,  tau = eta (grad u + grad u^T) - (2/3) eta (div u) I
//
// Cell-centred, one box. Discretisation: fluxes on faces; on a face normal to d the normal derivative of
// every component is the two-cell difference and the tangential derivative along e the mean of the
// centred differences of the two cells beside the face, with ghost cells filled direction by direction
// (Dirichlet 2 u_b - u_inner, Neumann u_inner, periodic wrap; the face values continued past an edge).
//
// Solver: defect correction. Each step takes the FP64 residual of the full operator and, per component,
// one V-cycle of its ABecLaplacian block (the normal-derivative part: b = 4/3 eta on the
// component's own faces, eta on the others, the component's boundary types) on a MacSolver hierarchy;
// the cross-derivative terms only enter the residual (as MLTensorOp treats them). The blocks' V-cycles run
// in FP32 (mixed form) or FP64. In the mixed form several block steps solve the correction equation of one
// FP64 residual in FP32 (the full operator's residual in FP32 between them, homogeneous boundary values).
#pragma once

#include <cuda_runtime.h>

#include "incflo_gb300.h"
#include "mac_solver.h"

namespace gbp {

class TensorSolver {
public:
    // bc_lo / bc_hi: [3 * component + direction], GBP_BC_PERIODIC / DIRICHLET / NEUMANN (INFLOW counts
    // as Dirichlet)
    int init(const gbp_geometry& geom, const int bc_lo[9], const int bc_hi[9], const gbp_options& opt,
             cudaStream_t stream);
    ~TensorSolver();
    // eta: cell field averaged to faces (eta_cc), face arrays (eta_f), or the constant eta0
    int set_coeffs(double alpha, const gbp_array4* a, double a0, double beta, const gbp_array4* eta_cc,
                   const gbp_array4* const eta_f[3], double eta0);
    int set_options(const gbp_options& o);
    // vel: 3 components, one ghost layer; its ghost cells next to the Dirichlet faces hold the boundary
    // values; the interior is the initial guess and receives the result
    int solve(const gbp_array4& rhs, gbp_array4& vel, gbp_stats* stats);
    // divtau = div tau of vel (with the boundary values in its ghost cells)
    int apply(const gbp_array4& vel, gbp_array4& divtau);
    size_t device_bytes() const;

private:
    int check_vel(const gbp_array4& v, bool need_ghosts) const;
    void load(const gbp_array4& vel);
    void fill_ghosts(const gbp_array4& vel);
    void fluxes();  // tau on every face, once per face

    gbp_options opt{};
    cudaStream_t st = nullptr;
    gbp_geometry geom{};
    int bclo[9] = {}, bchi[9] = {};
    MacSolver comp[3];
    DevicePool pool;
    double* u[3] = {};
    double* rhs[3] = {};
    double* r[3] = {};
    double* eta[3] = {};
    double* fl[3][3] = {};  // [face direction][component]: tau_{c,d} on the faces of direction d
    // the mixed form's FP32 inner steps: correction, scaled FP64 residual, FP32 residual, face eta, fluxes
#ifndef GBP_TENSOR_INNER
#define GBP_TENSOR_INNER 6
#endif
    static constexpr int kInner = GBP_TENSOR_INNER;  // block steps per FP64 residual
    float* e32[3] = {};
    float* b32[3] = {};
    float* r32[3] = {};
    float* eta32[3] = {};
    float* fl32[3][3] = {};
    double alpha = 0.0, beta = 0.0;
    bool ready = false;
    unsigned long long *dnorm = nullptr, *hnorm = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

}  // namespace gbp
