// incflo::ApplyCCProjection (src/projection/incflo_apply_cc_projection.cpp:199-487), one level, non-EB.
#pragma once

#include <cuda_runtime.h>

#include "incflo_gb300.h"
#include "mac_solver.h"

namespace gbp {

struct CcArgs {
    gbp_array4 vel;      // 3 comps, one ghost layer (inflow ghosts hold the inflow velocity)
    gbp_array4 vel_old;  // data == nullptr unless sub_old
    gbp_array4 rho;      // data == nullptr: constant density rho0 (ghost across Dirichlet faces used)
    gbp_array4 gp;       // data == nullptr: not written
    gbp_array4 p_cc;     // data == nullptr: not written
    double rho0, s;
    int add_gp, sub_old, use_inflow, incremental;
};

// umac[3]: face velocities written (projected) by the call; scratch: cc_scratch_doubles(geom) doubles
int cc_projection(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const CcArgs& a,
                  gbp_array4* umac[3], double* scratch, MacSolver& mac, gbp_stats* stats, cudaStream_t st);
size_t cc_scratch_doubles(const gbp_geometry& geom);

}  // namespace gbp
