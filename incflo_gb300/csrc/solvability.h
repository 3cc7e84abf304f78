// Inflow/outflow solvability (HydroUtils::enforceInOutSolvability as incflo calls it).
#pragma once

#include <cuda_runtime.h>

#include "incflo_gb300.h"

namespace gbp {

// cell-centred velocity (3 components) whose ghost cells hold the boundary values
int enforce_inout_cell(const gbp_geometry& geom, const int dd_lo[3], const int dd_hi[3], const gbp_array4& vel,
                       double* flux, cudaStream_t st);
// face velocities u[0..2] (one component each), boundary faces 0 and n
int enforce_inout_faces(const gbp_geometry& geom, const int dd_lo[3], const int dd_hi[3], const gbp_array4* u,
                        double* flux, cudaStream_t st);

// amrex::average_down of ncomp cell components over the coarse box [lo, hi]
int average_down(const gbp_array4& fine, const gbp_array4& crse, const int ratio[3], int ncomp, const int lo[3],
                 const int hi[3], cudaStream_t st);

}  // namespace gbp
