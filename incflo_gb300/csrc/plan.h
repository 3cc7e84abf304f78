// The object behind the C ABI's gbp_plan handle (shared by the ABI translation units).
#pragma once

#include <cuda_runtime.h>

#include "incflo_gb300.h"
#include "mac_solver.h"
#include "nodal_solver.h"

constexpr int kHostSlabs = 8;

struct gbp_plan {
    int kind;
    cudaStream_t stream;
    gbp_geometry geom;
    int bc_lo[3], bc_hi[3];
    gbp::NodalSolver* nodal = nullptr;
    gbp::MacSolver* mac = nullptr;
    // device staging for the host-buffer entry point, and the stream / events that overlap its
    // copies with the solve
    double* hbuf = nullptr;
    size_t hbuf_bytes = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_in = nullptr, ev_phi = nullptr, ev_out = nullptr;
    cudaEvent_t ev_slab[kHostSlabs] = {};  // one per z-slab of the copy-out
    cudaEvent_t ev_rhs[gbp::kRhsGroups] = {};  // one per z-slab of the upload
    double* dflux = nullptr;  // 2 device doubles: inflow / outflow of the solvability fix
    double* ccbuf = nullptr;  // cell-centred projection scratch (unprojected face velocities, phi)
    // multi-box levels: single-box staging of the fields and the device table of per-FAB transfers
    void* boxbuf = nullptr;
    size_t boxbuf_bytes = 0;
    void* boxtab = nullptr;
    size_t boxtab_bytes = 0;
};
