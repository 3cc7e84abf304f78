// Cut cells (embedded boundary) in the nodal projection: device tables and launchers (nodal_eb.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"
#include "nodal_kernels.h"

namespace gbp {

constexpr int kEbRegular = -1, kEbCovered = -2;

// A cut cell: its exact Q1 element matrix over the fluid part (K, row-major 8 x 8, without sigma),
// int grad N over the fluid part (G, 8 x 3) and grad N at the fluid centroid (Gc, 8 x 3); corner b of
// the cell is node p + (b & 1) + ((b >> 1) & 1) sy + (b >> 2) sz.
struct EbNodeCell {
    long long p;  // padded index of the cell (= of its low corner node)
    int i, j, k;
    double K[64];
    double G[24];
    double Gc[24];
};

// A node that touches at least one cut cell; cell[c] for its cell (i - 1 + (c & 1), j - 1 + ((c >> 1) & 1),
// k - 1 + (c >> 2)): index into the cut-cell table, kEbRegular or kEbCovered.
struct EbNodeEntry {
    int i, j, k;
    int cell[8];
};

struct EbNodal {
    const EbNodeEntry* nodes;
    const EbNodeCell* cells;
    int nnodes, ncells;
    const double* sig64;       // true sigma of the level (padded cells, aliases)
    const float* sig32;
    const double* kap;         // volume fraction (padded cells, aliases)
    const unsigned char* reg;  // 1 on regular cells (volume fraction 1)
    // EB inflow: F_c N_b(x_b) for corner b of cut cell c (8 per cell), F_c the EB inflow velocity's flux
    // out of the cell's fluid and x_b its boundary centroid; subtracted from the right-hand side of the
    // corner nodes. nullptr: the boundary carries no flux.
    const double* inflow;
};

// out = Jacobi update (mode 0) or residual (mode 1) on the EB nodes, from x and b
template <typename T>
void eb_nodes(const NodalGeom& g, const EbNodal& e, int mode, const T* x, const T* b, T* out, double omega,
              cudaStream_t st);
void eb_rhs(const NodalGeom& g, const EbNodal& e, const RhsArgs& a, double* rhs, cudaStream_t st);
// out[8 c + b] = F_c N_b(bcent_c) over the cut cells: F_c = sum_d eb_vel_d dap_d V / h_d (dap: the
// boundary's area vector over the cell's face areas, bcent: the boundary centroid in cell widths from
// the cell centre; 3 components each, cell arrays)
void eb_inflow_shares(const NodalGeom& g, const EbNodal& e, const gbp_array4& eb_vel, const gbp_array4& dap,
                      const gbp_array4& bcent, double* out, cudaStream_t st);
void eb_correct(const NodalGeom& g, const EbNodal& e, const CorrArgs& a, const double* phi, cudaStream_t st);
// s_in (the level's sigma as set) -> true sigma (e.sig64 / sig32), s64 / s32 = sigma on regular cells,
// sk = sigma x volume fraction (the coarsening source)
void eb_sigma(const NodalGeom& g, const EbNodal& e, const double* s_in, double* s64, float* s32, double* sk,
              cudaStream_t st);
// out = a AND b elementwise (a null array counts as all ones)
void mask_and(long long count, const unsigned char* a, const unsigned char* b, unsigned char* out, cudaStream_t st);
// max |v| / fluid volume of the node over the unique non-Dirichlet nodes (the stopping norm with cut cells)
void eb_norm(const NodalGeom& g, const double* v, const double* ivol, unsigned long long* norm, cudaStream_t st);
// dense copy (x fastest) of component c of a cell array over cells 0..n-1
void eb_pack_cells(const gbp_array4& in, int c, const int n[3], double* out, cudaStream_t st);

}  // namespace gbp
