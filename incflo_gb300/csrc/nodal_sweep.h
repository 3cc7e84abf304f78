// TMA-staged level sweeps of the nodal operator (nodal_sweep64.cu: FP64 and FP32 sweeps, tensor maps and
// launch helpers).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

// mode 0: Jacobi sweep out = x + omega (b - A x) / diag(A); mode 1: residual out = b - A x (with the
// strong-form max norm into *norm when norm != nullptr). err: device word, bit 0 = a bounded wait ran out.
template <typename T>
int nodal_sweep(const NodalGeom& g, int mode, const T* s, const T* x, const T* b, T* out, double omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st);
// Precomputed sigma sums of the shared-sum FP64 sweep (nodal_qsweep64.cu), one value per padded node:
// wsum = the 8 cells around the node; wx / wy / wz = the 4 cells around the edge to the +x / +y / +z
// neighbour.
struct QWeights {
    double *wsum, *wx, *wy, *wz;
};
bool qsweep_supported(const NodalGeom& g);
void nodal_qweights64(const NodalGeom& g, const double* s64, const QWeights& w, cudaStream_t st);
// mode 0: Jacobi sweep, 1: residual (+ strong-form max norm into *norm when norm != nullptr)
void nodal_qsweep64(const NodalGeom& g, int mode, const double* s64, const QWeights& w, const double* x,
                    const double* b, double* out, double omega, unsigned long long* norm, cudaStream_t st);

// whether the TMA sweep handles this level for elements of esize bytes (else the plain kernels do)
bool sweep_supported(const NodalGeom& g, int esize);
void sweep_forget_maps(const void* pool_base, size_t pool_bytes);

// helpers shared by the two sweep files
int make_tensor_map(const void* base, int esize, long long sy, long long sz, long long count, int boxx, int rows,
                    CUtensorMap* out);
// cuTensorMapEncodeTiled from the driver (nullptr when unavailable)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
int sweep_z_chunks(const NodalGeom& g, int xy_tiles, int resident);
int sm_count_cached();
int sweep32_run(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st);

// FP32 whole-row sweeps with fused grid transfers (nodal_vsweep32.cu), isotropic levels whose rows hold
// at most 512 nodes (Jacobi and residual also with an overset mask: masked nodes are held at 0).
bool vsweep32_supported(const NodalGeom& g);
// ... and whose coarse level is the standard coarsening by 2 (residual + restriction, prolongation + sweep),
// neither of them with an overset mask
bool vsweep32_transfer_supported(const NodalGeom& g, const NodalGeom& gc);
// mode 0: Jacobi sweep, 1: residual
int vsweep32(const NodalGeom& g, int mode, const float* s, const float* x, const float* b, float* out, float omega,
             unsigned* err, cudaStream_t st);
// bc (the coarse right-hand side) = full-weighting restriction of b - A x
int vsweep32_resid_restrict(const NodalGeom& g, const NodalGeom& gc, const float* s, const float* x, const float* b,
                            float* bc, unsigned* err, cudaStream_t st);
// out = one Jacobi sweep from x + P ec (ec: the coarse correction)
int vsweep32_prolong_jacobi(const NodalGeom& g, const NodalGeom& gc, const float* s, const float* x, const float* ec,
                            const float* b, float* out, float omega, unsigned* err, cudaStream_t st);
void vsweep32_forget_maps(const void* pool_base, size_t pool_bytes);

}  // namespace gbp
