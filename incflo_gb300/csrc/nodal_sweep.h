// TMA-staged level sweeps of the nodal operator (nodal_sweep.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

// mode 0: Jacobi sweep out = x + omega (b - A x) / diag(A); mode 1: residual out = b - A x (with the
// strong-form max norm into *norm when norm != nullptr). err: device word, bit 0 = a bounded wait ran out.
template <typename T>
int nodal_sweep(const NodalGeom& g, int mode, const T* s, const T* x, const T* b, T* out, double omega,
                unsigned* err, unsigned long long* norm, cudaStream_t st);
bool sweep_supported(const NodalGeom& g);
void sweep_forget_maps(const void* pool_base, size_t pool_bytes);

}  // namespace gbp
