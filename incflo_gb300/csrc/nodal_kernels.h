// Host-side launchers of the nodal projection kernels (nodal_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "gbp_internal.cuh"

namespace gbp {

// Inputs of the fused right-hand-side kernel: u' = u + (add_gp ? sigma*gp : 0) - (sub_old ? u_old : 0)
struct RhsArgs {
    gbp_array4 vel;
    gbp_array4 gp;
    gbp_array4 vel_old;
    int add_gp;
    int sub_old;
    int inflow_lo[3];
    int inflow_hi[3];
    double cf[3];  // h_e h_f / 4: integral of dN/dx_d over one cell, up to sign
    // cells that take part (padded cell layout, periodic aliases filled; nullptr = all): the leaf
    // cells of a level in a composite (AMR) projection
    const unsigned char* cmask;
};

// Outputs of the fused correction kernel.
struct CorrArgs {
    gbp_array4 vel;
    gbp_array4 gp;       // data == nullptr: not written
    gbp_array4 gradphi;  // data == nullptr: not written
    int add_gp;
    int incremental;
    double inv4h[3];
    const unsigned char* cmask;  // cells to update (padded cell layout), nullptr = all
};

template <typename T>
void nodal_jacobi(const NodalGeom& g, const T* s, const T* xin, const T* b, T* xout, double omega, bool zero,
                  cudaStream_t st);
template <typename T>
void nodal_resid(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, unsigned long long* norm,
                 cudaStream_t st);
template <typename T>
void nodal_restrict(const NodalGeom& gf, const NodalGeom& gc, const T* rf, T* bc, cudaStream_t st);
// r = b - A x at the n listed unique nodes (i, j, k) only
template <typename T>
void nodal_resid_list(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, const int4* nodes, int n,
                      cudaStream_t st);
template <typename T>
void nodal_prolong_add(const NodalGeom& gf, const NodalGeom& gc, const T* xc, T* xf, cudaStream_t st);
template <typename T>
void nodal_bottom(const NodalGeom& g, const double* s64, const T* b, T* x, double* scratch, int maxiter,
                  double rtol, double atol, int* info, int singular, cudaStream_t st);

template <typename T>
void nodal_bottom_dense(const NodalGeom& g, const double* M, const T* b, T* x, int singular, cudaStream_t st);

// The coarse end of a V-cycle in one launch: levels 0 .. nl-1 of this struct (a tail of the hierarchy
// whose last level is the bottom, solved with the dense inverse M) cycled from a zero start by one
// thread-block cluster, its CTAs meeting at cluster barriers between the phases (the smoothing sweeps,
// residual, restriction, bottom and prolongation of each level). Level data stays in L2 and is read
// with L2-coherent loads.
constexpr int kCoarseMaxLevels = 10;
// weights of the smoothing sweeps of one V-cycle level (pre and post each), repeated beyond this count
constexpr int kSweepWeights = 8;
template <typename T>
struct CoarseCycle {
    int nl;  // levels, >= 2 (at least one above the bottom)
    NodalGeom g[kCoarseMaxLevels];
    const T* s[kCoarseMaxLevels];
    T* x[kCoarseMaxLevels];
    T* t[kCoarseMaxLevels];
    T* b[kCoarseMaxLevels];  // b[0]: the right-hand side of the first level (written by the caller)
    T* r[kCoarseMaxLevels];
    const double* M;         // dense inverse of the bottom operator
    int singular;            // the bottom has the constants as null space
    T wpre[kSweepWeights];   // Jacobi weight of pre-smoothing sweep p: wpre[p % kSweepWeights]
    T wpost[kSweepWeights];  // ... and of post-smoothing sweep p
    int nu1, nu2;
};
constexpr int kCoarseThreads = 1024;
// cluster size the device co-schedules for the kernel: 16 (non-portable) when possible, else 8
int nodal_coarse_cluster_size();
template <typename T>
int nodal_coarse_vcycle(const CoarseCycle<T>& c, int cluster, cudaStream_t st);
// which buffer of level 0 of the struct holds the result after nodal_coarse_vcycle: 0 = x, 1 = t (the
// host's copy of the kernel's ping-pong)
int coarse_result_slot(int nu1, int nu2);

void nodal_sigma_from_rho(const NodalGeom& g, const gbp_array4* rho, double scale, double rho0, double* s64,
                          float* s32, cudaStream_t st);
void nodal_sigma_copy(const NodalGeom& g, const gbp_array4* sig, double cval, double* s64, float* s32,
                      cudaStream_t st);
void nodal_sigma_coarsen(const NodalGeom& gf, const NodalGeom& gc, const double* sf, double* sc64, float* sc32,
                         cudaStream_t st);
// part: per-block sums of the right-hand side (nodal_rhs_partials(g) of them), or nullptr
// z chunks zb0 .. zb1-1 of the launch grid (zb1 < 0: all); the partial sums keep their full-grid slots
void nodal_rhs(const NodalGeom& g, const RhsArgs& a, const double* s64, double* b, double* part, cudaStream_t st,
               int zb0 = 0, int zb1 = -1);
// number of z chunks of the right-hand-side launch and the node planes per chunk
int nodal_rhs_zchunks(const NodalGeom& g, int* kchunk);
int nodal_rhs_partials(const NodalGeom& g);
// mode 0: make b consistent (remove V-weighted mean; max norm of the result into *norm);
// mode 1: gauge x to zero V-weighted mean. have_partials: `partials` already holds nparts sums of v.
void nodal_remove_mean(const NodalGeom& g, double* v, double* partials, double* scal, int mode, int have_partials,
                       int nparts, unsigned long long* norm, cudaStream_t st);
void nodal_fold(const NodalGeom& g, const double* part, int nparts, double* scal, cudaStream_t st);
int nodal_partials_needed(const NodalGeom& g);
void nodal_norm(const NodalGeom& g, const double* v, unsigned long long* norm, cudaStream_t st);
template <typename TE>
void nodal_add_correction(const NodalGeom& g, double* x, const TE* e, double inv_scale, cudaStream_t st);
void nodal_to_f32(const NodalGeom& g, const double* r, float* r32, double scale, cudaStream_t st);
// cell planes k0 .. k1-1 (k1 < 0: to the last plane)
void nodal_correct(const NodalGeom& g, const CorrArgs& a, const double* s64, const double* phi, cudaStream_t st,
                   int k0 = 0, int k1 = -1);
void nodal_store_phi(const NodalGeom& g, const gbp_array4& out, const double* phi, int accumulate, cudaStream_t st);
void nodal_load_phi(const NodalGeom& g, const gbp_array4& in, double* phi, cudaStream_t st);
// streaming reference: out = a + b + c over n floats (n a multiple of 4, 16-byte aligned arrays)
void stream_triad(const float* a, const float* b, const float* c, float* out, long long n, cudaStream_t st);
// strong-form divergence -b_i / V_i into a nodal array (all nodes 0..n)
void nodal_store_div(const NodalGeom& g, const gbp_array4& out, const double* b, cudaStream_t st);
// overset mask: level 0 from the caller's int array (zeros counted into *zeros); a coarse node is free where
// every fine node of its support is
void nodal_mask_load(const NodalGeom& g, const gbp_iarray4& m, unsigned char* out, unsigned* zeros, cudaStream_t st);
void nodal_mask_coarsen(const NodalGeom& gf, const NodalGeom& gc, const unsigned char* mf, unsigned char* mc,
                        cudaStream_t st);

}  // namespace gbp
