// Nodal multigrid solver: the replacement of Hydro::NodalProjector + MLNodeLaplacian + MLMG for
// one single-box level (incflo::ApplyNodalProjection, src/projection/incflo_apply_nodal_projection.cpp).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "gbp_internal.cuh"
#include "nodal_kernels.h"
#include "nodal_eb.h"
#include "nodal_sweep.h"

namespace gbp {

namespace nn {
class UNet;
}

// an asynchronous copy to issue on `stream` after `ev` (recorded by the issuer) completes
struct HostCopy {
    void* dst;
    const void* src;
    size_t bytes;
    cudaStream_t stream;
    cudaEvent_t ev;
};

// The corrected cell fields copied back by z-slabs, each slab's copies issued on `stream` as soon as its
// correction is done (velocity and gp, 3 components each, component-major without ghost cells:
// component c of cell plane k starts at c * ncell + k * plane).
struct HostSlabs {
    double* hvel;
    double* hgp;
    const double* dvel;
    const double* dgp;
    size_t plane, ncell;
    int nslabs;
    cudaStream_t stream;
    cudaEvent_t* ev;  // nslabs events
};

// The right-hand side launched by groups of its z chunks, group q after event ev[q] (its cells uploaded);
// with a periodic z direction group 0 also waits for the last event (node plane 0 reads the top cells).
constexpr int kRhsGroups = 8;
struct RhsGroups {
    int n;
    int zb[kRhsGroups + 1];
    cudaEvent_t ev[kRhsGroups];
};

struct DevicePool {
    char* base = nullptr;
    size_t bytes = 0;
    size_t used = 0;
    int reserve(size_t nbytes);
    template <typename T>
    T* take(size_t count)
    {
        size_t off = (used + 255) & ~size_t(255);
        used = off + count * sizeof(T);
        return reinterpret_cast<T*>(base + off);
    }
    void release();
};

struct NodalLevel {
    NodalGeom g;
    double *s64 = nullptr, *x64 = nullptr, *t64 = nullptr, *b64 = nullptr, *r64 = nullptr;
    float *s32 = nullptr, *x32 = nullptr, *t32 = nullptr, *b32 = nullptr, *r32 = nullptr;
    unsigned char* mask8 = nullptr;  // overset mask storage (active when g.mask is set)
};

class NodalSolver {
public:
    static constexpr int kMaxInner = 8;  // FP32 V-cycles per refinement step, at most

    int init(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const gbp_options& opt,
             cudaStream_t stream);
    void destroy();
    ~NodalSolver() { destroy(); }

    int set_options(const gbp_options& opt);
    int set_sigma_from_density(const gbp_array4* rho, double scale, double rho0);
    int set_sigma(const gbp_array4* sigma, double cval);
    // overset mask (0 = phi held at 0) over nodes 0..n; nullptr removes it
    int set_mask(const gbp_iarray4* mask);
    // cut cells: moments (27 components M[p + 3 q + 9 r] = int xi^p eta^q zeta^r dV / V over the fluid
    // part of each cell, normalised coordinates in [-1/2, 1/2]); nullptr removes them. Sigma must be set
    // again afterwards.
    int set_eb(const gbp_array4* moments);
    // MLNodeLaplacian::setEBInflowVelocity: the velocity on the embedded boundary of every cell, with
    // the boundary's area vector over the face areas (dap) and its centroid (bcent), 3 components each;
    // enters the right-hand side of the next projections. eb_vel == nullptr removes it; set_eb drops it.
    int set_eb_inflow(const gbp_array4* eb_vel, const gbp_array4* dap, const gbp_array4* bcent);

    // full projection: rhs from vel (+ fused add-back / U^n subtraction), solve, correct.
    // phi_copy: a copy (e.g. p_nd to the host) issued on its own stream once phi_out is stored,
    // overlapping the velocity correction
    int project(const RhsArgs& rhs, const CorrArgs& corr, gbp_array4* phi_out, int phi_accumulate,
                const gbp_array4* phi_guess, gbp_stats* stats, const HostCopy* phi_copy = nullptr,
                const HostSlabs* out_slabs = nullptr, const RhsGroups* rhs_groups = nullptr);

    // nodal divergence of vel as the projection sees it (consistent for singular systems), strong form
    int divergence(const RhsArgs& rhs, const gbp_array4* out, double* max_norm);

    const NodalGeom& geom0() const { return L[0].g; }
    bool has_eb() const { return eb.on; }
    size_t device_bytes() const { return pool.bytes; }
    cudaStream_t stream() const { return st; }
    // solve A phi = g on the level-0 arrays already in place (used by project and tests)
    // from_prev: phi holds the plan's last solution (initial_guess = previous), a start the warm start
    // must beat
    int solve(bool have_guess, gbp_stats* stats, bool from_prev = false);

    // Preconditioner for a composite (two-level) driver: x += m V-cycles from zero on the FP64 level-0
    // residual r, in the plan's precision (FP32 V-cycles on r * scale in the mixed form). r and x are
    // level-0 arrays in the padded layout; r is not modified.
    void apply_vcycles(const double* r, double* x, int m, double scale, cudaStream_t s);
    // The same on an FP32 level-0 right-hand side already scaled (mixed form only): m FP32 V-cycles from
    // zero on b32; the correction stays in correction32() until the next V-cycle of this solver.
    void apply_vcycles32(const float* b32, int m, cudaStream_t s);
    const float* correction32() const { return (const float*)xres[0]; }
    // nu FP32 Jacobi sweeps from zero on level 0 only (b32 scaled as for apply_vcycles32); the correction
    // stays in correction32()
    void smooth32(const float* b32, int nu, cudaStream_t s);
    // For work issued through apply_vcycles / apply_vcycles32: GBP_OK, the first launch error (cleared), or
    // GBP_TIMEOUT when a bounded device wait of a level sweep ran out (the device error word is read and
    // cleared; synchronises s).
    int take_sweep_status(cudaStream_t s);
    float* sigma32() const { return L[0].s32; }

    void reset_count() { nk = 0; }
    long long kernel_count() const { return nk; }
    // time `reps` launches of one level-0 kernel (0/1: FP64/FP32 Jacobi, 2/3: FP64/FP32 residual)
    int time_kernel(int which, int reps, double* ms, double* bytes);
    // Test hook: the level-0 FP32 whole-row sweeps against the one-node-per-thread kernels on seeded
    // level-0 / level-1 data (the plan's sigma): max |new - reference| / max |reference| over every
    // padded position for [0] Jacobi, [1] residual, [2] residual + restriction (coarse level), [3]
    // prolongation + Jacobi ([2], [3] -1 with an overset mask). Overwrites solver scratch (the next solve
    // refills it).
    int check_level_kernels(double diff[4]);
    int check_level_kernels_on(float* A, float* C, double diff[4]);

    // Learned warm start for zero-guess solves: the network runs on multigrid level `level` (its
    // prediction is prolonged to level 0 and scaled by the Galerkin factor x.b / x.Ax); mode 0 off,
    // 1 on. The scaled prediction replaces the zero start only when its residual is smaller.
    int set_surrogate(nn::UNet* net, int level, int mode);
    const NodalLevel& level(int l) const { return L[l]; }
    int num_levels() const { return (int)L.size(); }

    double* phi64() const { return phi; }
    double* rhs64() const { return rhs0; }
    double* sigma64() const { return L[0].s64; }
    // r = rhs - A x in FP64 on level 0 (the operator and right-hand side of the last projection), into the
    // level-0 FP64 residual scratch; returns it (the network input of a start from x)
    double* residual_of(const double* x);

private:
    template <typename T>
    void vcycle(int l, const T* b, bool zero);
    template <typename T>
    void bottom(int l, const T* b, T* x);
    // Jacobi sweep / residual on one level: the TMA-staged sweep where the level is large enough,
    // the plain kernels on small levels
    template <typename T>
    void jacobi(const NodalGeom& g, const T* s, const T* x, const T* b, T* out, double w, cudaStream_t s_);
    template <typename T>
    void resid(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, unsigned long long* norm,
               cudaStream_t s_);
    void record_iteration(int m);
    int warm_start(double bnorm, double* rn, gbp_stats* stats, bool from_prev);
    void drop_graphs();
    int run_iteration(int m);
    int build_bottom();

    gbp_options opt{};
    cudaStream_t st = nullptr;
    cudaStream_t cap = nullptr;  // capture stream (graphs cannot be captured on the legacy stream)
    cudaStream_t cap_or_st = nullptr;  // stream the kernels of a refinement step are issued on
    std::vector<NodalLevel> L;
    DevicePool pool;
    double* phi = nullptr;       // level-0 solution (FP64)
    // the last solution (initial_guess = previous), FP64 level 0, and its injection onto the network's
    // level (the network's phi_prev input); allocated on first use
    double* phi_last = nullptr;
    bool have_last = false;
    double* net_prev = nullptr;
    size_t net_prev_count = 0;
    double* rhs0 = nullptr;      // level-0 right-hand side (FP64, weak form)
    double* res = nullptr;       // level-0 outer residual (FP64)
    double* partials = nullptr;  // reduction scratch
    double* bscr = nullptr;      // bottom CG scratch
    int* dinfo = nullptr;        // bottom iteration count
    unsigned long long* dnorm = nullptr;  // [0] rhs norm, [1] residual norm
    unsigned long long* hnorm = nullptr;  // pinned mirror
    bool singular = false;        // the system has the constants as null space (consistent RHS, gauge)
    // the FP32 levels with at most this many nodes (below the finest) run as one cluster launch per V-cycle
    // (measured at 256^3: 11.92 ms per projection against 11.98 with per-level launches and 12.12 with the
    // 33^3 level included; FP64 levels stay on per-level launches, which were faster there)
    static constexpr long long kCoarseNodes = 5000;
    bool use_coarse = true;
    int coarse_first() const;
public:
    // test hook: one FP32 V-cycle from the first cluster-cycled level on a seeded right-hand side, through
    // the per-level launches and through the cluster kernel; *diff = max |difference| / max |result|
    int check_coarse_cycle(double* diff);
private:
    double omega_eff = 0.85;  // the fixed smoother weight (see set_omega)
    // weights of the pre- and post-smoothing sweeps of a V-cycle level (sweep p: [p % kSweepWeights])
    double wpre[kSweepWeights] = {}, wpost[kSweepWeights] = {};
    void set_omega();
    bool bsing = false;           // the coarsest operator does (no node held at 0 on it)
    bool singular_faces = false;  // singular from the boundary types alone (no overset mask)
    int rebuild_masks();
    int finish_sigma();
    void resid0(const double* x, const double* b, double* r, unsigned long long* norm, cudaStream_t s);
    unsigned user_zeros = 0;
    unsigned char* umask8 = nullptr;  // the user's overset mask, level 0 (null: none)
    DevicePool auxpool;               // user mask storage
    struct EbState {
        DevicePool pool;
        EbNodal e{};
        // nodes touching fluid on each level (a coarse cell holds fluid when one of its fine cells does)
        unsigned char* active8[kMaxLevels] = {};
        double* ivol = nullptr;            // 1 / fluid volume of each node's dual cell (level 0)
        double* inflow_buf = nullptr;      // 8 EB inflow shares per cut cell (e.inflow when set)
        bool has_inactive = false;
        bool on = false;
    } eb;
    bool sigma_ready = false;
    double scale32 = 1.0;
    // result buffer of each level's V-cycle (ping-pong aware)
    void* xres[kMaxLevels] = {};
    cudaGraphExec_t gexec[kMaxInner + 1] = {};  // one refinement-step graph per inner-cycle count
    int gexec_prec = -1;
    double gexec_scale = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    static constexpr int kDenseBottomMax = 216;
    int nbottom = 0;
    bool dense_bottom = false;
    double* dmat = nullptr;      // dense inverse of the coarsest operator (transposed)
    double* dscal = nullptr;     // device scalars of the mean / gauge corrections
    unsigned* derr = nullptr;    // device error word of the TMA sweeps (bit 0: a bounded wait ran out)
    int launch_rc = 0;           // first failure while issuing a sweep (tensor-map encoding)
    bool use_tma = true;
    long long nk = 0;            // kernels issued (or replayed through graphs) since reset_count()
    long long step_kernels = 0;  // kernels in one refinement step (the last one recorded)
    long long step_kernels_m[kMaxInner + 1] = {};
    nn::UNet* net = nullptr;     // warm-start network (not owned)
    int net_level = 1, net_mode = 0;
    __nv_bfloat16* net_x0 = nullptr;  // network input tensor
    size_t net_x0_bytes = 0;
    double* net_scr = nullptr;   // 8 device doubles: input statistics, Galerkin dot products
    cudaEvent_t evw = nullptr;
    QWeights qw{};               // level-0 sigma sums of the shared-sum FP64 sweep (isotropic levels)
    bool use_qsweep = false;
    int warm_streak = 0;         // consecutive bypassed warm starts
    // cost model of a warm start, from the last solve: the per-V-cycle residual contraction and the device
    // time of one V-cycle (a candidate is taken only when the V-cycles its smaller residual saves cost more
    // than the network did)
    double vc_rho = 0.0, vc_ms = 0.0;
    cudaEvent_t evi0 = nullptr, evi1 = nullptr;
    int warm_skip = 0;           // solves left before the next attempt after a streak
};

}  // namespace gbp
