/*
 * incflo_gb300 -- GB300-native projection hot path of incflo behind a C ABI.
 *
 * The reference drives two C++ classes from AMReX-Hydro, not a C ABI:
 *   Hydro::NodalProjector, created per call in
 *     incflo::ApplyNodalProjection  (src/projection/incflo_apply_nodal_projection.cpp:29-267,
 *     constructor :187-192, setDomainBC :194, project :215, getPhi :218, getGradPhi :219)
 *   Hydro::MacProjector, held as incflo::macproj (src/incflo.H:420) and driven by
 *     incflo::compute_MAC_projected_velocities
 *     (src/convection/incflo_compute_MAC_projected_velocities.cpp:93-133 init/update,
 *      :272 setUMAC, :287-299 project).
 * Every entry point below replaces one of those calls; the one it replaces is cited beside it.
 * The header-only C++ shim include/gb_projectors.H re-exposes the Hydro method names.
 *
 * Conventions
 *  - All field pointers are DEVICE pointers unless an entry point says otherwise. They are
 *    described by gbp_array4, a plain mirror of amrex::Array4: element (i,j,k,n) lives at
 *    data[(i-lo[0]) + (j-lo[1])*jstride + (k-lo[2])*kstride + n*nstride], where lo/hi bound
 *    the allocated region including ghost cells, in the global index space of the level.
 *    AMReX MultiFab FABs therefore pass through with zero copies.
 *  - Cell-centred data is valid on cells 0..n-1; nodal data on nodes 0..n; face data in
 *    direction d on faces 0..n[d] (and cells in the other two directions).
 *  - Every call returns a gbp_status (never aborts) and runs on the plan's CUDA stream.
 *  - The library computes in FP64 (plain form) or FP32 V-cycles inside FP64 iterative
 *    refinement (mixed form); it never falls back to the CPU.
 */
#ifndef INCFLO_GB300_H
#define INCFLO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBP_ABI_VERSION 3

typedef enum {
    GBP_OK = 0,
    GBP_NOT_CONVERGED = 1, /* maxiter reached before max(rtol*|b|, atol) */
    GBP_NAN = 2,           /* a residual norm became NaN or Inf */
    GBP_BAD_ARG = 3,       /* invalid pointer, size, layout or option */
    GBP_CUDA_ERROR = 4,    /* a CUDA runtime call failed; see gbp_last_error() */
    GBP_TIMEOUT = 5,       /* a bounded device-side wait ran out */
    GBP_NO_DEVICE = 6      /* no CUDA device, or not an sm_103 device */
} gbp_status;

typedef enum { GBP_NODAL = 0, GBP_MAC = 1 } gbp_kind;

/* Mirrors amrex::LinOpBCType as produced by incflo::get_projection_bc and
 * incflo::get_mac_projection_bc (src/projection/incflo_projection_bc.cpp:5-79). */
typedef enum {
    GBP_BC_PERIODIC = 0,
    GBP_BC_DIRICHLET = 1, /* pressure_inflow / pressure_outflow: phi = 0 */
    GBP_BC_NEUMANN = 2,   /* slip / no-slip wall */
    GBP_BC_INFLOW = 3,    /* mass_inflow / direction_dependent (nodal): Neumann for phi, the
                             normal inflow velocity from the ghost cells enters the RHS */
    GBP_BC_ROBIN = 4      /* mixed (MAC plans): a phi + b dphi/dn = 0 per boundary face, data
                             from gbp_mac_set_robin; nodal plans reject it */
} gbp_bc;

typedef enum { GBP_PREC_FP64 = 0, GBP_PREC_MIXED = 1 } gbp_precision;

typedef struct {
    double* data;
    int lo[3];
    int hi[3];
    int ncomp;
    long long jstride;
    long long kstride;
    long long nstride;
} gbp_array4;

/* Integer mirror of amrex::Array4<int> (one component): the overset mask. */
typedef struct {
    const int* data;
    int lo[3];
    int hi[3];
    long long jstride;
    long long kstride;
} gbp_iarray4;

typedef struct {
    int n_cell[3];       /* cells of the (single-box) level */
    double prob_lo[3];
    double prob_hi[3];
} gbp_geometry;

/* Solver options. gbp_options_default() gives incflo's defaults (src/incflo.H:425-455,
 * src/setup/init.cpp:165-177) and the MLMG defaults incflo relies on; gbp_options_set()
 * accepts the ParmParse keys of the nodal_proj.* / mac_proj.* prefixes. */
typedef struct {
    double rtol;                 /* mg_rtol  (1e-11) */
    double atol;                 /* mg_atol  (1e-14) */
    int max_coarsening_level;    /* mg_max_coarsening_level (100) */
    int maxiter;                 /* maxiter (nodal 100, mac 200) */
    int bottom_maxiter;          /* bottom_maxiter (200) */
    double bottom_rtol;          /* bottom_rtol (1e-4) */
    double bottom_atol;          /* bottom_atol (-1: unused) */
    int verbose;                 /* verbose (0) */
    int bottom_verbose;          /* bottom_verbose (0) */
    int precision;               /* precision = fp64 | mixed  (new key; default fp64) */
    int nu1;                     /* num_pre_smooth  (2) */
    int nu2;                     /* num_post_smooth (2) */
    double omega;                /* Jacobi weight of the nodal smoother (0.85, capped for stretched cells);
                                    0 = per-sweep weights from the Chebyshev roots on [lb/4, lb], lb the
                                    Gershgorin bound of the Jacobi-scaled operator */
    int ir_inner_cycles;         /* mixed form: at most this many FP32 V-cycles per FP64
                                    refinement step (5); fewer when the observed contraction
                                    says fewer reach the tolerance */
    int use_graphs;              /* capture each V-cycle as a CUDA graph (1) */
    int always_use_bnorm;        /* relative tolerance against |b| (1) or |r0| (0) */
    int initial_guess;           /* initial_guess = zero (0, incflo's: every projection starts from
                                    phi = 0) | previous (1, nodal plans: start from the plan's last
                                    solution, the setting of a time-stepping run; with a learned
                                    warm start attached, the network predicts the increment on top
                                    of it and is bypassed when its residual is not below the
                                    previous-phi start's) */
} gbp_options;

typedef struct {
    int status;
    int vcycles;                 /* V-cycles over all refinement steps */
    int outer_iters;             /* FP64 residual evaluations (refinement steps + 1) */
    int num_levels;
    double rhs_norm;             /* max_i |b_i| (strong form: the divergence) */
    double initial_rel_resid;
    double final_rel_resid;      /* max_i |b_i - (L phi)_i| / rhs_norm */
    double ms_total;             /* device time of the whole call, CUDA events */
    double ms_solve;             /* device time of the solve alone */
    long long kernel_launches;   /* kernels this call ran on the device (graph nodes included) */
    int warm_start;              /* learned warm start: 0 not attached, 1 used, 2 bypassed,
                                    3 skipped (the two attempts before were bypassed; the plan
                                    retries after 16 skipped solves) */
    double warm_rel_resid;       /* residual of the scaled prediction / rhs_norm (when attempted) */
    double ms_warm;              /* device time of the warm start (network + scaling + residual) */
    double prev_rel_resid;       /* initial_guess = previous: residual of the previous-phi start /
                                    rhs_norm (0 when the solve started from zero) */
} gbp_stats;

typedef struct gbp_plan gbp_plan;

/* ---- library ------------------------------------------------------------------------- */
int         gbp_abi_version(void);
const char* gbp_status_string(int status);
const char* gbp_last_error(void);
int         gbp_device_check(void);

/* ---- options: the nodal_proj.* / mac_proj.* inputs surface ---------------------------- */
int gbp_options_default(int kind, gbp_options* opt);
/* key without prefix, e.g. "mg_rtol", "maxiter", "bottom_solver", "precision" */
int gbp_options_set(gbp_options* opt, const char* key, const char* value);
/* parse ParmParse-style text ("prefix.key = value" lines, '#' comments) for one prefix */
int gbp_options_parse(gbp_options* opt, const char* prefix, const char* text);

/* ---- plans ----------------------------------------------------------------------------
 * A plan owns the multigrid hierarchy for one level geometry and boundary set. It replaces
 * the per-call construction of Hydro::NodalProjector
 * (incflo_apply_nodal_projection.cpp:124,187-194) and Hydro::MacProjector construction plus
 * setDomainBC (src/incflo.cpp:286-292, incflo_compute_MAC_projected_velocities.cpp:93-114).
 * stream: a cudaStream_t (NULL = legacy default stream). */
int gbp_plan_create(const gbp_geometry* geom, int kind, const int bc_lo[3], const int bc_hi[3],
                    const gbp_options* opt, void* stream, gbp_plan** plan);
int gbp_plan_destroy(gbp_plan* plan);
int gbp_plan_set_options(gbp_plan* plan, const gbp_options* opt);
size_t gbp_plan_device_bytes(const gbp_plan* plan);

/* ---- nodal projection -----------------------------------------------------------------
 * sigma = scaling_factor / rho per cell, computed on the device
 * (incflo_apply_nodal_projection.cpp:101-121); constant density: rho == NULL and
 * sigma = scaling_factor / rho0 (:184-188). */
int gbp_nodal_set_sigma_from_density(gbp_plan* plan, const gbp_array4* rho, double scaling_factor,
                                     double rho0);
/* sigma given directly (cell array) or as a constant (sigma == NULL). */
int gbp_nodal_set_sigma(gbp_plan* plan, const gbp_array4* sigma, double const_sigma);

/* Hydro::NodalProjector::project(rtol, atol) plus getPhi/getGradPhi
 * (incflo_apply_nodal_projection.cpp:215-219): b = nodal div(vel), solve
 * div(sigma grad phi) = b, vel -= sigma grad phi in place. vel: 3 components, >= 1 ghost
 * cell; ghost cells are read only on GBP_BC_INFLOW faces (normal component). phi (nodal)
 * and gradphi (cell, 3 comps) may be NULL. phi_guess != 0: phi holds the initial guess. */
int gbp_nodal_project(gbp_plan* plan, gbp_array4* vel, gbp_array4* phi, gbp_array4* gradphi,
                      int phi_guess, gbp_stats* stats);

/* getLinOp().setOversetMask(lev, mask) (incflo_apply_nodal_projection.cpp:203-210, mask from
 * incflo::make_nodalBC_mask, src/boundary_conditions/incflo_set_bcs.cpp:10-53): nodal integer
 * mask over nodes 0..n, 0 = phi is held at 0 there (the Dirichlet part of a mixed boundary), nonzero
 * = solve. A coarse-level node is free where every fine node of its support (2I-1 .. 2I+1 per
 * direction) is. NULL (or data == NULL) removes the mask. */
int gbp_nodal_set_overset_mask(gbp_plan* plan, const gbp_iarray4* mask);

/* Cut cells of a nodal plan: the EB factory of the NodalProjector's MultiFabs
 * (incflo_apply_nodal_projection.cpp:95-267 on an EB level; MLNodeLaplacian builds its cut-cell
 * stencils from the EB volume moments). moments: cell array with 27 components, component p + 3q + 9r =
 * int xi^p eta^q zeta^r dV / V over the fluid part of the cell (p, q, r <= 2), in the cell's normalised
 * coordinates [-1/2, 1/2]^3; component 0 is the volume fraction. Each cut cell contributes its exact Q1
 * element matrix and int u . grad N over the fluid part; no flux through the embedded boundary; nodes
 * that touch no fluid are not unknowns; the correction uses grad phi at the fluid centroid of each cut
 * cell. NULL removes the cut cells. Sigma must be set again afterwards (gbp_apply_nodal_projection
 * does on every call). */
int gbp_nodal_set_eb(gbp_plan* plan, const gbp_array4* moments);

/* Velocity on the embedded boundary of a nodal plan's cut cells: MLNodeLaplacian::setEBInflowVelocity
 * (src/projection/incflo_apply_nodal_projection.cpp:196-201, eb_vel from incflo::set_eb_velocity,
 * src/boundary_conditions/incflo_set_bcs.cpp:195-280). Cell arrays with 3 components, valid cells:
 * eb_vel the velocity on the boundary; eb_dap the boundary's area vector int_EB n dA (n out of the
 * fluid) divided by the cell's face area of each direction, which equals the area-fraction difference
 * ap(low face) - ap(high face) (AMReX's barea x bnorm on cubic cells); eb_bcent the boundary centroid's
 * offset from the cell centre in cell widths (the EB factory's bcent). Each later projection adds the
 * weak form's boundary term -int_EB (u_eb . n) N_a dA = -F_c N_a(bcent) to the right-hand side of the
 * corners a of every cut cell c, F_c = sum_d eb_vel_d eb_dap_d V / h_d. The plan keeps the per-cell
 * terms, not the arrays. eb_vel == NULL removes the inflow; gbp_nodal_set_eb drops it.
 * GBP_BAD_ARG without cut cells on the plan. */
int gbp_nodal_set_eb_inflow(gbp_plan* plan, const gbp_array4* eb_vel, const gbp_array4* eb_dap,
                            const gbp_array4* eb_bcent);

/* The nodal divergence of vel as the projection sees it: the right-hand side of the nodal solve
 * (div_i = weak divergence / control volume, inflow normal velocity from the ghost cells when
 * use_inflow != 0, 0 on Dirichlet nodes), made consistent for singular boundary sets. div_out
 * (nodal, nodes 0..n, may be NULL) and its max norm (host double). This is the post-projection
 * check max|div u|; the reference computes the same quantity inside NodalProjector::project
 * (incflo_apply_nodal_projection.cpp:215) but exposes no call for it. */
int gbp_nodal_divergence(gbp_plan* plan, const gbp_array4* vel, int use_inflow, gbp_array4* div_out,
                         double* max_norm);

/* Allocation-free gbp_nodal_divergence. No counterpart in the reference. For callers that cannot
 * allocate device memory: a host program whose device memory belongs to another framework's
 * allocator (which may hold the whole pool or forbid cudaMalloc while it runs), or a plugin that may
 * not create a plan. Needs no plan; the only scratch is a static device array built into the library
 * (512 KB per GPU, held until the process exits), which caps the grid at 65536 blocks of 32x4x4
 * nodes (about 33.5 million nodes; larger grids return GBP_BAD_ARG). The first call on a device
 * (and the first after a reset of its context) looks up that array's address with the device
 * current, so make it before any stream capture. All calls share the array: calls that overlap on
 * the GPU race, so serialise them. Arguments as gbp_nodal_divergence, plus the level geometry,
 * boundary types and stream that a plan would otherwise hold; vel needs one ghost cell only across
 * the sides that are inflow faces. *max_norm is read back to the host before the call returns, so
 * the call synchronises the stream. */
int gbp_nodal_divergence_noalloc(const gbp_geometry* geom, const int bc_lo[3], const int bc_hi[3],
                                 const gbp_array4* vel, int use_inflow, gbp_array4* div_out,
                                 double* max_norm, void* stream);

/* incflo::ApplyNodalProjection(density, time, scaling_factor, incremental) end to end
 * (incflo_apply_nodal_projection.cpp:29-93 and :95-267 for one level): fuses the
 * add-back of scaling_factor*gp/rho (:39-62), the U^n subtraction for incremental or
 * small-dt projections (:65-71, :86-92), sigma = scaling_factor/rho, the solve, the
 * velocity correction and the gp / p_nd update (:221-256) into a few kernels.
 * vel_old may be NULL when neither incremental nor small-dt applies. rho == NULL means
 * constant density rho0. */
int gbp_apply_nodal_projection(gbp_plan* plan, gbp_array4* vel, const gbp_array4* vel_old,
                               const gbp_array4* rho, double rho0, gbp_array4* gp,
                               gbp_array4* p_nd, double time, double dt, double prev_dt,
                               double scaling_factor, int incremental, int set_inflow_bc,
                               gbp_stats* stats);

/* ---- MAC projection -------------------------------------------------------------------
 * beta on faces: MacProjector::initProjector(lp_info, beta) / updateCoeffs(beta)
 * (incflo_compute_MAC_projected_velocities.cpp:96-133). beta == NULL: constant beta
 * (initProjector(ba, dm, lp_info, dt/rho0) and updateBeta(dt/rho0)). */
int gbp_mac_set_beta(gbp_plan* plan, const gbp_array4* beta_x, const gbp_array4* beta_y,
                     const gbp_array4* beta_z, double const_beta);
/* beta = dt / (arithmetic face average of rho), the incflo construction
 * (average_cellcenter_to_face + invert(dt), :82-91); rho needs one ghost cell in every
 * non-periodic direction it is averaged across (read only at interior faces). */
int gbp_mac_set_beta_from_density(gbp_plan* plan, const gbp_array4* rho, double dt);

/* MacProjector::setUMAC + project(rtol, atol) or project(phi, rtol, atol)
 * (:272, :287-299): rhs = div(umac), solve div(beta grad phi) = rhs, umac -= beta grad phi
 * in place. phi (cell) may be NULL; phi_guess != 0 uses phi as the initial guess. */
int gbp_mac_project(gbp_plan* plan, gbp_array4* umac_x, gbp_array4* umac_y, gbp_array4* umac_z,
                    gbp_array4* phi, int phi_guess, gbp_stats* stats);

/* MacProjector::getFluxes(fluxes, phi, Location::FaceCenter / FaceCentroid)
 * (src/projection/incflo_apply_cc_projection.cpp:383-390): flux_d = -beta grad phi on the faces
 * 0..n of direction d ("MINUS (dt/rho) Gphi"), with the plan's boundary types (Dirichlet faces through
 * the zero boundary value, Neumann faces 0) and, with cut cells, the face-centroid gradient of cut
 * faces: exactly the correction gbp_mac_project subtracts from umac. phi: cells 0..n-1. Asynchronous
 * on the plan's stream. */
int gbp_mac_get_fluxes(gbp_plan* plan, const gbp_array4* phi, gbp_array4* flux_x, gbp_array4* flux_y,
                       gbp_array4* flux_z);

/* ---- cell-centred ABecLaplacian solve (scalar diffusion) ---------------------------------
 * The implicit scalar diffusion of DiffusionScalarOp::diffuse_scalar
 * (src/diffusion/DiffusionScalarOp.cpp:150-327): MLABecLaplacian alpha a phi - beta div(b grad phi) =
 * rhs (setScalars :193-195, setACoeffs :197-202, setBCoeffs with the face-averaged eta :251-252,
 * setLevelBC(lev, &phi) :295) solved by MLMG (:306-326), on a MAC plan (same levels, boundary types,
 * options: mg_rtol / mg_atol / maxiter / precision). Dirichlet sides take their boundary values from
 * the ghost cells of phi (the value on the face, linear extrapolation: maxorder 2 as incflo sets it);
 * Neumann sides are homogeneous; Robin sides and cut cells are rejected.
 * gbp_abec_set_coeffs: a (cells) or the constant a0 when a == NULL; b (face arrays of each direction)
 * or the constant b0 when bx == NULL; alpha = 0 restores the plan's Poisson operator.
 * gbp_abec_solve: rhs (cells); phi (cells, one ghost layer on Dirichlet sides) is the initial guess and
 * receives the solution. */
int gbp_abec_set_coeffs(gbp_plan* plan, double alpha, const gbp_array4* a, double a0, double beta,
                        const gbp_array4* bx, const gbp_array4* by, const gbp_array4* bz, double b0);
int gbp_abec_solve(gbp_plan* plan, const gbp_array4* rhs, gbp_array4* phi, gbp_stats* stats);
/* setBCoeffs(incflo::average_scalar_eta_to_faces(eta)) (src/diffusion/incflo_diffusion.cpp:289-343):
 * b = the face average of the cell field eta, the adjacent cell's eta on non-periodic domain sides. */
int gbp_abec_set_coeffs_eta(gbp_plan* plan, double alpha, const gbp_array4* a, double a0, double beta,
                            const gbp_array4* eta);

/* ---- tensor (velocity) diffusion ---------------------------------------------------------
 * DiffusionTensorOp (src/diffusion/DiffusionTensorOp.cpp:104-317) over MLTensorOp:
 *   alpha a u - beta div tau = rhs,  tau = eta (grad u + grad u^T) - (2/3) eta (div u) I
 * diffuse_velocity: alpha = 1, a = rho, beta = dt, rhs = rho u, eta on faces from
 * average_velocity_eta_to_faces (the face average of the cell field with the domain-side fix-up);
 * compute_divtau: div tau. One box, cell-centred. bc_lo / bc_hi: [3 * component + direction] (the
 * per-component table of incflo::get_diffuse_tensor_bc, incflo_diffusion.cpp:106-153):
 * GBP_BC_PERIODIC, GBP_BC_DIRICHLET (no-slip wall, mass inflow; GBP_BC_INFLOW is read as Dirichlet) or
 * GBP_BC_NEUMANN (outflow; tangential components at a slip wall). Velocity arrays carry 3 components
 * and one ghost layer on the non-periodic sides; the ghost cells next to Dirichlet faces hold the face
 * values (setLevelBC(lev, velocity)). */
typedef struct gbp_tensor gbp_tensor;
int gbp_tensor_create(const gbp_geometry* geom, const int bc_lo[9], const int bc_hi[9], const gbp_options* opt,
                      void* stream, gbp_tensor** out);
int gbp_tensor_destroy(gbp_tensor* t);
int gbp_tensor_set_options(gbp_tensor* t, const gbp_options* opt);
size_t gbp_tensor_device_bytes(const gbp_tensor* t);
/* setScalars(alpha, beta), setACoeffs(a) (a == NULL: the constant a0), setShearViscosity: eta as a cell
 * field averaged to the faces (eta_cc), as face arrays (eta_x/y/z, when eta_cc is NULL) or the
 * constant eta0 (all NULL). alpha > 0 for solves. */
int gbp_tensor_set_coeffs(gbp_tensor* t, double alpha, const gbp_array4* a, double a0, double beta,
                          const gbp_array4* eta_cc, const gbp_array4* eta_x, const gbp_array4* eta_y,
                          const gbp_array4* eta_z, double eta0);
/* MLMG::solve(velocity, rhs, rtol, atol): vel is the initial guess and receives the solution */
int gbp_tensor_solve(gbp_tensor* t, const gbp_array4* rhs, gbp_array4* vel, gbp_stats* stats);
/* MLMG::apply with setScalars(0, -1): divtau = div tau of vel */
int gbp_tensor_apply(gbp_tensor* t, const gbp_array4* vel, gbp_array4* divtau);

/* ---- two-level (AMR) composite nodal projection ----------------------------------------
 * incflo::ApplyNodalProjection(density, time, scaling_factor, incremental) over finest_level = 1
 * (src/projection/incflo_apply_nodal_projection.cpp:95-267): one NodalProjector over both levels
 * (:187-192) and MLNodeLaplacian's composite solve (:215), the levels' phi / grad phi (:218-219),
 * gp and p_nd per level (:221-257). Composite discretisation: conforming Q1 elements on the leaf cells
 * (fine cells of the fine boxes, coarse cells they do not cover); fine nodes on the coarse-fine
 * interface that are not coarse nodes hang (linear along the coarse face). Refinement ratio 2.
 * fine_boxes: nbox boxes of fine cells (lo[3], hi[3] inclusive, 6 ints each, in the fine index
 * space of the whole domain; disjoint, whole coarse cells: lo even, hi odd) — the fine level's
 * BoxArray. Boundaries: periodic, Dirichlet (outflow) and Neumann (walls); inflow is rejected. */
typedef struct gbp_amr gbp_amr;
int gbp_amr_create(const gbp_geometry* coarse, const int bc_lo[3], const int bc_hi[3], const int* fine_boxes,
                   int nbox, const gbp_options* opt, void* stream, gbp_amr** amr);
int gbp_amr_destroy(gbp_amr* amr);
int gbp_amr_set_options(gbp_amr* amr, const gbp_options* opt);
size_t gbp_amr_device_bytes(const gbp_amr* amr);
/* Coarse level: vel (3 comps), gp (3), rho (NULL: rho0), vel_old (incremental only, else NULL) cell
 * arrays, p_nd nodal (NULL: not written). Fine level: arrays of nbox pointers (the fine MultiFab's
 * FABs, in box order) with the same meaning; p_f covers each box's nodes. Non-incremental: u += s gp /
 * rho before the solve and gp = grad phi, p_nd = phi after; incremental: u -= vel_old before, gp +=,
 * p_nd += after, with vel_old added back. */
int gbp_amr_apply_nodal_projection(gbp_amr* amr, gbp_array4* vel_c, const gbp_array4* vel_old_c,
                                   const gbp_array4* rho_c, gbp_array4* gp_c, gbp_array4* p_c,
                                   gbp_array4* const* vel_f, const gbp_array4* const* vel_old_f,
                                   const gbp_array4* const* rho_f, gbp_array4* const* gp_f, gbp_array4* const* p_f,
                                   double rho0, double scaling_factor, int incremental, gbp_stats* stats);

/* ---- multi-box levels ---------------------------------------------------------------------
 * A level whose MultiFabs hold several FABs (incflo's amr.max_grid_size split; the MFIter loops of
 * src/projection/incflo_apply_nodal_projection.cpp:58-93, 124-192, 221-257 and
 * src/convection/incflo_compute_MAC_projected_velocities.cpp:82-90, 272-299). boxes: nbox boxes of
 * valid cells (lo[3], hi[3] inclusive, 6 ints each) that tile the plan's domain (disjoint, inside it,
 * covering it: the level's BoxArray); each field is an array of nbox gbp_array4, FAB b covering box b
 * (cell fields: its cells; nodal p_nd: nodes lo..hi+1; umac of direction d: faces lo..hi+1 in d), and
 * vel one ghost cell across inflow sides where the box touches them (rho of the MAC plan: across
 * Dirichlet sides). The plan gathers the FABs into its single-box staging (allocated on first use, kept
 * with the plan), runs the single-box entry point and scatters the outputs to every FAB (faces and
 * nodes shared by two boxes receive the same value). Same semantics, options and status codes as the
 * single-box calls. */
int gbp_apply_nodal_projection_boxes(gbp_plan* plan, int nbox, const int* boxes, gbp_array4* const* vel,
                                     const gbp_array4* const* vel_old, const gbp_array4* const* rho, double rho0,
                                     gbp_array4* const* gp, gbp_array4* const* p_nd, double time, double dt,
                                     double prev_dt, double scaling_factor, int incremental, int set_inflow_bc,
                                     gbp_stats* stats);
int gbp_mac_set_beta_from_density_boxes(gbp_plan* plan, int nbox, const int* boxes, const gbp_array4* const* rho,
                                        double dt);
int gbp_mac_project_boxes(gbp_plan* plan, int nbox, const int* boxes, gbp_array4* const* umac_x,
                          gbp_array4* const* umac_y, gbp_array4* const* umac_z, gbp_array4* const* phi,
                          int phi_guess, gbp_stats* stats);

/* ---- host-buffer convenience (end-to-end path) ----------------------------------------
 * Same as gbp_apply_nodal_projection with contiguous HOST arrays (no ghost cells):
 * vel [3][nz][ny][nx], rho [nz][ny][nx], gp [3][nz][ny][nx], p_nd nodal [nz+1][ny+1][nx+1].
 * The copies in and out run on the plan's stream inside the call. */
int gbp_apply_nodal_projection_host(gbp_plan* plan, double* vel, const double* rho, double rho0,
                                    double* gp, double* p_nd, double scaling_factor,
                                    int incremental, gbp_stats* stats);

/* ---- diagnostics ---------------------------------------------------------------------
 * No counterpart in the reference (its MLMG has only TINY_PROFILE timers). Times `reps`
 * back-to-back launches of one level-0 kernel of a nodal plan on the plan's stream with CUDA
 * events, on the arrays of the last solve, and reports the kernel's algorithmic bytes per launch.
 * which: 0 = FP64 Jacobi sweep, 1 = FP32 Jacobi sweep, 2 = FP64 residual, 3 = FP32 residual,
 * 4 = streaming triad over three level arrays (an HBM reference), 5 = FP32 Jacobi through the
 * plain kernel, 6 = FP32 prolongation level 1 -> 0, 7 = FP32 restriction level 0 -> 1,
 * 8 = fused FP32 residual + restriction 0 -> 1, 9 = fused FP32 prolongation 1 -> 0 + Jacobi. */
int gbp_plan_time_kernel(gbp_plan* plan, int which, int reps, double* ms_per_launch,
                         double* bytes_per_launch);

/* No counterpart in the reference: a test hook. On seeded level-0 / level-1 data of a nodal plan (its
 * sigma), runs the FP32 whole-row level kernels and the one-node-per-thread kernels they replace and
 * writes max |new - reference| / max |reference| over every padded position (periodic aliases
 * included) for diff[0] Jacobi, diff[1] residual, diff[2] residual + restriction, diff[3]
 * prolongation + Jacobi (-1 for [2] and [3] on a level with an overset mask, where the fused transfers do
 * not run). GBP_BAD_ARG when the whole-row kernels do not apply to the plan's level 0. */
int gbp_plan_check_level_kernels(gbp_plan* plan, double diff[4]);

/* No counterpart in the reference: a test hook. One FP32 V-cycle from the first level that a plan cycles
 * in one thread-block-cluster launch (the FP32 levels of at most 5000 nodes (nodal) / 40000 cells (MAC)
 * below the finest, with the dense bottom), on a seeded right-hand side, once through the per-level launches and
 * once through the cluster kernel; *diff = max |cluster - per-level| / max |per-level| over every padded
 * position. GBP_BAD_ARG when the plan has no such levels. */
int gbp_plan_check_coarse_cycle(gbp_plan* plan, double* diff);

/* MacProjector::setLevelBC(lev, nullptr, robin_a, robin_b, robin_f) for the GBP_BC_ROBIN sides
 * (incflo_compute_MAC_projected_velocities.cpp:116-123; data from incflo::make_robinBC_MFs,
 * src/boundary_conditions/incflo_set_bcs.cpp:121-192): cell arrays with one ghost layer whose
 * ghost cells next to a Robin face hold a, b, f of a phi + b dphi/dn = f on that face. The face
 * enters the operator with weight beta a h / (a h / 2 + b) (phi at the face = mean of the ghost and
 * interior values): b = 0 gives the Dirichlet face, a = 0 the Neumann one. f must be 0 (incflo's
 * MAC Robin data, prob_set_MAC_robinBCs, always has f = 0); robin_f may be NULL. */
int gbp_mac_set_robin(gbp_plan* plan, const gbp_array4* robin_a, const gbp_array4* robin_b,
                      const gbp_array4* robin_f);

/* Embedded-boundary cut cells of a MAC plan: what the reference's MacProjector takes from the
 * EBFArrayBoxFactory of its beta MultiFabs (incflo's EB factory, src/incflo.H:743-752; the projector
 * is built with MLMG::Location::FaceCentroid for umac and beta, src/incflo.cpp:286-292, and
 * MLEBABecLap, src/convection/incflo_compute_MAC_projected_velocities.cpp:82-90). vfrac: volume
 * fractions (cells); area_x/y/z: area fractions (faces 0..n of each direction); fcent_x/y/z: face
 * centroids, 2 components = offsets of the open part's centroid from the face centre in cell widths
 * ([-0.5, 0.5]) along the two tangential directions in increasing order (AMReX's fcx / fcy / fcz).
 * The operator becomes the cut-cell one: flux = area fraction x beta x the normal derivative at the
 * face centroid (bilinear blend of neighbouring face-centre differences), no flux through the EB,
 * RHS = area-weighted divergence of the face-centroid velocities, stopping norm max |r| / vfrac,
 * singular systems made consistent and gauged with vfrac weights, covered cells phi = 0. Beta must
 * be set again after this call. vfrac == NULL removes the EB. */
int gbp_mac_set_eb(gbp_plan* plan, const gbp_array4* vfrac, const gbp_array4* area_x, const gbp_array4* area_y,
                   const gbp_array4* area_z, const gbp_array4* fcent_x, const gbp_array4* fcent_y,
                   const gbp_array4* fcent_z);

/* MacProjector::setEBInflowVelocity(lev, eb_vel)
 * (src/convection/incflo_compute_MAC_projected_velocities.cpp:274-281): eb_vel (cells, 3 components,
 * valid cells) is the velocity on each cut cell's embedded boundary. Its flux out of the fluid,
 * sum_d eb_vel_d (ap_d(low face) - ap_d(high face)) V / h_d (the boundary's area vector from the area
 * fractions set by gbp_mac_set_eb), is part of the divergence of the following projections. The plan
 * keeps the per-cell flux, not the array. eb_vel == NULL removes it; gbp_mac_set_eb drops it.
 * GBP_BAD_ARG without cut cells on the plan. */
int gbp_mac_set_eb_inflow(gbp_plan* plan, const gbp_array4* eb_vel);

/* incflo::ApplyCCProjection(density, umac, time, scaling_factor, incremental) for one level,
 * non-EB (src/projection/incflo_apply_cc_projection.cpp:199-487; option incflo.use_cc_proj):
 * gp add-back (:214-238), U^n subtraction for incremental / small-dt projections (:241-249),
 * method-of-lines face velocities (MOL::ExtrapVelToFaces, :350-353: monotonised-central slopes,
 * upwinded by the face-state average; wall faces 0, inflow faces the ghost value, outflow faces
 * the adjacent cell), the MAC solve with beta = scaling_factor / rho_face (arithmetic mean of the
 * two cells; rho == NULL: scaling_factor / rho0) (:276-366), fluxes -beta grad phi averaged to
 * cells (:383-399), u += gphi, p_cc = phi (+= when incremental), gp = -gphi rho / s (-=)
 * (:401-463), U^n added back (:471-477). plan: a MAC plan. umac_x/y/z receive the projected face
 * velocities (they are the reference's u_mac/v_mac/w_mac arguments). */
int gbp_apply_cc_projection(gbp_plan* plan, gbp_array4* vel, const gbp_array4* vel_old,
                            const gbp_array4* rho, double rho0, gbp_array4* gp, gbp_array4* p_cc,
                            gbp_array4* umac_x, gbp_array4* umac_y, gbp_array4* umac_z, double time,
                            double dt, double prev_dt, double scaling_factor, int incremental,
                            int set_inflow_bc, gbp_stats* stats);

/* amrex::average_down(fine, crse, 0, ncomp, ratio) as incflo applies it to gp after the nodal
 * projection on an AMR hierarchy (incflo_apply_nodal_projection.cpp:258-266): every coarse cell
 * of [crse_lo, crse_hi] (the coarsened fine region, coarse-level indices) becomes the mean of its
 * ratio[0] x ratio[1] x ratio[2] fine cells, for components 0..ncomp-1. stream: cudaStream_t. */
int gbp_average_down(const gbp_array4* fine, gbp_array4* crse, const int ratio[3], int ncomp,
                     const int crse_lo[3], const int crse_hi[3], void* stream);

/* ---- inflow / outflow solvability -----------------------------------------------------
 * HydroUtils::enforceInOutSolvability as incflo calls it before the nodal projection
 * (incflo_apply_nodal_projection.cpp:166-179; has_inout_bndry && set_inflow_bc): vel is the
 * cell-centred velocity (3 comps, one ghost layer whose boundary ghost cells hold the boundary
 * values); dd_lo / dd_hi mark the direction_dependent faces. The flux into the domain through
 * those faces (face area x normal velocity) is split into inflow and outflow and every outflow
 * normal velocity is multiplied by inflow / outflow, so the net flux is zero (no change when
 * there is no outflow). inflow_outflow (host, 2 doubles, may be NULL) receives the two fluxes
 * before scaling. */
int gbp_enforce_inout_solvability(gbp_plan* plan, gbp_array4* vel, const int dd_lo[3],
                                  const int dd_hi[3], double* inflow_outflow);
/* The same on the MAC face velocities' boundary faces 0 and n
 * (incflo_compute_MAC_projected_velocities.cpp:266-270). */
int gbp_mac_enforce_inout_solvability(gbp_plan* plan, gbp_array4* ux, gbp_array4* uy,
                                      gbp_array4* uz, const int dd_lo[3], const int dd_hi[3],
                                      double* inflow_outflow);

/* ---- warm-start network building blocks (no reference counterpart) -------------------
 * Activations are channels-last BF16 matrices [R][C] over a grid of dims[0] x dims[1] x
 * dims[2] voxels with a one-voxel zero halo, R = (dims[0]+2)(dims[1]+2)(dims[2]+2), row
 * p = (z+1)(dims[1]+2)(dims[0]+2) + (y+1)(dims[0]+2) + (x+1). Channel counts are 16, 32 or
 * multiples of 64; all pointers are device pointers, 16-byte aligned. Both calls
 * synchronise the stream and return GBP_TIMEOUT if a bounded wait inside the kernel ran out. */

/* out = epilogue(sum over inputs i, taps t, channels c of in_i[p + off(t)][c] w[t][n][c0_i + c])
 * with w [ntaps][cout][sum cin] BF16 (ntaps 27: 3x3x3 cross-correlation, tap t = 9(dz+1) +
 * 3(dy+1) + (dx+1); ntaps 1: pointwise), off negated when flip != 0. Output channel n goes to
 * segment s (seg_c[s] channels each, [R][seg_c[s]]). flags: 1 = forward GELU (out = gelu(acc +
 * bias), aux = acc + bias when aux[s] != NULL), 2 = add the existing out, 4 = multiply by
 * gelu'(aux). Halo rows of out are written as zeros. */
int gbp_nn_conv3d(const int dims[3], int nin, void* const in[], const int cin[], const void* w,
                  int ntaps, int flip, int cout, const float* bias, int nseg, void* const out[],
                  void* const aux[], const int seg_c[], int flags, void* stream);

/* dw[t][o][ci0 + c] += sum_p gout[p][o] in[p + off(t)][c], FP32 dw [ntaps][cout][cin_tot]. */
int gbp_nn_conv3d_wgrad(const int dims[3], const void* in, int cin, int ci0, int cin_tot,
                        const void* gout, int cout, int ntaps, float* dw, void* stream);

/* ---- learned warm start (surrogate U-Net) ----------------------------------------------
 * A four-level 3-D U-Net (16/32/64/128 channels, 3x3x3 convolutions + GELU, ~1.5 M
 * parameters) that predicts the shape of phi from the nodal right-hand side, the node-averaged
 * sigma and (optionally) the previous phi. Trained on the GPU with Adam on pairs produced by this
 * library's own solver; attached to a nodal plan it supplies the initial guess of zero-guess
 * solves, scaled by the Galerkin factor x.b / x.Ax, and is bypassed when the scaled guess has a
 * larger residual than the zero start (stats.warm_start = 2). No reference counterpart. */
typedef struct gbp_surrogate gbp_surrogate;
int gbp_surrogate_create(int base_channels, unsigned long long seed, gbp_surrogate** out);
int gbp_surrogate_destroy(gbp_surrogate* s);
long long gbp_surrogate_num_params(const gbp_surrogate* s);
int gbp_surrogate_get_params(const gbp_surrogate* s, float* host, long long n);
int gbp_surrogate_set_params(gbp_surrogate* s, const float* host, long long n);
int gbp_surrogate_get_grads(const gbp_surrogate* s, float* host, long long n);
int gbp_surrogate_save(const gbp_surrogate* s, const char* path);
int gbp_surrogate_load(gbp_surrogate* s, const char* path);
/* one forward + backward (+ Adam step when lr > 0) on a device input [R][16] BF16 and target
 * [R] FP32 over a network grid dims (multiples of 8); loss over voxels below dom */
int gbp_surrogate_train_pair(gbp_surrogate* s, const int dims[3], const int dom[3], const void* x0,
                             const float* target, float lr, double* loss, void* stream);
/* forward pass; hout (device, [R][16] BF16, channel 0 = prediction) may be NULL */
int gbp_surrogate_predict(gbp_surrogate* s, const int dims[3], const void* x0, void* hout,
                          void* stream);
/* append a training pair from a nodal plan after gbp_nodal_project: input channels from the plan's
 * right-hand side minus A phi_prev (the residual of the previous solution in this projection's system;
 * the right-hand side itself when phi_prev is NULL), sigma and phi_prev (nodal); target = the plan's
 * phi - phi_prev (the increment the network predicts on top of the previous solution; phi without one) */
int gbp_surrogate_add_sample(gbp_surrogate* s, gbp_plan* plan, const gbp_array4* phi_prev);
/* one training step on the pair of a nodal plan's last projection (built as gbp_surrogate_add_sample
 * builds it, used once, not stored): forward + backward, and an Adam step when lr > 0; *loss (host,
 * may be NULL) = the normalised MSE. Training on a stream of such pairs needs no sample storage. */
int gbp_surrogate_train_step(gbp_surrogate* s, gbp_plan* plan, const gbp_array4* phi_prev, float lr,
                             double* loss);
int gbp_surrogate_num_samples(const gbp_surrogate* s);
int gbp_surrogate_clear_samples(gbp_surrogate* s);
/* steps (<= 60 per call) Adam steps on randomly drawn samples; losses[steps] (host) may be NULL */
int gbp_surrogate_train(gbp_surrogate* s, int steps, float lr, unsigned long long seed,
                        float* losses, void* stream);
/* attach (s != NULL) or detach a surrogate: the network runs on multigrid level `level` of the
 * plan (0 = finest); mode 1 = use with the bypass rule, 0 = off. With initial_guess = zero it predicts
 * phi and competes with the zero start; with initial_guess = previous it predicts the increment on top
 * of the plan's last solution and competes with that start. */
int gbp_plan_set_surrogate(gbp_plan* plan, gbp_surrogate* s, int level, int mode);

#ifdef __cplusplus
}
#endif
#endif
