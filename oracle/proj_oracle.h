/*
 * CPU oracle for the incflo projection hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may load
 * this library, and only as the checker or the timed CPU baseline. Nothing in the shipped
 * solver calls it.
 *
 * Parity status: "parity unpinned". The reference's solver arithmetic lives in AMReX
 * (MLNodeLaplacian, MLPoisson, MLABecLaplacian, MLMG) and AMReX-Hydro (NodalProjector,
 * MacProjector). Neither is vendored with incflo (src/Make.incflo:31-59, CMakeLists.txt:122-179)
 * and the reference ships no golden outputs for the projection (its regression plotfiles are
 * generated, not committed: test_3d/README.md). What pins this restatement instead:
 *   - the analytic pressure of incflo's Taylor-Green case (src/derive/incflo_error.cpp:33-34)
 *     recovered by projecting u_TG + grad(p_exact) at second order (tests/test_oracle.py);
 *   - an independent element-by-element assembly of the same finite-element matrix in numpy;
 *   - discrete identities: symmetry, the constant null space, D = -G^T, div after projection.
 *
 * Discretisation (restated from the mathematics of the approximate projection used by
 * incflo::ApplyNodalProjection, src/projection/incflo_apply_nodal_projection.cpp:95-267):
 *   nodal: phi on nodes, sigma = s/rho per cell; A = integral(sigma grad N_i . grad N_j) over
 *   trilinear (Q1) elements; right-hand side g_i = integral(u . grad N_i) - boundary flux of
 *   the inflow velocity (weak form of -div u); gradient = cell average of the four edge
 *   differences per direction; correction u -= sigma * grad phi.
 *   mac: phi on cells, beta on faces; 7-point flux form (Hydro::MacProjector semantics used at
 *   src/convection/incflo_compute_MAC_projected_velocities.cpp:272-299).
 * Boundary codes follow incflo's maps (src/projection/incflo_projection_bc.cpp:5-79).
 */
#ifndef PROJ_ORACLE_H
#define PROJ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_PERIODIC = 0, OR_DIRICHLET = 1, OR_NEUMANN = 2, OR_INFLOW = 3 };

typedef struct {
    int n[3];        /* cells per direction */
    double h[3];     /* cell size */
    int bclo[3];     /* OR_* per direction, low side */
    int bchi[3];     /* OR_* per direction, high side */
    const unsigned char* mask; /* nodal: unique-node overset mask, 0 = phi fixed at 0 (NULL: none) */
} or_grid;

/* ---- nodal ---------------------------------------------------------------------------
 * node arrays: unique nodes, nn[d] = n[d] (periodic) or n[d]+1, x fastest.
 * cell arrays: n[0]*n[1]*n[2], x fastest.
 * velocity with one ghost layer: [3][n2+2][n1+2][n0+2]. Ghost cells are read only on
 * OR_INFLOW faces, and only for the face-normal component (the inflow value). */
void   or_nodal_dims(const or_grid* g, int nn[3]);
void   or_nodal_volume(const or_grid* g, double* vol);
void   or_nodal_stencil(const or_grid* g, const double* sigma, double* st27);
void   or_nodal_apply(const or_grid* g, const double* sigma, const double* phi, double* out);
void   or_nodal_rhs(const or_grid* g, const double* vel_g, double* rhs);
void   or_nodal_gradient(const or_grid* g, const double* phi, double* grad);
double or_nodal_resid_norm(const or_grid* g, const double* sigma, const double* rhs,
                           const double* phi, double* rhs_norm);
int    or_nodal_solve(const or_grid* g, const double* sigma, const double* rhs, double* phi,
                      double rtol, double atol, int maxiter, double* stats);
int    or_nodal_project(const or_grid* g, const double* sigma, double* vel_g, double* phi,
                        double* gradphi, double rtol, double atol, int maxiter, double* stats);

/* ---- MAC (cell-centred phi, face beta/velocity) ------------------------------------------
 * x-face arrays [n2][n1][n0+1], y-face [n2][n1+1][n0], z-face [n2+1][n1][n0].
 * In a periodic direction face n is the same face as face 0: reads use face 0, the
 * correction writes both. */
void   or_mac_rhs(const or_grid* g, const double* ux, const double* uy, const double* uz,
                  double* rhs);
void   or_mac_apply(const or_grid* g, const double* bx, const double* by, const double* bz,
                    const double* phi, double* out);
void   or_mac_correct(const or_grid* g, const double* bx, const double* by, const double* bz,
                      const double* phi, double* ux, double* uy, double* uz);
int    or_mac_solve(const or_grid* g, const double* bx, const double* by, const double* bz,
                    const double* rhs, double* phi, double rtol, double atol, int maxiter,
                    double* stats);
int    or_mac_project(const or_grid* g, const double* bx, const double* by, const double* bz,
                      double* ux, double* uy, double* uz, double* phi, int phi_is_guess,
                      double rtol, double atol, int maxiter, double* stats);

int    or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
