/*
 * CPU oracle for the incflo projection hot path -- TEST INFRASTRUCTURE ONLY.
 * See proj_oracle.h for the parity status ("parity unpinned") and the discretisation.
 *
 * Implementation strategy (deliberately unlike the GPU solver): every operator is assembled
 * into an explicit per-unknown stencil (27 coefficients per node, 7 per cell) by summing
 * element contributions, neighbours are found by periodic index wrapping rather than ghost
 * layers, and the solver is a conjugate-gradient iteration preconditioned by a symmetric
 * multigrid V-cycle with 8-colour Gauss-Seidel smoothing and a dense direct bottom solve.
 * It converges to the discrete solution regardless of how good the preconditioner is, so
 * the GPU solver is compared with the discrete operator, not with this solver's path.
 */
#include "proj_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXLEV 20

int or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int is_per(const or_grid* g, int d) { return g->bclo[d] == OR_PERIODIC; }

/* ------------------------------------------------------------------------------------------
 * generic stencil level
 * ---------------------------------------------------------------------------------------- */
typedef struct {
    int dims[3];
    int per[3];
    int nst;
    int off[27][3];
    long loff[27]; /* linear offset of each stencil entry (nodes away from every side need no wrap) */
    long n;
    double* st;
    double* vol;
    unsigned char* fixed;
    unsigned char* color;
    /* dense bottom (LU with partial pivoting) */
    double* lu;
    int* piv;
    int singular;
    int first_free;
    int dirichlet; /* some boundary holds phi = 0: the system is nonsingular */
} lvl;

static inline int wrap(int i, int n, int per)
{
    if (per) {
        i %= n;
        if (i < 0) i += n;
        return i;
    }
    return (i < 0 || i >= n) ? -1 : i;
}

static inline long lid(const lvl* L, int i, int j, int k)
{
    return (long)i + (long)L->dims[0] * ((long)j + (long)L->dims[1] * k);
}

static inline long nb(const lvl* L, int i, int j, int k, int m)
{
    int a = wrap(i + L->off[m][0], L->dims[0], L->per[0]);
    int b = wrap(j + L->off[m][1], L->dims[1], L->per[1]);
    int c = wrap(k + L->off[m][2], L->dims[2], L->per[2]);
    if (a < 0 || b < 0 || c < 0) return -1;
    return lid(L, a, b, c);
}

static void lvl_alloc(lvl* L, const int dims[3], const int per[3], int nst)
{
    memset(L, 0, sizeof(*L));
    for (int d = 0; d < 3; ++d) {
        L->dims[d] = dims[d];
        L->per[d] = per[d];
    }
    L->nst = nst;
    L->n = (long)dims[0] * dims[1] * dims[2];
    L->st = (double*)calloc((size_t)L->n * nst, sizeof(double));
    L->vol = (double*)calloc((size_t)L->n, sizeof(double));
    L->fixed = (unsigned char*)calloc((size_t)L->n, 1);
    L->color = (unsigned char*)calloc((size_t)L->n, 1);
    if (nst == 27) {
        int m = 0;
        for (int c = -1; c <= 1; ++c)
            for (int b = -1; b <= 1; ++b)
                for (int a = -1; a <= 1; ++a) {
                    L->off[m][0] = a;
                    L->off[m][1] = b;
                    L->off[m][2] = c;
                    ++m;
                }
    } else {
        static const int o7[7][3] = {{0, 0, 0}, {-1, 0, 0}, {1, 0, 0}, {0, -1, 0},
                                     {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
        memcpy(L->off, o7, sizeof(o7));
    }
    for (int m = 0; m < nst; ++m)
        L->loff[m] = (long)L->off[m][0] + (long)dims[0] * ((long)L->off[m][1] + (long)dims[1] * L->off[m][2]);
    for (int k = 0; k < dims[2]; ++k)
        for (int j = 0; j < dims[1]; ++j)
            for (int i = 0; i < dims[0]; ++i)
                L->color[lid(L, i, j, k)] = (unsigned char)((i & 1) | ((j & 1) << 1) | ((k & 1) << 2));
}

static void lvl_free(lvl* L)
{
    free(L->st);
    free(L->vol);
    free(L->fixed);
    free(L->color);
    free(L->lu);
    free(L->piv);
    memset(L, 0, sizeof(*L));
}

static int center_index(const lvl* L) { return L->nst == 27 ? 13 : 0; }

/* sum over the stencil row of node u = (i, j, k): nodes away from every side take the linear offsets,
 * the others wrap (periodic) or drop (outside) each neighbour; zero coefficients are skipped either way */
static inline double row_dot(const lvl* L, int i, int j, int k, long u, const double* x)
{
    const double* s = L->st + u * L->nst;
    double acc = 0.0;
    if (i >= 1 && i < L->dims[0] - 1 && j >= 1 && j < L->dims[1] - 1 && k >= 1 && k < L->dims[2] - 1) {
        for (int m = 0; m < L->nst; ++m)
            if (s[m] != 0.0) acc += s[m] * x[u + L->loff[m]];
    } else {
        for (int m = 0; m < L->nst; ++m) {
            if (s[m] == 0.0) continue;
            long v = nb(L, i, j, k, m);
            if (v >= 0) acc += s[m] * x[v];
        }
    }
    return acc;
}

static void lvl_apply(const lvl* L, const double* x, double* y)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < L->dims[2]; ++k)
        for (int j = 0; j < L->dims[1]; ++j)
            for (int i = 0; i < L->dims[0]; ++i) {
                long u = lid(L, i, j, k);
                y[u] = L->fixed[u] ? 0.0 : row_dot(L, i, j, k, u, x);
            }
}

static void lvl_resid(const lvl* L, const double* b, const double* x, double* r)
{
    lvl_apply(L, x, r);
#pragma omp parallel for schedule(static)
    for (long u = 0; u < L->n; ++u) r[u] = L->fixed[u] ? 0.0 : b[u] - r[u];
}

/* one colour-ordered Gauss-Seidel pass; dir=+1 colours 0..7, dir=-1 colours 7..0. Colour
 * (i&1) | (j&1)<<1 | (k&1)<<2: the nodes of one colour are visited with stride 2 in each direction */
static void lvl_gs(const lvl* L, const double* b, double* x, int dir)
{
    int c0 = dir > 0 ? 0 : 7;
    for (int cc = 0; cc < 8; ++cc) {
        int col = c0 + dir * cc;
        const int i0 = col & 1, j0 = (col >> 1) & 1, k0 = (col >> 2) & 1;
#pragma omp parallel for schedule(static)
        for (int k = k0; k < L->dims[2]; k += 2)
            for (int j = j0; j < L->dims[1]; j += 2)
                for (int i = i0; i < L->dims[0]; i += 2) {
                    long u = lid(L, i, j, k);
                    if (L->fixed[u]) continue;
                    double acc = row_dot(L, i, j, k, u, x);
                    double dg = L->st[u * L->nst + center_index(L)];
                    if (dg != 0.0) x[u] += (b[u] - acc) / dg;
                }
    }
}

static int any_fixed(const lvl* L) { return L->dirichlet; }

/* dense LU of the level operator; a singular (all periodic / Neumann) system gets the row
 * of its first free unknown replaced by the volume-weighted mean constraint */
static void lvl_dense_factor(lvl* L)
{
    long N = L->n;
    L->lu = (double*)calloc((size_t)(N * N), sizeof(double));
    L->piv = (int*)calloc((size_t)N, sizeof(int));
    double* M = L->lu;
    for (int k = 0; k < L->dims[2]; ++k)
        for (int j = 0; j < L->dims[1]; ++j)
            for (int i = 0; i < L->dims[0]; ++i) {
                long u = lid(L, i, j, k);
                if (L->fixed[u]) {
                    M[u * N + u] = 1.0;
                    continue;
                }
                const double* s = L->st + u * L->nst;
                for (int m = 0; m < L->nst; ++m) {
                    long v = nb(L, i, j, k, m);
                    if (v >= 0 && !L->fixed[v]) M[u * N + v] += s[m];
                }
            }
    L->singular = !any_fixed(L);
    L->first_free = 0;
    if (L->singular) {
        for (long v = 0; v < N; ++v) M[v] = L->vol[v];
    }
    for (long c = 0; c < N; ++c) {
        long p = c;
        double best = fabs(M[c * N + c]);
        for (long r = c + 1; r < N; ++r)
            if (fabs(M[r * N + c]) > best) {
                best = fabs(M[r * N + c]);
                p = r;
            }
        L->piv[c] = (int)p;
        if (p != c)
            for (long q = 0; q < N; ++q) {
                double t = M[c * N + q];
                M[c * N + q] = M[p * N + q];
                M[p * N + q] = t;
            }
        double d = M[c * N + c];
        if (d == 0.0) continue;
        for (long r = c + 1; r < N; ++r) {
            double f = M[r * N + c] / d;
            M[r * N + c] = f;
            if (f != 0.0)
                for (long q = c + 1; q < N; ++q) M[r * N + q] -= f * M[c * N + q];
        }
    }
}

static void lvl_dense_solve(const lvl* L, const double* b, double* x)
{
    long N = L->n;
    const double* M = L->lu;
    for (long u = 0; u < N; ++u) x[u] = L->fixed[u] ? 0.0 : b[u];
    if (L->singular) x[0] = 0.0;
    /* P A = L U: apply every row interchange first, then the two triangular solves */
    for (long c = 0; c < N; ++c) {
        long p = L->piv[c];
        if (p != c) {
            double t = x[c];
            x[c] = x[p];
            x[p] = t;
        }
    }
    for (long c = 0; c < N; ++c)
        for (long r = c + 1; r < N; ++r) x[r] -= M[r * N + c] * x[c];
    for (long c = N - 1; c >= 0; --c) {
        double acc = x[c];
        for (long q = c + 1; q < N; ++q) acc -= M[c * N + q] * x[q];
        x[c] = M[c * N + c] != 0.0 ? acc / M[c * N + c] : 0.0;
    }
}

/* ------------------------------------------------------------------------------------------
 * nodal discretisation
 * ---------------------------------------------------------------------------------------- */
void or_nodal_dims(const or_grid* g, int nn[3])
{
    for (int d = 0; d < 3; ++d) nn[d] = is_per(g, d) ? g->n[d] : g->n[d] + 1;
}

/* element stiffness of a trilinear brick, indexed by which directions the two corners differ
 * in (bit d set = differ in direction d): integral of grad N_a . grad N_b over the cell */
static void q1_element(const double h[3], double K[8])
{
    double V = h[0] * h[1] * h[2];
    for (int mask = 0; mask < 8; ++mask) {
        double acc = 0.0;
        for (int d = 0; d < 3; ++d) {
            double t = ((mask >> d) & 1) ? -1.0 : 1.0;
            t /= h[d] * h[d];
            for (int e = 0; e < 3; ++e) {
                if (e == d) continue;
                t *= ((mask >> e) & 1) ? (1.0 / 6.0) : (1.0 / 3.0);
            }
            acc += t;
        }
        K[mask] = V * acc;
    }
}

static int node_fixed(const or_grid* g, int i, int j, int k)
{
    int idx[3] = {i, j, k};
    if (g->mask) {
        /* incflo's mixed boundaries: the solver's overset mask marks nodes whose phi is known (0),
           src/boundary_conditions/incflo_set_bcs.cpp:10-53 */
        int nn[3];
        or_nodal_dims(g, nn);
        if (!g->mask[i + (long)nn[0] * (j + (long)nn[1] * k)]) return 1;
    }
    for (int d = 0; d < 3; ++d) {
        if (is_per(g, d)) continue;
        if (idx[d] == 0 && g->bclo[d] == OR_DIRICHLET) return 1;
        if (idx[d] == g->n[d] && g->bchi[d] == OR_DIRICHLET) return 1;
    }
    return 0;
}

static void nodal_level(const or_grid* g, const double* sigma, lvl* L)
{
    int nn[3], per[3];
    or_nodal_dims(g, nn);
    for (int d = 0; d < 3; ++d) per[d] = is_per(g, d);
    lvl_alloc(L, nn, per, 27);
    double K[8];
    q1_element(g->h, K);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nn[2]; ++k)
        for (int j = 0; j < nn[1]; ++j)
            for (int i = 0; i < nn[0]; ++i) {
                long u = lid(L, i, j, k);
                int idx[3] = {i, j, k};
                double v = 1.0;
                for (int d = 0; d < 3; ++d) {
                    int bnd = !per[d] && (idx[d] == 0 || idx[d] == g->n[d]);
                    v *= bnd ? 0.5 * g->h[d] : g->h[d];
                }
                L->vol[u] = v;
                L->fixed[u] = (unsigned char)node_fixed(g, i, j, k);
                if (L->fixed[u]) {
                    L->dirichlet = 1;
                    continue;
                }
                double* s = L->st + u * 27;
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b)
                        for (int a = 0; a < 2; ++a) {
                            int ci = wrap(i - 1 + a, g->n[0], per[0]);
                            int cj = wrap(j - 1 + b, g->n[1], per[1]);
                            int ck = wrap(k - 1 + c, g->n[2], per[2]);
                            if (ci < 0 || cj < 0 || ck < 0) continue;
                            double sg = sigma[ci + (long)g->n[0] * (cj + (long)g->n[1] * ck)];
                            /* node (i,j,k) is corner (1-a,1-b,1-c) of this cell */
                            for (int r = 0; r < 2; ++r)
                                for (int q = 0; q < 2; ++q)
                                    for (int p = 0; p < 2; ++p) {
                                        int mask = (p != 1 - a) | ((q != 1 - b) << 1) | ((r != 1 - c) << 2);
                                        int di = a + p - 1, dj = b + q - 1, dk = c + r - 1;
                                        s[(di + 1) + 3 * (dj + 1) + 9 * (dk + 1)] += sg * K[mask];
                                    }
                        }
            }
}

void or_nodal_volume(const or_grid* g, double* vol)
{
    int nn[3];
    or_nodal_dims(g, nn);
    for (int k = 0; k < nn[2]; ++k)
        for (int j = 0; j < nn[1]; ++j)
            for (int i = 0; i < nn[0]; ++i) {
                int idx[3] = {i, j, k};
                double v = 1.0;
                for (int d = 0; d < 3; ++d) {
                    int bnd = !is_per(g, d) && (idx[d] == 0 || idx[d] == g->n[d]);
                    v *= bnd ? 0.5 * g->h[d] : g->h[d];
                }
                vol[i + (long)nn[0] * (j + (long)nn[1] * k)] = v;
            }
}

void or_nodal_stencil(const or_grid* g, const double* sigma, double* st27)
{
    lvl L;
    nodal_level(g, sigma, &L);
    memcpy(st27, L.st, sizeof(double) * 27 * (size_t)L.n);
    lvl_free(&L);
}

void or_nodal_apply(const or_grid* g, const double* sigma, const double* phi, double* out)
{
    lvl L;
    nodal_level(g, sigma, &L);
    lvl_apply(&L, phi, out);
    lvl_free(&L);
}

/* g_i = integral(u . grad N_i) - integral over inflow faces of (u_bc . n) N_i; the minus of
 * the weak divergence, so that A phi = g and u - sigma grad phi is (weakly) divergence free */
void or_nodal_rhs(const or_grid* g, const double* vel_g, double* rhs)
{
    int nn[3];
    or_nodal_dims(g, nn);
    const int G0 = g->n[0] + 2, G1 = g->n[1] + 2, G2 = g->n[2] + 2;
    const long GC = (long)G0 * G1 * G2;
    const double cf[3] = {0.25 * g->h[1] * g->h[2], 0.25 * g->h[0] * g->h[2], 0.25 * g->h[0] * g->h[1]};
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nn[2]; ++k)
        for (int j = 0; j < nn[1]; ++j)
            for (int i = 0; i < nn[0]; ++i) {
                long u = i + (long)nn[0] * (j + (long)nn[1] * k);
                if (node_fixed(g, i, j, k)) {
                    rhs[u] = 0.0;
                    continue;
                }
                int idx[3] = {i, j, k};
                double acc = 0.0;
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b)
                        for (int a = 0; a < 2; ++a) {
                            int sel[3] = {a, b, c};
                            int cell[3];
                            int nout = 0, dout = -1;
                            for (int d = 0; d < 3; ++d) {
                                int ci = idx[d] - 1 + sel[d];
                                if (is_per(g, d)) {
                                    ci = wrap(ci, g->n[d], 1);
                                } else if (ci < 0 || ci >= g->n[d]) {
                                    ++nout;
                                    dout = d;
                                }
                                cell[d] = ci;
                            }
                            long gi = (cell[0] + 1) + (long)G0 * ((cell[1] + 1) + (long)G1 * (cell[2] + 1));
                            if (nout == 0) {
                                for (int d = 0; d < 3; ++d) {
                                    double s = sel[d] ? 1.0 : -1.0;
                                    acc += s * cf[d] * vel_g[d * GC + gi];
                                }
                            } else if (nout == 1) {
                                int bc = cell[dout] < 0 ? g->bclo[dout] : g->bchi[dout];
                                if (bc == OR_INFLOW) {
                                    double s = sel[dout] ? 1.0 : -1.0;
                                    acc += s * cf[dout] * vel_g[dout * GC + gi];
                                }
                            }
                        }
                rhs[u] = -acc;
            }
}

void or_nodal_gradient(const or_grid* g, const double* phi, double* grad)
{
    int nn[3];
    or_nodal_dims(g, nn);
    const long NC = (long)g->n[0] * g->n[1] * g->n[2];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g->n[2]; ++k)
        for (int j = 0; j < g->n[1]; ++j)
            for (int i = 0; i < g->n[0]; ++i) {
                double v[2][2][2];
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b)
                        for (int a = 0; a < 2; ++a) {
                            int ni = wrap(i + a, nn[0], is_per(g, 0));
                            int nj = wrap(j + b, nn[1], is_per(g, 1));
                            int nk = wrap(k + c, nn[2], is_per(g, 2));
                            v[c][b][a] = phi[ni + (long)nn[0] * (nj + (long)nn[1] * nk)];
                        }
                double gx = 0, gy = 0, gz = 0;
                for (int p = 0; p < 2; ++p)
                    for (int q = 0; q < 2; ++q) {
                        gx += v[p][q][1] - v[p][q][0];
                        gy += v[p][1][q] - v[p][0][q];
                        gz += v[1][p][q] - v[0][p][q];
                    }
                long c = i + (long)g->n[0] * (j + (long)g->n[1] * k);
                grad[c] = gx / (4.0 * g->h[0]);
                grad[NC + c] = gy / (4.0 * g->h[1]);
                grad[2 * NC + c] = gz / (4.0 * g->h[2]);
            }
}

/* ------------------------------------------------------------------------------------------
 * MAC discretisation
 * ---------------------------------------------------------------------------------------- */
static inline long fx_id(const or_grid* g, int i, int j, int k)
{
    if (is_per(g, 0) && i == g->n[0]) i = 0;
    return i + (long)(g->n[0] + 1) * (j + (long)g->n[1] * k);
}
static inline long fy_id(const or_grid* g, int i, int j, int k)
{
    if (is_per(g, 1) && j == g->n[1]) j = 0;
    return i + (long)g->n[0] * (j + (long)(g->n[1] + 1) * k);
}
static inline long fz_id(const or_grid* g, int i, int j, int k)
{
    if (is_per(g, 2) && k == g->n[2]) k = 0;
    return i + (long)g->n[0] * (j + (long)g->n[1] * k);
}
static inline long face_id(const or_grid* g, int d, int i, int j, int k)
{
    return d == 0 ? fx_id(g, i, j, k) : (d == 1 ? fy_id(g, i, j, k) : fz_id(g, i, j, k));
}

static void mac_level(const or_grid* g, const double* bx, const double* by, const double* bz, lvl* L)
{
    int per[3];
    for (int d = 0; d < 3; ++d) per[d] = is_per(g, d);
    lvl_alloc(L, g->n, per, 7);
    for (int d = 0; d < 3; ++d)
        if (!per[d] && (g->bclo[d] == OR_DIRICHLET || g->bchi[d] == OR_DIRICHLET)) L->dirichlet = 1;
    const double* beta[3] = {bx, by, bz};
    double V = g->h[0] * g->h[1] * g->h[2];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g->n[2]; ++k)
        for (int j = 0; j < g->n[1]; ++j)
            for (int i = 0; i < g->n[0]; ++i) {
                long u = lid(L, i, j, k);
                L->vol[u] = V;
                double* s = L->st + u * 7;
                int idx[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    double w = V / (g->h[d] * g->h[d]);
                    for (int side = 0; side < 2; ++side) {
                        int f[3] = {i, j, k};
                        f[d] += side; /* face index: low face = idx, high face = idx+1 */
                        double b = beta[d][face_id(g, d, f[0], f[1], f[2])];
                        int at_bnd = !per[d] && ((side == 0 && idx[d] == 0) || (side == 1 && idx[d] == g->n[d] - 1));
                        if (at_bnd) {
                            int bc = side == 0 ? g->bclo[d] : g->bchi[d];
                            if (bc == OR_DIRICHLET) s[0] += 2.0 * w * b;
                        } else {
                            s[0] += w * b;
                            s[1 + 2 * d + side] -= w * b;
                        }
                    }
                }
            }
}

void or_mac_rhs(const or_grid* g, const double* ux, const double* uy, const double* uz, double* rhs)
{
    double V = g->h[0] * g->h[1] * g->h[2];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g->n[2]; ++k)
        for (int j = 0; j < g->n[1]; ++j)
            for (int i = 0; i < g->n[0]; ++i) {
                double dv = (ux[fx_id(g, i + 1, j, k)] - ux[fx_id(g, i, j, k)]) / g->h[0] +
                            (uy[fy_id(g, i, j + 1, k)] - uy[fy_id(g, i, j, k)]) / g->h[1] +
                            (uz[fz_id(g, i, j, k + 1)] - uz[fz_id(g, i, j, k)]) / g->h[2];
                rhs[i + (long)g->n[0] * (j + (long)g->n[1] * k)] = -V * dv;
            }
}

void or_mac_apply(const or_grid* g, const double* bx, const double* by, const double* bz,
                  const double* phi, double* out)
{
    lvl L;
    mac_level(g, bx, by, bz, &L);
    lvl_apply(&L, phi, out);
    lvl_free(&L);
}

void or_mac_correct(const or_grid* g, const double* bx, const double* by, const double* bz,
                    const double* phi, double* ux, double* uy, double* uz)
{
    const double* beta[3] = {bx, by, bz};
    double* vel[3] = {ux, uy, uz};
    for (int d = 0; d < 3; ++d) {
        int fn[3] = {g->n[0], g->n[1], g->n[2]};
        fn[d] += 1;
        int per = is_per(g, d);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < fn[2]; ++k)
            for (int j = 0; j < fn[1]; ++j)
                for (int i = 0; i < fn[0]; ++i) {
                    int f[3] = {i, j, k};
                    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
                    lo[d] -= 1;
                    double phl, phh;
                    long fid = f[0] + (long)fn[0] * (f[1] + (long)fn[1] * f[2]);
                    double b = beta[d][face_id(g, d, i, j, k)];
                    if (per) {
                        lo[d] = wrap(lo[d], g->n[d], 1);
                        hi[d] = wrap(hi[d], g->n[d], 1);
                        phl = phi[lo[0] + (long)g->n[0] * (lo[1] + (long)g->n[1] * lo[2])];
                        phh = phi[hi[0] + (long)g->n[0] * (hi[1] + (long)g->n[1] * hi[2])];
                    } else if (f[d] == 0) {
                        if (g->bclo[d] != OR_DIRICHLET) continue;
                        phh = phi[hi[0] + (long)g->n[0] * (hi[1] + (long)g->n[1] * hi[2])];
                        phl = -phh;
                    } else if (f[d] == g->n[d]) {
                        if (g->bchi[d] != OR_DIRICHLET) continue;
                        phl = phi[lo[0] + (long)g->n[0] * (lo[1] + (long)g->n[1] * lo[2])];
                        phh = -phl;
                    } else {
                        phl = phi[lo[0] + (long)g->n[0] * (lo[1] + (long)g->n[1] * lo[2])];
                        phh = phi[hi[0] + (long)g->n[0] * (hi[1] + (long)g->n[1] * hi[2])];
                    }
                    vel[d][fid] -= b * (phh - phl) / g->h[d];
                }
    }
}

/* ------------------------------------------------------------------------------------------
 * multigrid-preconditioned conjugate gradients
 * ---------------------------------------------------------------------------------------- */
typedef struct {
    int kind; /* 0 nodal, 1 mac */
    int nlev;
    or_grid grid[MAXLEV];
    lvl L[MAXLEV];
    double* x[MAXLEV];
    double* b[MAXLEV];
    double* r[MAXLEV];
    int nu;
    unsigned char* owned_mask[MAXLEV]; /* coarse overset masks built by injection */
} mg_t;

static int can_coarsen(const or_grid* g)
{
    for (int d = 0; d < 3; ++d)
        if ((g->n[d] & 1) || g->n[d] / 2 < 2) return 0;
    return 1;
}

static void coarse_grid(const or_grid* f, or_grid* c)
{
    *c = *f;
    for (int d = 0; d < 3; ++d) {
        c->n[d] = f->n[d] / 2;
        c->h[d] = f->h[d] * 2.0;
    }
}

static void mg_alloc_vectors(mg_t* mg)
{
    for (int l = 0; l < mg->nlev; ++l) {
        size_t n = (size_t)mg->L[l].n;
        mg->x[l] = (double*)calloc(n, sizeof(double));
        mg->b[l] = (double*)calloc(n, sizeof(double));
        mg->r[l] = (double*)calloc(n, sizeof(double));
    }
    lvl* B = &mg->L[mg->nlev - 1];
    if (B->n <= 4096) lvl_dense_factor(B);
}

static void mg_build_nodal(mg_t* mg, const or_grid* g, const double* sigma)
{
    memset(mg, 0, sizeof(*mg));
    mg->kind = 0;
    mg->nu = 2;
    mg->grid[0] = *g;
    double* sg = (double*)malloc(sizeof(double) * (size_t)g->n[0] * g->n[1] * g->n[2]);
    memcpy(sg, sigma, sizeof(double) * (size_t)g->n[0] * g->n[1] * g->n[2]);
    int l = 0;
    for (;;) {
        nodal_level(&mg->grid[l], sg, &mg->L[l]);
        if (l + 1 >= MAXLEV || !can_coarsen(&mg->grid[l])) break;
        or_grid* f = &mg->grid[l];
        or_grid* c = &mg->grid[l + 1];
        coarse_grid(f, c);
        if (f->mask) {
            /* coarse mask by injection: coarse node I is fixed iff fine node 2I is */
            int fn[3], cn[3];
            or_nodal_dims(f, fn);
            or_nodal_dims(c, cn);
            unsigned char* cm = (unsigned char*)malloc((size_t)cn[0] * cn[1] * cn[2]);
            for (int k = 0; k < cn[2]; ++k)
                for (int j = 0; j < cn[1]; ++j)
                    for (int i = 0; i < cn[0]; ++i)
                        cm[i + (long)cn[0] * (j + (long)cn[1] * k)] =
                            f->mask[2 * i + (long)fn[0] * (2 * j + (long)fn[1] * 2 * k)];
            c->mask = cm;
            mg->owned_mask[l + 1] = cm;
        }
        double* cs = (double*)malloc(sizeof(double) * (size_t)c->n[0] * c->n[1] * c->n[2]);
        for (int k = 0; k < c->n[2]; ++k)
            for (int j = 0; j < c->n[1]; ++j)
                for (int i = 0; i < c->n[0]; ++i) {
                    double acc = 0.0;
                    for (int q = 0; q < 8; ++q) {
                        int fi = 2 * i + (q & 1), fj = 2 * j + ((q >> 1) & 1), fk = 2 * k + ((q >> 2) & 1);
                        acc += sg[fi + (long)f->n[0] * (fj + (long)f->n[1] * fk)];
                    }
                    cs[i + (long)c->n[0] * (j + (long)c->n[1] * k)] = 0.125 * acc;
                }
        free(sg);
        sg = cs;
        ++l;
    }
    free(sg);
    mg->nlev = l + 1;
    mg_alloc_vectors(mg);
}

static void mg_build_mac(mg_t* mg, const or_grid* g, const double* bx, const double* by, const double* bz)
{
    memset(mg, 0, sizeof(*mg));
    mg->kind = 1;
    mg->nu = 2;
    mg->grid[0] = *g;
    const double* beta[3] = {bx, by, bz};
    double* cur[3];
    for (int d = 0; d < 3; ++d) {
        int fn[3] = {g->n[0], g->n[1], g->n[2]};
        fn[d] += 1;
        size_t n = (size_t)fn[0] * fn[1] * fn[2];
        cur[d] = (double*)malloc(n * sizeof(double));
        memcpy(cur[d], beta[d], n * sizeof(double));
    }
    int l = 0;
    for (;;) {
        mac_level(&mg->grid[l], cur[0], cur[1], cur[2], &mg->L[l]);
        if (l + 1 >= MAXLEV || !can_coarsen(&mg->grid[l])) break;
        or_grid* f = &mg->grid[l];
        or_grid* c = &mg->grid[l + 1];
        coarse_grid(f, c);
        for (int d = 0; d < 3; ++d) {
            int fn[3] = {f->n[0], f->n[1], f->n[2]};
            int cn[3] = {c->n[0], c->n[1], c->n[2]};
            fn[d] += 1;
            cn[d] += 1;
            double* nbeta = (double*)malloc(sizeof(double) * (size_t)cn[0] * cn[1] * cn[2]);
            for (int k = 0; k < cn[2]; ++k)
                for (int j = 0; j < cn[1]; ++j)
                    for (int i = 0; i < cn[0]; ++i) {
                        int ci[3] = {i, j, k};
                        double acc = 0.0;
                        for (int q = 0; q < 4; ++q) {
                            int fi[3];
                            int t = 0;
                            for (int e = 0; e < 3; ++e) {
                                if (e == d) {
                                    fi[e] = 2 * ci[e];
                                } else {
                                    fi[e] = 2 * ci[e] + ((q >> t) & 1);
                                    ++t;
                                }
                            }
                            acc += cur[d][fi[0] + (long)fn[0] * (fi[1] + (long)fn[1] * fi[2])];
                        }
                        nbeta[i + (long)cn[0] * (j + (long)cn[1] * k)] = 0.25 * acc;
                    }
            free(cur[d]);
            cur[d] = nbeta;
        }
        ++l;
    }
    for (int d = 0; d < 3; ++d) free(cur[d]);
    mg->nlev = l + 1;
    mg_alloc_vectors(mg);
}

static void mg_free(mg_t* mg)
{
    for (int l = 0; l < mg->nlev; ++l) {
        lvl_free(&mg->L[l]);
        free(mg->x[l]);
        free(mg->b[l]);
        free(mg->r[l]);
    }
    for (int l = 0; l < MAXLEV; ++l) {
        free(mg->owned_mask[l]);
        mg->owned_mask[l] = NULL;
    }
    mg->nlev = 0;
}

/* nodal restriction = transpose of trilinear interpolation */
static void restrict_nodal(const mg_t* mg, int l, const double* rf, double* bc)
{
    const lvl* F = &mg->L[l];
    const lvl* C = &mg->L[l + 1];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < C->dims[2]; ++k)
        for (int j = 0; j < C->dims[1]; ++j)
            for (int i = 0; i < C->dims[0]; ++i) {
                long u = lid(C, i, j, k);
                if (C->fixed[u]) {
                    bc[u] = 0.0;
                    continue;
                }
                double acc = 0.0;
                for (int c = -1; c <= 1; ++c)
                    for (int b = -1; b <= 1; ++b)
                        for (int a = -1; a <= 1; ++a) {
                            int fi = wrap(2 * i + a, F->dims[0], F->per[0]);
                            int fj = wrap(2 * j + b, F->dims[1], F->per[1]);
                            int fk = wrap(2 * k + c, F->dims[2], F->per[2]);
                            if (fi < 0 || fj < 0 || fk < 0) continue;
                            double w = (a ? 0.5 : 1.0) * (b ? 0.5 : 1.0) * (c ? 0.5 : 1.0);
                            acc += w * rf[lid(F, fi, fj, fk)];
                        }
                bc[u] = acc;
            }
}

static void prolong_nodal_add(const mg_t* mg, int l, const double* xc, double* xf)
{
    const lvl* F = &mg->L[l];
    const lvl* C = &mg->L[l + 1];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < F->dims[2]; ++k)
        for (int j = 0; j < F->dims[1]; ++j)
            for (int i = 0; i < F->dims[0]; ++i) {
                long u = lid(F, i, j, k);
                if (F->fixed[u]) continue;
                int idx[3] = {i, j, k};
                int lo[3][2];
                int cnt[3];
                for (int d = 0; d < 3; ++d) {
                    if ((idx[d] & 1) == 0) {
                        lo[d][0] = idx[d] / 2;
                        cnt[d] = 1;
                    } else {
                        lo[d][0] = (idx[d] - 1) / 2;
                        lo[d][1] = wrap((idx[d] + 1) / 2, C->dims[d], C->per[d]);
                        cnt[d] = 2;
                    }
                }
                double acc = 0.0;
                for (int c = 0; c < cnt[2]; ++c)
                    for (int b = 0; b < cnt[1]; ++b)
                        for (int a = 0; a < cnt[0]; ++a) {
                            double w = (cnt[0] == 2 ? 0.5 : 1.0) * (cnt[1] == 2 ? 0.5 : 1.0) * (cnt[2] == 2 ? 0.5 : 1.0);
                            acc += w * xc[lid(C, lo[0][a], lo[1][b], lo[2][c])];
                        }
                xf[u] += acc;
            }
}

static void restrict_mac(const mg_t* mg, int l, const double* rf, double* bc)
{
    const lvl* F = &mg->L[l];
    const lvl* C = &mg->L[l + 1];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < C->dims[2]; ++k)
        for (int j = 0; j < C->dims[1]; ++j)
            for (int i = 0; i < C->dims[0]; ++i) {
                double acc = 0.0;
                for (int q = 0; q < 8; ++q)
                    acc += rf[lid(F, 2 * i + (q & 1), 2 * j + ((q >> 1) & 1), 2 * k + ((q >> 2) & 1))];
                bc[lid(C, i, j, k)] = acc;
            }
}

static void prolong_mac_add(const mg_t* mg, int l, const double* xc, double* xf)
{
    const lvl* F = &mg->L[l];
    const lvl* C = &mg->L[l + 1];
#pragma omp parallel for schedule(static)
    for (int k = 0; k < F->dims[2]; ++k)
        for (int j = 0; j < F->dims[1]; ++j)
            for (int i = 0; i < F->dims[0]; ++i) xf[lid(F, i, j, k)] += xc[lid(C, i / 2, j / 2, k / 2)];
}

static void make_consistent(const lvl* L, double* b)
{
    if (any_fixed(L)) return;
    double s = 0.0, v = 0.0;
    for (long u = 0; u < L->n; ++u) {
        s += b[u];
        v += L->vol[u];
    }
    double c = s / v;
    for (long u = 0; u < L->n; ++u) b[u] -= c * L->vol[u];
}

static void vcycle(mg_t* mg, int l)
{
    lvl* L = &mg->L[l];
    double* x = mg->x[l];
    double* b = mg->b[l];
    if (l == mg->nlev - 1) {
        if (L->lu) {
            double* tb = (double*)malloc(sizeof(double) * (size_t)L->n);
            memcpy(tb, b, sizeof(double) * (size_t)L->n);
            make_consistent(L, tb);
            lvl_dense_solve(L, tb, x);
            free(tb);
        } else {
            memset(x, 0, sizeof(double) * (size_t)L->n);
            for (int s = 0; s < 40; ++s) {
                lvl_gs(L, b, x, +1);
                lvl_gs(L, b, x, -1);
            }
        }
        return;
    }
    memset(x, 0, sizeof(double) * (size_t)L->n);
    for (int s = 0; s < mg->nu; ++s) lvl_gs(L, b, x, +1);
    lvl_resid(L, b, x, mg->r[l]);
    if (mg->kind == 0)
        restrict_nodal(mg, l, mg->r[l], mg->b[l + 1]);
    else
        restrict_mac(mg, l, mg->r[l], mg->b[l + 1]);
    vcycle(mg, l + 1);
    if (mg->kind == 0)
        prolong_nodal_add(mg, l, mg->x[l + 1], x);
    else
        prolong_mac_add(mg, l, mg->x[l + 1], x);
#pragma omp parallel for schedule(static)
    for (long u = 0; u < L->n; ++u)
        if (L->fixed[u]) x[u] = 0.0;
    for (int s = 0; s < mg->nu; ++s) lvl_gs(L, b, x, -1);
}

static double dot(const lvl* L, const double* a, const double* b)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long u = 0; u < L->n; ++u) s += a[u] * b[u];
    return s;
}

static double strong_max(const lvl* L, const double* r)
{
    double m = 0.0;
#pragma omp parallel for reduction(max : m) schedule(static)
    for (long u = 0; u < L->n; ++u) {
        double v = fabs(r[u]) / L->vol[u];
        if (v > m) m = v;
    }
    return m;
}

static void gauge(const lvl* L, double* x)
{
    if (any_fixed(L)) return;
    double s = 0.0, v = 0.0;
    for (long u = 0; u < L->n; ++u) {
        s += L->vol[u] * x[u];
        v += L->vol[u];
    }
    double c = s / v;
    for (long u = 0; u < L->n; ++u) x[u] -= c;
}

/* Singular systems (no phi held at 0): the constants are the null space and r stays orthogonal to
 * them; the preconditioned residual is projected the same way (its mean removed), so that rounding in
 * the V-cycle and in the reductions cannot grow a null-space component across iterations. */
static void remove_null_space(const lvl* L, double* z)
{
    if (any_fixed(L)) return;
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long u = 0; u < L->n; ++u) s += z[u];
    s /= (double)L->n;
#pragma omp parallel for schedule(static)
    for (long u = 0; u < L->n; ++u) z[u] -= s;
}

/* stats: [0] iterations, [1] final relative residual (max norm of the strong form),
 *        [2] rhs max norm (strong form), [3] initial relative residual */
static int pcg(mg_t* mg, const double* rhs_in, double* phi, double rtol, double atol, int maxiter, double* stats)
{
    lvl* L = &mg->L[0];
    long n = L->n;
    double* g = (double*)malloc(sizeof(double) * (size_t)n);
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* z = (double*)malloc(sizeof(double) * (size_t)n);
    double* p = (double*)malloc(sizeof(double) * (size_t)n);
    double* q = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(g, rhs_in, sizeof(double) * (size_t)n);
    for (long u = 0; u < n; ++u)
        if (L->fixed[u]) {
            g[u] = 0.0;
            phi[u] = 0.0;
        }
    make_consistent(L, g);
    double bnorm = strong_max(L, g);
    double target = fmax(rtol * bnorm, atol);
    lvl_resid(L, g, phi, r);
    double rn = strong_max(L, r);
    double r0 = rn;
    int it = 0;
    int status = 0;
    if (rn > target) {
        memcpy(mg->b[0], r, sizeof(double) * (size_t)n);
        vcycle(mg, 0);
        memcpy(z, mg->x[0], sizeof(double) * (size_t)n);
        remove_null_space(L, z);
        memcpy(p, z, sizeof(double) * (size_t)n);
        double rz = dot(L, r, z);
        for (it = 1; it <= maxiter; ++it) {
            lvl_apply(L, p, q);
            double pq = dot(L, p, q);
            if (pq == 0.0) break;
            double alpha = rz / pq;
#pragma omp parallel for schedule(static)
            for (long u = 0; u < n; ++u) {
                phi[u] += alpha * p[u];
                r[u] -= alpha * q[u];
            }
            /* recompute the true residual now and then to avoid drift */
            if (it % 10 == 0) lvl_resid(L, g, phi, r);
            rn = strong_max(L, r);
            if (rn <= target) break;
            memcpy(mg->b[0], r, sizeof(double) * (size_t)n);
            vcycle(mg, 0);
            memcpy(z, mg->x[0], sizeof(double) * (size_t)n);
            remove_null_space(L, z);
            double rz2 = dot(L, r, z);
            double beta = rz2 / rz;
            rz = rz2;
#pragma omp parallel for schedule(static)
            for (long u = 0; u < n; ++u) p[u] = z[u] + beta * p[u];
        }
        if (it > maxiter) status = 1;
    }
    gauge(L, phi);
    lvl_resid(L, g, phi, r);
    rn = strong_max(L, r);
    if (stats) {
        stats[0] = it;
        stats[1] = bnorm > 0 ? rn / bnorm : rn;
        stats[2] = bnorm;
        stats[3] = bnorm > 0 ? r0 / bnorm : r0;
    }
    free(g);
    free(r);
    free(z);
    free(p);
    free(q);
    return status;
}

double or_nodal_resid_norm(const or_grid* g, const double* sigma, const double* rhs, const double* phi,
                           double* rhs_norm)
{
    lvl L;
    nodal_level(g, sigma, &L);
    double* r = (double*)malloc(sizeof(double) * (size_t)L.n);
    lvl_resid(&L, rhs, phi, r);
    double rn = strong_max(&L, r);
    if (rhs_norm) {
        double* t = (double*)malloc(sizeof(double) * (size_t)L.n);
        for (long u = 0; u < L.n; ++u) t[u] = L.fixed[u] ? 0.0 : rhs[u];
        *rhs_norm = strong_max(&L, t);
        free(t);
    }
    free(r);
    lvl_free(&L);
    return rn;
}

int or_nodal_solve(const or_grid* g, const double* sigma, const double* rhs, double* phi, double rtol,
                   double atol, int maxiter, double* stats)
{
    mg_t mg;
    mg_build_nodal(&mg, g, sigma);
    int st = pcg(&mg, rhs, phi, rtol, atol, maxiter, stats);
    mg_free(&mg);
    return st;
}

int or_nodal_project(const or_grid* g, const double* sigma, double* vel_g, double* phi, double* gradphi,
                     double rtol, double atol, int maxiter, double* stats)
{
    int nn[3];
    or_nodal_dims(g, nn);
    long nnode = (long)nn[0] * nn[1] * nn[2];
    long nc = (long)g->n[0] * g->n[1] * g->n[2];
    double* rhs = (double*)malloc(sizeof(double) * (size_t)nnode);
    or_nodal_rhs(g, vel_g, rhs);
    memset(phi, 0, sizeof(double) * (size_t)nnode);
    int st = or_nodal_solve(g, sigma, rhs, phi, rtol, atol, maxiter, stats);
    or_nodal_gradient(g, phi, gradphi);
    const int G0 = g->n[0] + 2, G1 = g->n[1] + 2, G2 = g->n[2] + 2;
    const long GC = (long)G0 * G1 * G2;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g->n[2]; ++k)
        for (int j = 0; j < g->n[1]; ++j)
            for (int i = 0; i < g->n[0]; ++i) {
                long c = i + (long)g->n[0] * (j + (long)g->n[1] * k);
                long gi = (i + 1) + (long)G0 * ((j + 1) + (long)G1 * (k + 1));
                for (int d = 0; d < 3; ++d) vel_g[d * GC + gi] -= sigma[c] * gradphi[d * nc + c];
            }
    free(rhs);
    return st;
}

int or_mac_solve(const or_grid* g, const double* bx, const double* by, const double* bz, const double* rhs,
                 double* phi, double rtol, double atol, int maxiter, double* stats)
{
    mg_t mg;
    mg_build_mac(&mg, g, bx, by, bz);
    int st = pcg(&mg, rhs, phi, rtol, atol, maxiter, stats);
    mg_free(&mg);
    return st;
}

int or_mac_project(const or_grid* g, const double* bx, const double* by, const double* bz, double* ux,
                   double* uy, double* uz, double* phi, int phi_is_guess, double rtol, double atol,
                   int maxiter, double* stats)
{
    long nc = (long)g->n[0] * g->n[1] * g->n[2];
    double* rhs = (double*)malloc(sizeof(double) * (size_t)nc);
    or_mac_rhs(g, ux, uy, uz, rhs);
    if (!phi_is_guess) memset(phi, 0, sizeof(double) * (size_t)nc);
    int st = or_mac_solve(g, bx, by, bz, rhs, phi, rtol, atol, maxiter, stats);
    or_mac_correct(g, bx, by, bz, phi, ux, uy, uz);
    free(rhs);
    return st;
}
