// Nodal multigrid driver (host side). One plan = one level geometry + boundary set, kept across
// calls; the reference rebuilds its NodalProjector on every projection
// (src/projection/incflo_apply_nodal_projection.cpp:124,187-192).
//
// Solve structure (residual-correction form, the same loop for both precisions):
//   r = g - A phi (FP64, max norm on the device)        -> stop when |r| <= max(rtol |g|, atol)
//   e = V-cycle(r)   FP64 levels            (plain form)
//     = m V-cycles on (float) r, FP64 bottom (mixed form: FP32 inner solve of iterative refinement)
//   phi += e
// One refinement step (V-cycles + update + residual + norm read-back) is captured once as a
// CUDA graph and replayed; the host reads one 8-byte norm per step.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "nn_unet.h"
#include "nodal_solver.h"
#include "nodal_sweep.h"

namespace gbp {

int DevicePool::reserve(size_t nbytes)
{
    release();
    cudaError_t e = cudaMalloc(&base, nbytes);
    if (e != cudaSuccess) {
        base = nullptr;
        return cuda_fail(e, "cudaMalloc(plan pool)");
    }
    bytes = nbytes;
    used = 0;
    e = cudaMemset(base, 0, nbytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(plan pool)");
    return GBP_OK;
}

void DevicePool::release()
{
    if (base) cudaFree(base);
    base = nullptr;
    bytes = used = 0;
}

static void q1_element(const double h[3], double K[8])
{
    const double V = h[0] * h[1] * h[2];
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

static NodalGeom make_geom(const int n[3], const double h[3], const int per[3], const int dlo[3], const int dhi[3])
{
    NodalGeom g;
    memset(&g, 0, sizeof(g));
    for (int d = 0; d < 3; ++d) {
        g.n[d] = n[d];
        g.per[d] = per[d];
        g.nu[d] = per[d] ? n[d] : n[d] + 1;
        g.dlo[d] = per[d] ? 0 : dlo[d];
        g.dhi[d] = per[d] ? 0 : dhi[d];
        g.h[d] = h[d];
    }
    const long long P0 = padded_row(n[0]);
    g.sy = P0;
    g.sz = P0 * (long long)(n[1] + 3);
    g.count = g.sz * (long long)(n[2] + 3);
    q1_element(h, g.K);
    g.vol = h[0] * h[1] * h[2];
    g.ivol = 1.0 / g.vol;
    const double hm = std::max(h[0], std::max(h[1], h[2]));
    g.iso = fabs(h[0] - h[1]) <= 1e-12 * hm && fabs(h[0] - h[2]) <= 1e-12 * hm;
    if (g.iso) {
        // equal spacing: edge-neighbour couplings vanish, the four far corners share one weight
        const double kc = (g.K[3] + g.K[5] + g.K[6] + g.K[7]) * 0.25;
        g.K[1] = g.K[2] = g.K[4] = 0.0;
        g.K[3] = g.K[5] = g.K[6] = g.K[7] = kc;
        g.K[0] = -4.0 * kc;
    }
    return g;
}

void NodalSolver::destroy()
{
    drop_graphs();
    if (hnorm) cudaFreeHost(hnorm);
    hnorm = nullptr;
    if (cap) cudaStreamDestroy(cap);
    cap = nullptr;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev2) cudaEventDestroy(ev2);
    if (evw) cudaEventDestroy(evw);
    if (evi0) cudaEventDestroy(evi0);
    if (evi1) cudaEventDestroy(evi1);
    evi0 = evi1 = nullptr;
    ev0 = ev1 = ev2 = evw = nullptr;
    if (net_x0) cudaFree(net_x0);
    if (net_scr) cudaFree(net_scr);
    if (phi_last) cudaFree(phi_last);
    if (net_prev) cudaFree(net_prev);
    phi_last = net_prev = nullptr;
    have_last = false;
    net_prev_count = 0;
    net_x0 = nullptr;
    net_scr = nullptr;
    net_x0_bytes = 0;
    net = nullptr;
    if (pool.base) {
        sweep_forget_maps(pool.base, pool.bytes);
        vsweep32_forget_maps(pool.base, pool.bytes);
    }
    eb.pool.release();
    eb = EbState{};
    auxpool.release();
    umask8 = nullptr;
    user_zeros = 0;
    pool.release();
    L.clear();
    sigma_ready = false;
}

int NodalSolver::set_options(const gbp_options& o)
{
    if (o.nu1 < 0 || o.nu2 < 0 || o.nu1 + o.nu2 < 1 || !(o.omega >= 0.0 && o.omega < 2.0) ||
        o.ir_inner_cycles < 1 || o.maxiter < 0) {
        set_error("nodal options: need nu1+nu2 >= 1, 0 <= omega < 2, ir_inner_cycles >= 1, maxiter >= 0");
        return GBP_BAD_ARG;
    }
    const bool regraph = o.precision != opt.precision || o.nu1 != opt.nu1 || o.nu2 != opt.nu2 ||
                         o.omega != opt.omega || o.ir_inner_cycles != opt.ir_inner_cycles ||
                         o.bottom_maxiter != opt.bottom_maxiter || o.bottom_rtol != opt.bottom_rtol ||
                         o.bottom_atol != opt.bottom_atol;
    const int maxc = opt.max_coarsening_level;
    opt = o;
    opt.max_coarsening_level = maxc;  // hierarchy depth is fixed at plan creation
    set_omega();
    if (regraph) {
        drop_graphs();
    }
    return GBP_OK;
}

// The smoother's weights. The Jacobi-scaled operator has lambda_max(D^-1 A) <= lb = 1 + sum_{q != 0} |K_q| /
// K_0 per element (Gershgorin; every cell's row of a node has that ratio, so the sigma-weighted sum does
// too): 2 for cubic cells, more for cells stretched beyond an aspect ratio of about 2, whose positive
// couplings would make a damped Jacobi at 0.85 diverge. All levels share the ratio (every direction
// coarsens by 2).
// omega > 0 (0.85 by default): that fixed weight for every sweep, capped at 0.85 * 2 / lb. omega = 0: the
// nu sweeps of a level's pre- (post-) smoothing take the weights 1 / lambda_k, lambda_k the roots of the
// degree-nu Chebyshev polynomial on [lb / 4, lb], so that together they minimise the largest amplification
// over that interval: for cubic cells and two sweeps 0.220 against 0.490 at 0.85 (the constant-coefficient
// high-frequency modes, lambda in [0.5, 1.5]: 0.220 against 0.331). Post-smoothing takes the weights in
// the reverse order. Cut cells keep the fixed weight (their elements' couplings are not bounded by lb).
// On the 256^3 interface workload the V-cycle contraction is set by the coarse-grid correction: 0.093 per
// V-cycle with the Chebyshev weights against 0.113 at 0.85, but a weaker first V-cycle, and both reach
// 1e-10 in 10 V-cycles, so the fixed weight stays the default.
void NodalSolver::set_omega()
{
    const double w0 = opt.omega > 0.0 ? opt.omega : 0.85;
    omega_eff = w0;
    double lb = 2.0;
    if (!L.empty()) {
        const double* K = L[0].g.K;
        double off = 0.0;
        for (int q = 1; q < 8; ++q) off += fabs(K[q]);
        if (K[0] > 0.0) {
            lb = 1.0 + off / K[0];
            omega_eff = std::min(w0, 0.85 * 2.0 / lb);
        }
    }
    const bool cheb = opt.omega == 0.0 && !eb.on;
    auto fill = [&](double* w, int nu, bool reverse) {
        const int deg = std::max(1, std::min(nu, kSweepWeights));
        for (int p = 0; p < kSweepWeights; ++p) {
            if (!cheb) {
                w[p] = omega_eff;
                continue;
            }
            const int k = (reverse ? deg - 1 - (p % deg) : (p % deg));
            // roots in decreasing order: the smallest weight first
            const double lam = 0.625 * lb + 0.375 * lb * cos((2 * k + 1) * M_PI / (2 * deg));
            w[p] = 1.0 / lam;
        }
    };
    fill(wpre, opt.nu1, false);
    fill(wpost, opt.nu2, true);
}

int NodalSolver::init(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const gbp_options& o,
                      cudaStream_t stream)
{
    destroy();
    opt = o;
    st = stream;
    int n[3], per[3], dlo[3], dhi[3];
    double h[3];
    singular = true;
    for (int d = 0; d < 3; ++d) {
        n[d] = geom.n_cell[d];
        if (n[d] < 2) {
            set_error("nodal plan: every direction needs at least 2 cells");
            return GBP_BAD_ARG;
        }
        h[d] = (geom.prob_hi[d] - geom.prob_lo[d]) / n[d];
        if (!(h[d] > 0.0)) {
            set_error("nodal plan: prob_hi must exceed prob_lo");
            return GBP_BAD_ARG;
        }
        if ((bc_lo[d] == GBP_BC_PERIODIC) != (bc_hi[d] == GBP_BC_PERIODIC)) {
            set_error("nodal plan: a periodic direction must be periodic on both sides");
            return GBP_BAD_ARG;
        }
        for (int s = 0; s < 2; ++s) {
            int b = s ? bc_hi[d] : bc_lo[d];
            if (b < GBP_BC_PERIODIC || b > GBP_BC_INFLOW) {
                set_error("nodal plan: boundary type must be periodic, Dirichlet, Neumann or inflow");
                return GBP_BAD_ARG;
            }
        }
        per[d] = bc_lo[d] == GBP_BC_PERIODIC;
        dlo[d] = bc_lo[d] == GBP_BC_DIRICHLET;
        dhi[d] = bc_hi[d] == GBP_BC_DIRICHLET;
        if (dlo[d] || dhi[d]) singular = false;
    }
    int rc = set_options(o);
    if (rc) return rc;
    opt.max_coarsening_level = o.max_coarsening_level;
    // hierarchy: coarsen by 2 while every direction stays even with >= 2 coarse cells
    L.clear();
    int cn[3] = {n[0], n[1], n[2]};
    double ch[3] = {h[0], h[1], h[2]};
    for (;;) {
        NodalLevel lv;
        lv.g = make_geom(cn, ch, per, dlo, dhi);
        L.push_back(lv);
        bool ok = (int)L.size() <= opt.max_coarsening_level && (int)L.size() < kMaxLevels;
        for (int d = 0; d < 3; ++d) ok = ok && (cn[d] % 2 == 0) && (cn[d] / 2 >= 2);
        if (!ok) break;
        for (int d = 0; d < 3; ++d) {
            cn[d] /= 2;
            ch[d] *= 2.0;
        }
    }
    set_omega();
    const NodalLevel& B = L.back();
    if ((long long)B.g.nu[0] * B.g.nu[1] * B.g.nu[2] > 200000) {
        set_error("nodal plan: the coarsest level is too large for the single-CTA bottom solver "
                  "(cell counts need more factors of 2)");
        return GBP_BAD_ARG;
    }
    // one device pool for the whole plan, zeroed so that all padding holds 0
    size_t need = 0;
    auto add = [&](size_t cnt, size_t sz) { need = ((need + 255) & ~size_t(255)) + cnt * sz; };
    for (auto& lv : L) {
        for (int q = 0; q < 5; ++q) add(lv.g.count, 8);
        for (int q = 0; q < 5; ++q) add(lv.g.count, 4);
        add(lv.g.count, 1);
    }
    const NodalGeom& G0 = L[0].g;
    for (int q = 0; q < 3; ++q) add(G0.count, 8);
    use_qsweep = qsweep_supported(G0);
    if (use_qsweep)
        for (int q = 0; q < 4; ++q) add(G0.count, 8);
    add(nodal_partials_needed(G0) + 64, 8);
    add(5 * B.g.count, 8);
    add(16, 4);
    add(8, 8);
    add(8, 8);
    nbottom = B.g.nu[0] * B.g.nu[1] * B.g.nu[2];
    dense_bottom = nbottom <= kDenseBottomMax;
    if (dense_bottom) add((size_t)nbottom * nbottom, 8);
    need += 4096;
    rc = pool.reserve(need);
    if (rc) return rc;
    for (auto& lv : L) {
        lv.s64 = pool.take<double>(lv.g.count);
        lv.x64 = pool.take<double>(lv.g.count);
        lv.t64 = pool.take<double>(lv.g.count);
        lv.b64 = pool.take<double>(lv.g.count);
        lv.r64 = pool.take<double>(lv.g.count);
        lv.s32 = pool.take<float>(lv.g.count);
        lv.x32 = pool.take<float>(lv.g.count);
        lv.t32 = pool.take<float>(lv.g.count);
        lv.b32 = pool.take<float>(lv.g.count);
        lv.r32 = pool.take<float>(lv.g.count);
        lv.mask8 = pool.take<unsigned char>(lv.g.count);
    }
    singular_faces = singular;
    bsing = singular;
    phi = pool.take<double>(G0.count);
    rhs0 = pool.take<double>(G0.count);
    res = pool.take<double>(G0.count);
    if (use_qsweep) {
        qw.wsum = pool.take<double>(G0.count);
        qw.wx = pool.take<double>(G0.count);
        qw.wy = pool.take<double>(G0.count);
        qw.wz = pool.take<double>(G0.count);
    }
    partials = pool.take<double>(nodal_partials_needed(G0) + 64);
    bscr = pool.take<double>(5 * B.g.count);
    dinfo = pool.take<int>(16);
    derr = reinterpret_cast<unsigned*>(dinfo + 8);
    dnorm = pool.take<unsigned long long>(8);
    dscal = pool.take<double>(8);
    if (dense_bottom) dmat = pool.take<double>((size_t)nbottom * nbottom);
    GBP_CUDA(cudaMallocHost(&hnorm, 8 * sizeof(unsigned long long)));
    memset(hnorm, 0, 8 * sizeof(unsigned long long));
    GBP_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    GBP_CUDA(cudaEventCreate(&ev0));
    GBP_CUDA(cudaEventCreate(&ev1));
    GBP_CUDA(cudaEventCreate(&ev2));
    return GBP_OK;
}

int NodalSolver::set_sigma_from_density(const gbp_array4* rho, double scale, double rho0)
{
    if (!rho && !(rho0 > 0.0)) {
        set_error("sigma: constant density rho0 must be positive");
        return GBP_BAD_ARG;
    }
    nodal_sigma_from_rho(L[0].g, rho, scale, rho0, L[0].s64, L[0].s32, st);
    return finish_sigma();
}

int NodalSolver::set_sigma(const gbp_array4* sigma, double cval)
{
    nodal_sigma_copy(L[0].g, sigma, cval, L[0].s64, L[0].s32, st);
    return finish_sigma();
}

// level 0 holds the caller's sigma: with cut cells keep it aside, leave it on the regular cells only and
// coarsen sigma x volume fraction; then the coarse levels and the bottom
int NodalSolver::finish_sigma()
{
    const double* src0 = L[0].s64;
    if (eb.on) {
        eb_sigma(L[0].g, eb.e, L[0].s64, L[0].s64, L[0].s32, L[0].t64, st);
        src0 = L[0].t64;
    }
    for (size_t l = 1; l < L.size(); ++l)
        nodal_sigma_coarsen(L[l - 1].g, L[l].g, l == 1 ? src0 : L[l - 1].s64, L[l].s64, L[l].s32, st);
    nk += (long long)L.size();
    GBP_CUDA(cudaGetLastError());
    sigma_ready = true;
    return build_bottom();
}

// Dense inverse of the coarsest operator, assembled on the host from the coarsest sigma: the
// bottom solve becomes one FP64 matrix-vector product in one CTA. Singular systems (no Dirichlet
// face) use (A + c 1 1^T)^-1, which solves A x = b exactly for consistent b (sum b = 0).
int NodalSolver::build_bottom()
{
    if (use_qsweep) nodal_qweights64(L[0].g, L[0].s64, qw, st);
    if (!dense_bottom) return GBP_OK;
    const NodalLevel& B = L.back();
    const NodalGeom& g = B.g;
    std::vector<double> sg((size_t)g.count);
    GBP_CUDA(cudaMemcpyAsync(sg.data(), B.s64, sizeof(double) * g.count, cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    const int N = nbottom;
    std::vector<double> A((size_t)N * N, 0.0);
    auto wrapn = [&](int i, int d) { return g.per[d] ? ((i % g.n[d]) + g.n[d]) % g.n[d] : i; };
    std::vector<unsigned char> hm;
    if (g.mask) {
        hm.resize((size_t)g.count);
        GBP_CUDA(cudaMemcpyAsync(hm.data(), g.mask, g.count, cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
    }
    auto dir = [&](int i, int j, int k) {
        return (g.dlo[0] && i == 0) || (g.dhi[0] && i == g.n[0]) || (g.dlo[1] && j == 0) || (g.dhi[1] && j == g.n[1]) ||
               (g.dlo[2] && k == 0) || (g.dhi[2] && k == g.n[2]) ||
               (g.mask && !hm[(size_t)pidx(g.sy, g.sz, i, j, k)]);
    };
    for (int k = 0; k < g.nu[2]; ++k)
        for (int j = 0; j < g.nu[1]; ++j)
            for (int i = 0; i < g.nu[0]; ++i) {
                const int u = i + g.nu[0] * (j + g.nu[1] * k);
                if (dir(i, j, k)) {
                    A[(size_t)u * N + u] = 1.0;
                    continue;
                }
                for (int c = 0; c < 2; ++c)
                    for (int b = 0; b < 2; ++b)
                        for (int a = 0; a < 2; ++a) {
                            int cell[3] = {i - 1 + a, j - 1 + b, k - 1 + c};
                            bool inside = true;
                            for (int d = 0; d < 3; ++d) {
                                if (g.per[d])
                                    cell[d] = wrapn(cell[d], d);
                                else if (cell[d] < 0 || cell[d] >= g.n[d])
                                    inside = false;
                            }
                            if (!inside) continue;
                            const double s = sg[(size_t)pidx(g.sy, g.sz, cell[0], cell[1], cell[2])];
                            for (int r = 0; r < 2; ++r)
                                for (int q = 0; q < 2; ++q)
                                    for (int pp = 0; pp < 2; ++pp) {
                                        int nd[3] = {cell[0] + pp, cell[1] + q, cell[2] + r};
                                        for (int d = 0; d < 3; ++d)
                                            if (g.per[d]) nd[d] = wrapn(nd[d], d);
                                        if (dir(nd[0], nd[1], nd[2])) continue;
                                        const int mask = (pp != 1 - a) | ((q != 1 - b) << 1) | ((r != 1 - c) << 2);
                                        const int v = nd[0] + g.nu[0] * (nd[1] + g.nu[1] * nd[2]);
                                        A[(size_t)u * N + v] += s * g.K[mask];
                                    }
                        }
            }
    if (bsing) {
        double tr = 0.0;
        for (int u = 0; u < N; ++u) tr += A[(size_t)u * N + u];
        const double c = tr / ((double)N * N);
        for (auto& v : A) v += c;
    }
    // Gauss-Jordan inverse with partial pivoting
    std::vector<double> M((size_t)N * N, 0.0);
    for (int u = 0; u < N; ++u) M[(size_t)u * N + u] = 1.0;
    for (int col = 0; col < N; ++col) {
        int piv = col;
        for (int r = col + 1; r < N; ++r)
            if (fabs(A[(size_t)r * N + col]) > fabs(A[(size_t)piv * N + col])) piv = r;
        if (A[(size_t)piv * N + col] == 0.0) {
            set_error("nodal plan: the coarsest operator is singular beyond its constant null space");
            return GBP_BAD_ARG;
        }
        if (piv != col)
            for (int q = 0; q < N; ++q) {
                std::swap(A[(size_t)piv * N + q], A[(size_t)col * N + q]);
                std::swap(M[(size_t)piv * N + q], M[(size_t)col * N + q]);
            }
        const double inv = 1.0 / A[(size_t)col * N + col];
        for (int q = 0; q < N; ++q) {
            A[(size_t)col * N + q] *= inv;
            M[(size_t)col * N + q] *= inv;
        }
        for (int r = 0; r < N; ++r) {
            if (r == col) continue;
            const double f = A[(size_t)r * N + col];
            if (f == 0.0) continue;
            for (int q = 0; q < N; ++q) {
                A[(size_t)r * N + q] -= f * A[(size_t)col * N + q];
                M[(size_t)r * N + q] -= f * M[(size_t)col * N + q];
            }
        }
    }
    // Dirichlet nodes stay 0: zero their rows and columns
    for (int k = 0; k < g.nu[2]; ++k)
        for (int j = 0; j < g.nu[1]; ++j)
            for (int i = 0; i < g.nu[0]; ++i)
                if (dir(i, j, k)) {
                    const int u = i + g.nu[0] * (j + g.nu[1] * k);
                    for (int q = 0; q < N; ++q) M[(size_t)u * N + q] = M[(size_t)q * N + u] = 0.0;
                }
    // stored transposed: step v of the product reads M[v][*] across the threads
    std::vector<double> Mt((size_t)N * N);
    for (int u = 0; u < N; ++u)
        for (int v = 0; v < N; ++v) Mt[(size_t)v * N + u] = M[(size_t)u * N + v];
    GBP_CUDA(cudaMemcpyAsync(dmat, Mt.data(), sizeof(double) * Mt.size(), cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    return GBP_OK;
}

template <>
void NodalSolver::bottom<double>(int l, const double* b, double* x)
{
    const NodalLevel& lv = L[l];
    if (dense_bottom)
        nodal_bottom_dense<double>(lv.g, dmat, b, x, bsing ? 1 : 0, cap_or_st);
    else
        nodal_bottom<double>(lv.g, lv.s64, b, x, bscr, opt.bottom_maxiter, opt.bottom_rtol, opt.bottom_atol, dinfo,
                             bsing ? 1 : 0, cap_or_st);
    xres[l] = x;
}

template <>
void NodalSolver::bottom<float>(int l, const float* b, float* x)
{
    const NodalLevel& lv = L[l];
    if (dense_bottom)
        nodal_bottom_dense<float>(lv.g, dmat, b, x, bsing ? 1 : 0, cap_or_st);
    else
        nodal_bottom<float>(lv.g, lv.s64, b, x, bscr, opt.bottom_maxiter, opt.bottom_rtol, opt.bottom_atol, dinfo,
                            bsing ? 1 : 0, cap_or_st);
    xres[l] = x;
}

template <typename T>
struct LevelBufs;
template <>
struct LevelBufs<double> {
    static double* s(const NodalLevel& l) { return l.s64; }
    static double* x(const NodalLevel& l) { return l.x64; }
    static double* t(const NodalLevel& l) { return l.t64; }
    static double* b(const NodalLevel& l) { return l.b64; }
    static double* r(const NodalLevel& l) { return l.r64; }
};
template <>
struct LevelBufs<float> {
    static float* s(const NodalLevel& l) { return l.s32; }
    static float* x(const NodalLevel& l) { return l.x32; }
    static float* t(const NodalLevel& l) { return l.t32; }
    static float* b(const NodalLevel& l) { return l.b32; }
    static float* r(const NodalLevel& l) { return l.r32; }
};

template <typename T>
void NodalSolver::jacobi(const NodalGeom& g, const T* s, const T* x, const T* b, T* out, double w, cudaStream_t s_)
{
    if (sizeof(T) == 8 && use_qsweep && &g == &L[0].g) {
        nodal_qsweep64(g, 0, reinterpret_cast<const double*>(s), qw, reinterpret_cast<const double*>(x),
                       reinterpret_cast<const double*>(b), reinterpret_cast<double*>(out), w, nullptr, s_);
    } else if (sizeof(T) == 4 && use_tma && vsweep32_supported(g)) {
        int rc = vsweep32(g, 0, reinterpret_cast<const float*>(s), reinterpret_cast<const float*>(x),
                          reinterpret_cast<const float*>(b), reinterpret_cast<float*>(out), (float)w, derr, s_);
        if (rc && !launch_rc) launch_rc = rc;
    } else if (use_tma && sweep_supported(g, (int)sizeof(T))) {
        int rc = nodal_sweep<T>(g, 0, s, x, b, out, w, derr, nullptr, s_);
        if (rc && !launch_rc) launch_rc = rc;
    } else {
        nodal_jacobi<T>(g, s, x, b, out, w, false, s_);
    }
}

template <typename T>
void NodalSolver::resid(const NodalGeom& g, const T* s, const T* x, const T* b, T* r, unsigned long long* norm,
                        cudaStream_t s_)
{
    if (sizeof(T) == 8 && use_qsweep && &g == &L[0].g) {
        nodal_qsweep64(g, 1, reinterpret_cast<const double*>(s), qw, reinterpret_cast<const double*>(x),
                       reinterpret_cast<const double*>(b), reinterpret_cast<double*>(r), omega_eff, norm, s_);
    } else if (sizeof(T) == 4 && !norm && use_tma && vsweep32_supported(g)) {
        int rc = vsweep32(g, 1, reinterpret_cast<const float*>(s), reinterpret_cast<const float*>(x),
                          reinterpret_cast<const float*>(b), reinterpret_cast<float*>(r), 0.f, derr, s_);
        if (rc && !launch_rc) launch_rc = rc;
    } else if (use_tma && sweep_supported(g, (int)sizeof(T))) {
        int rc = nodal_sweep<T>(g, 1, s, x, b, r, omega_eff, derr, norm, s_);
        if (rc && !launch_rc) launch_rc = rc;
    } else {
        nodal_resid<T>(g, s, x, b, r, norm, s_);
    }
}

// First level of the hierarchy cycled by the cluster kernel (k_coarse_vcycle): the first level below
// the finest with at most kCoarseNodes nodes, when the bottom uses the dense inverse and the tail fits
// the kernel's level table; -1 otherwise (every level on its own launches).
int NodalSolver::coarse_first() const
{
    if (!dense_bottom || !use_coarse) return -1;
    for (int l = 1; l + 1 < (int)L.size(); ++l) {
        const NodalGeom& g = L[l].g;
        if ((long long)g.nu[0] * g.nu[1] * g.nu[2] <= kCoarseNodes)
            return ((int)L.size() - l <= kCoarseMaxLevels) ? l : -1;
    }
    return -1;
}

// V-cycle for A x = b on level l. zero: x starts at 0; otherwise from xres[l].
template <typename T>
void NodalSolver::vcycle(int l, const T* b, bool zero)
{
    using B = LevelBufs<T>;
    const NodalLevel& lv = L[l];
    const cudaStream_t s = cap_or_st;
    if (l == (int)L.size() - 1) {
        bottom<T>(l, b, B::x(lv));
        ++nk;
        return;
    }
    // the small levels (this one down to the bottom) in one cluster-resident launch
    if (sizeof(T) == 4 && zero && l >= 1 && l == coarse_first()) {
        CoarseCycle<T> c{};
        c.nl = (int)L.size() - l;
        for (int q = 0; q < c.nl; ++q) {
            const NodalLevel& v = L[l + q];
            c.g[q] = v.g;
            c.s[q] = B::s(v);
            c.x[q] = B::x(v);
            c.t[q] = B::t(v);
            c.b[q] = B::b(v);
            c.r[q] = B::r(v);
        }
        c.b[0] = const_cast<T*>(b);
        c.M = dmat;
        c.singular = bsing ? 1 : 0;
        for (int q = 0; q < kSweepWeights; ++q) {
            c.wpre[q] = (T)wpre[q];
            c.wpost[q] = (T)wpost[q];
        }
        c.nu1 = opt.nu1;
        c.nu2 = opt.nu2;
        int rc = nodal_coarse_vcycle<T>(c, nodal_coarse_cluster_size(), s);
        if (rc && !launch_rc) launch_rc = rc;
        ++nk;
        xres[l] = coarse_result_slot(opt.nu1, opt.nu2) ? B::t(lv) : B::x(lv);
        return;
    }
    T* x = zero ? B::x(lv) : (T*)xres[l];
    T* t = (x == B::x(lv)) ? B::t(lv) : B::x(lv);
    int pre = opt.nu1;
    // cut cells (finest level): the EB nodes are recomputed from the same input after each sweep
    const bool cut = l == 0 && eb.on;
    int q0 = 0;  // pre-smoothing sweeps done
    if (zero) {
        if (pre > 0) {
            nodal_jacobi<T>(lv.g, B::s(lv), nullptr, b, x, wpre[0], true, s);
            if (cut) eb_nodes<T>(lv.g, eb.e, 0, nullptr, b, x, wpre[0], s);
            ++nk;
            q0 = 1;
        } else {
            cudaMemsetAsync(x, 0, sizeof(T) * lv.g.count, s);
        }
    }
    for (int q = q0; q < pre; ++q) {
        const double w = wpre[q % kSweepWeights];
        jacobi<T>(lv.g, B::s(lv), x, b, t, w, s);
        if (cut) eb_nodes<T>(lv.g, eb.e, 0, x, b, t, w, s);
        ++nk;
        std::swap(x, t);
    }
    const NodalLevel& cv = L[l + 1];
    // FP32 levels with whole-row sweeps: residual + restriction in one pass, and the prolongation fused
    // into the first post-smoothing sweep (the coarse level must not be the bottom: the sweeps read the
    // coarse correction's periodic aliases, which the level sweeps write)
    if constexpr (sizeof(T) == 4) {
        if (!cut && use_tma && opt.nu2 >= 1 && l + 2 < (int)L.size() && vsweep32_transfer_supported(lv.g, cv.g)) {
            int rc = vsweep32_resid_restrict(lv.g, cv.g, B::s(lv), x, b, B::b(cv), derr, s);
            if (rc && !launch_rc) launch_rc = rc;
            ++nk;
            vcycle<T>(l + 1, B::b(cv), true);
            rc = vsweep32_prolong_jacobi(lv.g, cv.g, B::s(lv), x, (const T*)xres[l + 1], b, t, (float)wpost[0], derr,
                                         s);
            if (rc && !launch_rc) launch_rc = rc;
            ++nk;
            std::swap(x, t);
            for (int q = 1; q < opt.nu2; ++q) {
                jacobi<T>(lv.g, B::s(lv), x, b, t, wpost[q % kSweepWeights], s);
                ++nk;
                std::swap(x, t);
            }
            xres[l] = x;
            return;
        }
    }
    resid<T>(lv.g, B::s(lv), x, b, B::r(lv), nullptr, s);
    if (cut) eb_nodes<T>(lv.g, eb.e, 1, x, b, B::r(lv), omega_eff, s);
    nodal_restrict<T>(lv.g, cv.g, B::r(lv), B::b(cv), s);
    nk += 2;
    vcycle<T>(l + 1, B::b(cv), true);
    nodal_prolong_add<T>(lv.g, cv.g, (const T*)xres[l + 1], x, s);
    ++nk;
    for (int q = 0; q < opt.nu2; ++q) {
        const double w = wpost[q % kSweepWeights];
        jacobi<T>(lv.g, B::s(lv), x, b, t, w, s);
        if (cut) eb_nodes<T>(lv.g, eb.e, 0, x, b, t, w, s);
        ++nk;
        std::swap(x, t);
    }
    xres[l] = x;
}

// FP64 residual r = b - A x of level 0 with its max norm (into *norm when given)
void NodalSolver::resid0(const double* x, const double* b, double* r, unsigned long long* norm, cudaStream_t s)
{
    const NodalLevel& l0 = L[0];
    if (!eb.on) {
        resid<double>(l0.g, l0.s64, x, b, r, norm, s);
        return;
    }
    resid<double>(l0.g, l0.s64, x, b, r, nullptr, s);
    eb_nodes<double>(l0.g, eb.e, 1, x, b, r, omega_eff, s);
    if (norm) eb_norm(l0.g, r, eb.ivol, norm, s);
}

void NodalSolver::drop_graphs()
{
    for (auto& g : gexec) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// one refinement step, issued on cap_or_st: V-cycle(s) on res, phi += e, res = g - A phi, norm
// (m: FP32 V-cycles of the mixed form's inner solve)
void NodalSolver::record_iteration(int m)
{
    const NodalLevel& l0 = L[0];
    const cudaStream_t s = cap_or_st;
    const long long nk0 = nk;
    if (opt.precision == GBP_PREC_MIXED) {
        nodal_to_f32(l0.g, res, l0.b32, scale32, s);
        vcycle<float>(0, l0.b32, true);
        for (int c = 1; c < m; ++c) vcycle<float>(0, l0.b32, false);
        nodal_add_correction<float>(l0.g, phi, (const float*)xres[0], 1.0 / scale32, s);
        ++nk;
    } else {
        vcycle<double>(0, res, true);
        nodal_add_correction<double>(l0.g, phi, (const double*)xres[0], 1.0, s);
    }
    cudaMemsetAsync(dnorm + 1, 0, sizeof(unsigned long long), s);
    resid0(phi, rhs0, res, dnorm + 1, s);
    nk += 2;
    cudaMemcpyAsync(hnorm + 1, dnorm + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    step_kernels = nk - nk0;
}

void NodalSolver::apply_vcycles(const double* r, double* x, int m, double scale, cudaStream_t s)
{
    const NodalLevel& l0 = L[0];
    cap_or_st = s;
    if (opt.precision == GBP_PREC_MIXED) {
        nodal_to_f32(l0.g, r, l0.b32, scale, s);
        vcycle<float>(0, l0.b32, true);
        for (int c = 1; c < m; ++c) vcycle<float>(0, l0.b32, false);
        nodal_add_correction<float>(l0.g, x, (const float*)xres[0], 1.0 / scale, s);
    } else {
        vcycle<double>(0, r, true);
        for (int c = 1; c < m; ++c) vcycle<double>(0, r, false);
        nodal_add_correction<double>(l0.g, x, (const double*)xres[0], 1.0, s);
    }
    cap_or_st = st;
}

void NodalSolver::apply_vcycles32(const float* b32, int m, cudaStream_t s)
{
    cap_or_st = s;
    vcycle<float>(0, b32, true);
    for (int c = 1; c < m; ++c) vcycle<float>(0, b32, false);
    cap_or_st = st;
}

void NodalSolver::smooth32(const float* b32, int nu, cudaStream_t s)
{
    const NodalLevel& l0 = L[0];
    cap_or_st = s;
    float* x = l0.x32;
    float* t = l0.t32;
    nodal_jacobi<float>(l0.g, l0.s32, nullptr, b32, x, wpre[0], true, s);
    for (int q = 1; q < nu; ++q) {
        jacobi<float>(l0.g, l0.s32, x, b32, t, wpre[q % kSweepWeights], s);
        std::swap(x, t);
    }
    xres[0] = x;
    cap_or_st = st;
}

int NodalSolver::take_sweep_status(cudaStream_t s)
{
    if (launch_rc) {
        const int rc = launch_rc;
        launch_rc = 0;
        return rc;
    }
    unsigned herr = 0;
    GBP_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    GBP_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        GBP_CUDA(cudaMemsetAsync(derr, 0, sizeof(unsigned), s));
        set_error("nodal V-cycle: a bounded device wait (TMA pipeline) ran out");
        return GBP_TIMEOUT;
    }
    return GBP_OK;
}

int NodalSolver::run_iteration(int m)
{
    if (!opt.use_graphs) {
        cap_or_st = st;
        record_iteration(m);
        GBP_CUDA(cudaGetLastError());
        return GBP_OK;
    }
    if (gexec_prec != opt.precision || gexec_scale != scale32) {
        drop_graphs();
        gexec_prec = opt.precision;
        gexec_scale = scale32;
    }
    cudaGraphExec_t& ge = gexec[m];
    if (!ge) {
        cudaGraph_t graph = nullptr;
        cap_or_st = cap;
        GBP_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        record_iteration(m);
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        cap_or_st = st;
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(refinement step)");
        if (launch_rc) {
            cudaGraphDestroy(graph);
            return launch_rc;
        }
        e = cudaGraphInstantiate(&ge, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ge = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate(refinement step)");
        }
        nk -= step_kernels;  // capture issued nothing; the launch below runs them
        step_kernels_m[m] = step_kernels;
    }
    GBP_CUDA(cudaGraphLaunch(ge, st));
    nk += step_kernels_m[m];
    return GBP_OK;
}

static inline double bits_to_double(unsigned long long b)
{
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
}

int NodalSolver::solve(bool have_guess, gbp_stats* stats, bool from_prev)
{
    const NodalLevel& l0 = L[0];
    cap_or_st = st;
    GBP_CUDA(cudaEventRecord(ev1, st));
    if (!have_guess) GBP_CUDA(cudaMemsetAsync(phi, 0, sizeof(double) * l0.g.count, st));
    // dnorm[0] holds |b| (written by project); dnorm[1] receives the initial residual norm
    GBP_CUDA(cudaMemsetAsync(dnorm + 1, 0, 3 * sizeof(unsigned long long), st));
    GBP_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int), st));
    GBP_CUDA(cudaMemsetAsync(derr, 0, sizeof(unsigned), st));
    launch_rc = 0;
    if (have_guess) {
        resid0(phi, rhs0, res, dnorm + 1, st);
        if (launch_rc) return launch_rc;
        ++nk;
    } else {
        // phi = 0: the initial residual is b itself, no FP64 stencil needed
        GBP_CUDA(cudaMemcpyAsync(res, rhs0, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
        GBP_CUDA(cudaMemcpyAsync(dnorm + 1, dnorm, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    }
    GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    const double bnorm = bits_to_double(hnorm[0]);
    double rn = bits_to_double(hnorm[1]);
    if (!isfinite(bnorm) || !isfinite(rn)) {
        set_error("nodal solve: right-hand side or initial residual is not finite");
        if (stats) stats->status = GBP_NAN;
        return GBP_NAN;
    }
    // the tolerance refers to the caller's start (zero or the given guess), not to a warm start
    const double ref = opt.always_use_bnorm ? bnorm : rn;
    const double target = std::max(opt.rtol * ref, opt.atol);
    // power-of-two scale that keeps the FP32 inner right-hand side near unit size
    if (bnorm > 0.0) {
        int ex = 0;
        frexp(bnorm * l0.g.vol, &ex);
        scale32 = ldexp(1.0, -ex);
    }
    if (stats) {
        stats->warm_start = 0;
        stats->warm_rel_resid = 0.0;
        stats->ms_warm = 0.0;
        stats->prev_rel_resid = from_prev ? (bnorm > 0.0 ? rn / bnorm : rn) : 0.0;
    }
    if ((!have_guess || from_prev) && net && net_mode && rn > target) {
        if (warm_skip > 0) {
            // the last attempts were all bypassed: do not pay for the network on this solve
            --warm_skip;
            if (stats) stats->warm_start = 3;
        } else {
            int rc = warm_start(bnorm, &rn, stats, from_prev);
            if (rc) return rc;
        }
    }
    int it = 0, vcycles = 0;
    int status = GBP_OK;
    const double r0 = rn;
    const bool mixed = opt.precision == GBP_PREC_MIXED;
    const int mmax = std::min(opt.ir_inner_cycles, kMaxInner);
    int m = mixed ? mmax : 1;
    if (!evi0) {
        GBP_CUDA(cudaEventCreate(&evi0));
        GBP_CUDA(cudaEventCreate(&evi1));
    }
    GBP_CUDA(cudaEventRecord(evi0, st));
    while (rn > target) {
        if (it >= opt.maxiter) {
            status = GBP_NOT_CONVERGED;
            set_error("solve: maxiter reached before the tolerance");
            break;
        }
        int rc = run_iteration(m);
        if (rc) return rc;
        GBP_CUDA(cudaStreamSynchronize(st));
        const double rprev = rn;
        rn = bits_to_double(hnorm[1]);
        ++it;
        vcycles += m;
        if (mixed && rn > target && rn < rprev && rn > 0.0) {
            // next inner solve: as many V-cycles as the observed per-cycle contraction says the
            // remaining reduction needs (+1/4 cycle of margin), capped by ir_inner_cycles and by
            // what an FP32 inner solve can deliver (about 1e-6 of its right-hand side)
            const double rho = std::min(0.9, std::max(1e-3, pow(rn / rprev, 1.0 / m)));
            const double need = log(std::max(target / rn, 1e-6)) / log(rho);
            m = std::max(1, std::min(mmax, (int)ceil(need + 0.25)));
        }
        if (opt.verbose > 1) fprintf(stderr, "gbp nodal: iter %d rel resid %.3e\n", it, bnorm > 0 ? rn / bnorm : rn);
        if (!isfinite(rn)) {
            status = GBP_NAN;
            set_error("nodal solve: residual became NaN/Inf");
            break;
        }
    }
    GBP_CUDA(cudaEventRecord(evi1, st));
    if (it > 0 && rn > 0.0 && r0 > rn && isfinite(rn)) {
        // the warm start's cost model for the next solve
        float ms_it = 0.f;
        GBP_CUDA(cudaEventSynchronize(evi1));
        cudaEventElapsedTime(&ms_it, evi0, evi1);
        vc_rho = std::min(0.9, pow(rn / r0, 1.0 / vcycles));
        vc_ms = ms_it / vcycles;
    }
    if (singular) {
        nodal_remove_mean(l0.g, phi, partials, dscal, 1, 0, 0, nullptr, st);
        nk += 3;
    }
    if (launch_rc) return launch_rc;
    {
        unsigned herr = 0;
        GBP_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        if (herr) {
            set_error("nodal solve: a bounded device wait (TMA pipeline) ran out");
            if (stats) stats->status = GBP_TIMEOUT;
            return GBP_TIMEOUT;
        }
    }
    GBP_CUDA(cudaEventRecord(ev2, st));
    GBP_CUDA(cudaGetLastError());
    if (stats) {
        stats->status = status;
        stats->outer_iters = it + 1;
        stats->vcycles = vcycles;
        stats->num_levels = (int)L.size();
        stats->rhs_norm = bnorm;
        stats->initial_rel_resid = bnorm > 0 ? r0 / bnorm : r0;
        stats->final_rel_resid = bnorm > 0 ? rn / bnorm : rn;
        GBP_CUDA(cudaEventSynchronize(ev2));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev1, ev2);
        stats->ms_solve = ms;
    }
    if (opt.verbose)
        fprintf(stderr, "gbp nodal: %s after %d steps, rel resid %.3e\n", status == GBP_OK ? "converged" : "stopped",
                it, bnorm > 0 ? rn / bnorm : rn);
    return status;
}

int NodalSolver::set_mask(const gbp_iarray4* m)
{
    user_zeros = 0;
    if (m && m->data) {
        if (!umask8) {
            int rc = auxpool.reserve(L[0].g.count + 4096);
            if (rc) return rc;
            umask8 = auxpool.take<unsigned char>(L[0].g.count);
        }
        unsigned* dz = reinterpret_cast<unsigned*>(dscal + 7);
        GBP_CUDA(cudaMemsetAsync(dz, 0, sizeof(unsigned), st));
        nodal_mask_load(L[0].g, *m, umask8, dz, st);
        GBP_CUDA(cudaMemcpyAsync(&user_zeros, dz, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
    }
    return rebuild_masks();
}

// Level masks from the user's overset mask (nodes held at 0, which pin phi; a coarse node is free where its
// whole fine support is)
// and the cut-cell geometry (nodes that touch no fluid on their own level, which do not pin phi).
int NodalSolver::rebuild_masks()
{
    have_last = false;  // the node set changed: the last solution no longer fits
    const bool um = umask8 && user_zeros > 0;
    const bool em = eb.on && eb.has_inactive;
    if (!um && !em) {
        for (auto& lv : L) lv.g.mask = nullptr;
    } else {
        mask_and(L[0].g.count, um ? umask8 : nullptr, nullptr, L[0].mask8, st);
        L[0].g.mask = L[0].mask8;
        for (size_t l = 1; l < L.size(); ++l) {
            nodal_mask_coarsen(L[l - 1].g, L[l].g, L[l - 1].mask8, L[l].mask8, st);
            L[l].g.mask = L[l].mask8;
        }
        if (em)
            for (size_t l = 0; l < L.size(); ++l) mask_and(L[l].g.count, L[l].mask8, eb.active8[l], L[l].mask8, st);
        GBP_CUDA(cudaGetLastError());
    }
    // nodes that touch no fluid are decoupled on every level (their cells hold no fluid there), so the
    // cut-cell system keeps the constant null space of its free nodes down to the bottom
    singular = singular_faces && !um;
    bsing = singular;
    // the level geometries (captured by value in the graphs) changed
    drop_graphs();
    return sigma_ready ? build_bottom() : GBP_OK;
}

// Q1 element of a cut cell from the second moments of its fluid part (M[p + 3q + 9r] = int xi^p eta^q
// zeta^r dV / V, normalised coordinates in [-1/2, 1/2]): K_ab = int grad N_a . grad N_b, G_a = int grad
// N_a over the fluid part, Gc_a = grad N_a at the fluid centroid. N_a = prod_d (1/2 + s_d xi_d), s = +-1.
static void eb_element(const double* M, const double h[3], double* K, double* G, double* Gc)
{
    auto mom = [&](int p, int q, int r) { return M[p + 3 * q + 9 * r]; };
    auto sg = [](int a, int d) { return ((a >> d) & 1) ? 1.0 : -1.0; };
    const double V = h[0] * h[1] * h[2];
    for (int a = 0; a < 8; ++a) {
        for (int d = 0; d < 3; ++d) {
            const int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
            double acc = 0.0;
            for (int pe = 0; pe < 2; ++pe)
                for (int pf = 0; pf < 2; ++pf) {
                    int idx[3] = {0, 0, 0};
                    idx[e] = pe;
                    idx[f] = pf;
                    acc += (pe ? sg(a, e) : 0.5) * (pf ? sg(a, f) : 0.5) * mom(idx[0], idx[1], idx[2]);
                }
            G[3 * a + d] = sg(a, d) / h[d] * V * acc;
        }
        for (int b = 0; b < 8; ++b) {
            double sum = 0.0;
            for (int d = 0; d < 3; ++d) {
                const int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
                const double ce[3] = {0.25, 0.5 * (sg(a, e) + sg(b, e)), sg(a, e) * sg(b, e)};
                const double cf[3] = {0.25, 0.5 * (sg(a, f) + sg(b, f)), sg(a, f) * sg(b, f)};
                double acc = 0.0;
                for (int pe = 0; pe < 3; ++pe)
                    for (int pf = 0; pf < 3; ++pf) {
                        int idx[3] = {0, 0, 0};
                        idx[e] = pe;
                        idx[f] = pf;
                        acc += ce[pe] * cf[pf] * mom(idx[0], idx[1], idx[2]);
                    }
                sum += sg(a, d) * sg(b, d) / (h[d] * h[d]) * V * acc;
            }
            K[8 * a + b] = sum;
        }
    }
    const double vol = mom(0, 0, 0);
    const double cen[3] = {vol > 0 ? mom(1, 0, 0) / vol : 0.0, vol > 0 ? mom(0, 1, 0) / vol : 0.0,
                           vol > 0 ? mom(0, 0, 1) / vol : 0.0};
    for (int a = 0; a < 8; ++a) {
        double fac[3];
        for (int d = 0; d < 3; ++d) fac[d] = 0.5 + sg(a, d) * cen[d];
        for (int d = 0; d < 3; ++d) {
            const int e = d == 0 ? 1 : 0, f = d == 2 ? 1 : 2;
            Gc[3 * a + d] = sg(a, d) / h[d] * fac[e] * fac[f];
        }
    }
}

int NodalSolver::set_eb(const gbp_array4* M)
{
    drop_graphs();
    GBP_CUDA(cudaStreamSynchronize(st));
    eb.pool.release();
    eb = EbState{};
    sigma_ready = false;  // the level-0 sigma split depends on the geometry: set sigma again
    set_omega();          // cut cells take the fixed smoother weight
    if (!M || !M->data) return rebuild_masks();
    if (M->ncomp < 27) {
        set_error("nodal_set_eb: the moments array needs 27 components");
        return GBP_BAD_ARG;
    }
    const NodalGeom& g = L[0].g;
    const int* n = g.n;
    for (int d = 0; d < 3; ++d)
        if (M->lo[d] > 0 || M->hi[d] < n[d] - 1) {
            set_error("nodal_set_eb: the moments array must cover the cells");
            return GBP_BAD_ARG;
        }
    const long long nc = (long long)n[0] * n[1] * n[2];
    std::vector<double> Mh((size_t)(27 * nc));
    double* tmp = nullptr;
    GBP_CUDA(cudaMalloc(&tmp, sizeof(double) * (size_t)nc));
    int rc = GBP_OK;
    for (int c = 0; c < 27 && !rc; ++c) {
        eb_pack_cells(*M, c, n, tmp, st);
        cudaError_t e = cudaMemcpyAsync(Mh.data() + (size_t)c * nc, tmp, sizeof(double) * (size_t)nc,
                                        cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_fail(e, "nodal_set_eb: copy of the moments");
    }
    cudaFree(tmp);
    if (rc) return rc;
    auto cid = [&](int i, int j, int k) { return i + (long long)n[0] * (j + (long long)n[1] * k); };
    auto kap = [&](long long c) { return Mh[(size_t)c]; };
    // cells: -2 covered, -1 regular, >= 0 cut (table index)
    std::vector<int> ctype((size_t)nc);
    std::vector<EbNodeCell> cells;
    double M27[27];
    for (int k = 0; k < n[2]; ++k)
        for (int j = 0; j < n[1]; ++j)
            for (int i = 0; i < n[0]; ++i) {
                const long long c = cid(i, j, k);
                const double kv = kap(c);
                if (!(kv >= -1e-12 && kv <= 1.0 + 1e-12)) {
                    set_error("nodal_set_eb: volume fractions (moment 0) must lie in [0, 1]");
                    return GBP_BAD_ARG;
                }
                if (kv <= 1e-12) {
                    ctype[(size_t)c] = kEbCovered;
                } else if (kv >= 1.0 - 1e-12) {
                    ctype[(size_t)c] = kEbRegular;
                } else {
                    EbNodeCell ec{};
                    ec.p = pidx(g.sy, g.sz, i, j, k);
                    ec.i = i;
                    ec.j = j;
                    ec.k = k;
                    for (int q = 0; q < 27; ++q) M27[q] = Mh[(size_t)q * nc + c];
                    eb_element(M27, g.h, ec.K, ec.G, ec.Gc);
                    ctype[(size_t)c] = (int)cells.size();
                    cells.push_back(ec);
                }
            }
    auto wrapc = [&](int v, int d, bool& inside) {
        if (g.per[d]) return ((v % n[d]) + n[d]) % n[d];
        inside = inside && v >= 0 && v < n[d];
        return v;
    };
    // nodes: active (touches fluid), EB (touches a cut cell)
    std::vector<EbNodeEntry> nodes;
    std::vector<unsigned char> act_u((size_t)g.nu[0] * g.nu[1] * g.nu[2], 0);
    bool inactive = false;
    for (int k = 0; k < g.nu[2]; ++k)
        for (int j = 0; j < g.nu[1]; ++j)
            for (int i = 0; i < g.nu[0]; ++i) {
                EbNodeEntry nd{};
                nd.i = i;
                nd.j = j;
                nd.k = k;
                bool has_cut = false, has_fluid = false;
                for (int c = 0; c < 8; ++c) {
                    bool inside = true;
                    const int ci = wrapc(i - 1 + (c & 1), 0, inside), cj = wrapc(j - 1 + ((c >> 1) & 1), 1, inside),
                              ck = wrapc(k - 1 + (c >> 2), 2, inside);
                    int t = kEbCovered;
                    if (inside) t = ctype[(size_t)cid(ci, cj, ck)];
                    nd.cell[c] = t;
                    has_cut = has_cut || t >= 0;
                    has_fluid = has_fluid || t != kEbCovered;
                }
                act_u[(size_t)(i + g.nu[0] * ((size_t)j + (size_t)g.nu[1] * k))] = has_fluid;
                inactive = inactive || !has_fluid;
                if (has_cut) nodes.push_back(nd);
            }
    // padded arrays (periodic aliases filled): volume fraction, regular-cell flag, active-node flag
    std::vector<double> kap_p((size_t)g.count, 0.0), ivol_p((size_t)g.count, 0.0);
    std::vector<unsigned char> reg_p((size_t)g.count, 0), act_p((size_t)g.count, 0);
    // fluid volume of each unique node's dual cell: kappa V / 8 from each of its 8 cells
    std::vector<double> vf_u(act_u.size(), 0.0);
    for (int k = 0; k < g.nu[2]; ++k)
        for (int j = 0; j < g.nu[1]; ++j)
            for (int i = 0; i < g.nu[0]; ++i) {
                double v = 0.0;
                for (int c = 0; c < 8; ++c) {
                    bool inside = true;
                    const int ci = wrapc(i - 1 + (c & 1), 0, inside), cj = wrapc(j - 1 + ((c >> 1) & 1), 1, inside),
                              ck = wrapc(k - 1 + (c >> 2), 2, inside);
                    if (inside) v += kap(cid(ci, cj, ck)) * g.vol / 8.0;
                }
                vf_u[(size_t)(i + g.nu[0] * ((size_t)j + (size_t)g.nu[1] * k))] = v;
            }
    for (int k = -1; k <= n[2]; ++k)
        for (int j = -1; j <= n[1]; ++j)
            for (int i = -1; i <= n[0]; ++i) {
                bool inside = true;
                const int ci = wrapc(i, 0, inside), cj = wrapc(j, 1, inside), ck = wrapc(k, 2, inside);
                const long long p = pidx(g.sy, g.sz, i, j, k);
                if (inside) {
                    const long long c = cid(ci, cj, ck);
                    kap_p[(size_t)p] = kap(c);
                    reg_p[(size_t)p] = ctype[(size_t)c] == kEbRegular;
                }
                // node (i, j, k): unique index by periodic wrap of the node index space
                bool nin = true;
                int ni[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    if (g.per[d])
                        ni[d] = ((ni[d] % n[d]) + n[d]) % n[d];
                    else if (ni[d] < 0 || ni[d] >= g.nu[d])
                        nin = false;
                }
                if (nin) {
                    const size_t u = (size_t)(ni[0] + g.nu[0] * ((size_t)ni[1] + (size_t)g.nu[1] * ni[2]));
                    act_p[(size_t)p] = act_u[u];
                    ivol_p[(size_t)p] = vf_u[u] > 0.0 ? 1.0 / vf_u[u] : 0.0;
                }
            }
    // coarse levels: a cell holds fluid when one of its 8 fine cells does; a node is active when one of
    // its cells holds fluid. (Injecting the level-0 flags instead would pin the coarse nodes that lie in
    // the body next to fluid and stall the coarse correction along the boundary.)
    std::vector<std::vector<unsigned char>> act_lv(L.size());
    act_lv[0] = act_p;
    {
        std::vector<unsigned char> fl((size_t)nc);
        for (long long c = 0; c < nc; ++c) fl[(size_t)c] = ctype[(size_t)c] != kEbCovered;
        for (size_t l = 1; l < L.size(); ++l) {
            const NodalGeom& f = L[l - 1].g;
            const NodalGeom& cg = L[l].g;
            const int* m = cg.n;
            std::vector<unsigned char> cf((size_t)m[0] * m[1] * m[2], 0);
            for (int k = 0; k < m[2]; ++k)
                for (int j = 0; j < m[1]; ++j)
                    for (int i = 0; i < m[0]; ++i) {
                        unsigned char v = 0;
                        for (int c = 0; c < 8; ++c)
                            v |= fl[(size_t)((2 * i + (c & 1)) +
                                             (long long)f.n[0] * ((2 * j + ((c >> 1) & 1)) +
                                                                  (long long)f.n[1] * (2 * k + (c >> 2))))];
                        cf[(size_t)(i + (long long)m[0] * (j + (long long)m[1] * k))] = v;
                    }
            std::vector<unsigned char> ap((size_t)cg.count, 0);
            for (int k = -1; k <= m[2]; ++k)
                for (int j = -1; j <= m[1]; ++j)
                    for (int i = -1; i <= m[0]; ++i) {
                        int ni[3] = {i, j, k};
                        bool nin = true;
                        for (int d = 0; d < 3; ++d) {
                            if (cg.per[d])
                                ni[d] = ((ni[d] % m[d]) + m[d]) % m[d];
                            else if (ni[d] < 0 || ni[d] > m[d])
                                nin = false;
                        }
                        if (!nin) continue;
                        unsigned char v = 0;
                        for (int c = 0; c < 8; ++c) {
                            int ci[3] = {ni[0] - 1 + (c & 1), ni[1] - 1 + ((c >> 1) & 1), ni[2] - 1 + (c >> 2)};
                            bool in = true;
                            for (int d = 0; d < 3; ++d) {
                                if (cg.per[d])
                                    ci[d] = ((ci[d] % m[d]) + m[d]) % m[d];
                                else
                                    in = in && ci[d] >= 0 && ci[d] < m[d];
                            }
                            if (in) v |= cf[(size_t)(ci[0] + (long long)m[0] * (ci[1] + (long long)m[1] * ci[2]))];
                        }
                        ap[(size_t)pidx(cg.sy, cg.sz, i, j, k)] = v;
                    }
            act_lv[l].swap(ap);
            fl.swap(cf);
        }
    }
    size_t need = 0;
    auto add = [&](size_t cnt, size_t sz) { need = ((need + 255) & ~size_t(255)) + cnt * sz; };
    add(nodes.size() + 1, sizeof(EbNodeEntry));
    add(cells.size() + 1, sizeof(EbNodeCell));
    add(g.count, 8);
    add(g.count, 1);
    for (size_t l = 0; l < L.size(); ++l) add(L[l].g.count, 1);
    add(g.count, 8);
    add(g.count, 4);
    add(g.count, 8);
    add(8 * cells.size() + 8, 8);
    need += 4096;
    rc = eb.pool.reserve(need);
    if (rc) return rc;
    EbNodeEntry* dn = eb.pool.take<EbNodeEntry>(nodes.size() + 1);
    EbNodeCell* dc = eb.pool.take<EbNodeCell>(cells.size() + 1);
    double* dk = eb.pool.take<double>(g.count);
    unsigned char* dr = eb.pool.take<unsigned char>(g.count);
    for (size_t l = 0; l < L.size(); ++l) eb.active8[l] = eb.pool.take<unsigned char>(L[l].g.count);
    double* s64t = eb.pool.take<double>(g.count);
    float* s32t = eb.pool.take<float>(g.count);
    eb.ivol = eb.pool.take<double>(g.count);
    eb.inflow_buf = eb.pool.take<double>(8 * cells.size() + 8);
    if (!nodes.empty())
        GBP_CUDA(cudaMemcpyAsync(dn, nodes.data(), sizeof(EbNodeEntry) * nodes.size(), cudaMemcpyHostToDevice, st));
    if (!cells.empty())
        GBP_CUDA(cudaMemcpyAsync(dc, cells.data(), sizeof(EbNodeCell) * cells.size(), cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dk, kap_p.data(), sizeof(double) * g.count, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dr, reg_p.data(), g.count, cudaMemcpyHostToDevice, st));
    for (size_t l = 0; l < L.size(); ++l)
        GBP_CUDA(cudaMemcpyAsync(eb.active8[l], act_lv[l].data(), L[l].g.count, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(eb.ivol, ivol_p.data(), sizeof(double) * g.count, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemsetAsync(s64t, 0, sizeof(double) * g.count, st));
    GBP_CUDA(cudaMemsetAsync(s32t, 0, sizeof(float) * g.count, st));
    GBP_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
    eb.e.nodes = dn;
    eb.e.cells = dc;
    eb.e.nnodes = (int)nodes.size();
    eb.e.ncells = (int)cells.size();
    eb.e.sig64 = s64t;
    eb.e.sig32 = s32t;
    eb.e.kap = dk;
    eb.e.reg = dr;
    eb.has_inactive = inactive;
    eb.on = true;
    set_omega();
    return rebuild_masks();
}

double* NodalSolver::residual_of(const double* x)
{
    cap_or_st = st;
    launch_rc = 0;
    resid0(x, rhs0, L[0].r64, nullptr, st);
    return L[0].r64;
}

int NodalSolver::set_eb_inflow(const gbp_array4* eb_vel, const gbp_array4* dap, const gbp_array4* bcent)
{
    if (!eb_vel) {
        eb.e.inflow = nullptr;
        return GBP_OK;
    }
    if (!eb.on) {
        set_error("nodal_set_eb_inflow: the plan has no embedded boundary (nodal_set_eb first)");
        return GBP_BAD_ARG;
    }
    eb.e.inflow = nullptr;  // the shares are computed from the table without the old ones
    eb_inflow_shares(L[0].g, eb.e, *eb_vel, *dap, *bcent, eb.inflow_buf, st);
    GBP_CUDA(cudaGetLastError());
    eb.e.inflow = eb.inflow_buf;
    return GBP_OK;
}

int NodalSolver::set_surrogate(nn::UNet* n, int level, int mode)
{
    if (n && (level < 0 || level >= (int)L.size())) {
        set_error("set_surrogate: level must be a multigrid level of the plan");
        return GBP_BAD_ARG;
    }
    if (n != net || level != net_level) warm_streak = warm_skip = 0;
    net = n;
    net_level = level;
    net_mode = n ? mode : 0;
    if (!n) return GBP_OK;
    int dims[3];
    nn::net_dims(L[level].g, dims);
    const size_t need = (size_t)(dims[0] + 2) * (dims[1] + 2) * (dims[2] + 2) * nn::kInC * sizeof(__nv_bfloat16);
    if (need > net_x0_bytes) {
        if (net_x0) cudaFree(net_x0);
        net_x0 = nullptr;
        net_x0_bytes = 0;
        GBP_CUDA(cudaMalloc(&net_x0, need));
        GBP_CUDA(cudaMemset(net_x0, 0, need));
        net_x0_bytes = need;
    }
    if (!net_scr) GBP_CUDA(cudaMalloc(&net_scr, 8 * sizeof(double)));
    if (!evw) GBP_CUDA(cudaEventCreate(&evw));
    return net->workspace(dims, false);
}

// Warm start from the network: restrict the FP32 residual of the start it would replace (the right-hand
// side itself from a zero start) to the network's level, predict,
// prolong to level 0, scale by the Galerkin factor alpha = x.r / x.Ax (the scaled prediction is the best
// multiple of x in the energy norm), then take it only if its FP64 residual beats the start it would
// replace. From a zero start the network predicts phi (input phi_prev = 0) and competes with phi = 0;
// from the previous solution (from_prev: phi / res hold it and its residual) it predicts the increment
// with phi_prev injected onto its level, the candidate is phi_prev + alpha x, and it competes with the
// previous-phi start. On return phi / res / *rn describe the chosen start.
int NodalSolver::warm_start(double bnorm, double* rn, gbp_stats* stats, bool from_prev)
{
    const NodalLevel& l0 = L[0];
    const int lv = net_level;
    const long long nk0 = net->launches();
    GBP_CUDA(cudaEventRecord(evw, st));
    launch_rc = 0;
    // channel 0: the residual of the start being replaced (the right-hand side itself from zero)
    nodal_to_f32(l0.g, from_prev ? res : rhs0, l0.b32, scale32, st);
    for (int l = 0; l < lv; ++l) nodal_restrict<float>(L[l].g, L[l + 1].g, L[l].b32, L[l + 1].b32, st);
    int dims[3];
    nn::net_dims(L[lv].g, dims);
    int rc = net->workspace(dims, false);
    const double* prev_lv = nullptr;
    if (!rc && from_prev) {
        if ((size_t)L[lv].g.count > net_prev_count) {
            if (net_prev) cudaFree(net_prev);
            net_prev = nullptr;
            net_prev_count = 0;
            GBP_CUDA(cudaMalloc(&net_prev, sizeof(double) * L[lv].g.count));
            GBP_CUDA(cudaMemsetAsync(net_prev, 0, sizeof(double) * L[lv].g.count, st));
            net_prev_count = L[lv].g.count;
        }
        rc = nn::inject_nodes(l0.g, L[lv].g, 1 << lv, phi, net_prev, st);
        prev_lv = net_prev;
    }
    if (!rc) rc = nn::build_input<float>(L[lv].g, L[lv].b32, L[lv].s32, prev_lv, net->grid0(), net_x0, net_scr, st);
    if (!rc) rc = net->forward(net_x0, st);
    if (!rc) rc = nn::extract_output(net->grid0(), net->hout(), L[lv].g, L[lv].x32, st);
    if (rc) return rc;
    for (int l = lv - 1; l >= 0; --l) {
        GBP_CUDA(cudaMemsetAsync(L[l].x32, 0, sizeof(float) * L[l].g.count, st));
        nodal_prolong_add<float>(L[l].g, L[l + 1].g, L[l + 1].x32, L[l].x32, st);
    }
    // Galerkin factor against the residual of the start being replaced (b32 still holds it); the
    // scaled prediction is then smoothed by two Jacobi sweeps of A x = b32 (the short-wavelength error a
    // prediction leaves dominates its residual, and the smoother removes it for 0.2 ms) and scaled again
    double d[2] = {0.0, 0.0};
    double alpha = 0.0;
    for (int pass = 0; pass < 2; ++pass) {
        resid<float>(l0.g, l0.s32, l0.x32, l0.b32, l0.r32, nullptr, st);
        if (launch_rc) return launch_rc;
        rc = nn::node_dot2(l0.g, l0.x32, l0.b32, l0.r32, net_scr, st);
        if (rc) return rc;
        GBP_CUDA(cudaMemcpyAsync(d, net_scr, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        const double xax = d[0] - d[1];  // x.(b - r) = x.Ax in the scaled units of b32
        const double a = (xax > 0.0 && isfinite(d[0])) ? d[0] / xax : 0.0;
        if (pass == 1 || a == 0.0) {
            alpha = a / scale32;
            break;
        }
        rc = nn::scale32(l0.g.count, l0.x32, (float)a, st);
        if (rc) return rc;
        for (int q = 0; q < 2; ++q) {
            float* xin = q == 0 ? l0.x32 : l0.t32;
            float* xout = q == 0 ? l0.t32 : l0.x32;
            jacobi<float>(l0.g, l0.s32, xin, l0.b32, xout, omega_eff, st);
            if (eb.on) eb_nodes<float>(l0.g, eb.e, 0, xin, l0.b32, xout, omega_eff, st);
        }
        if (launch_rc) return launch_rc;
    }
    nk += net->launches() - nk0 + 6 + 2 * lv + (from_prev ? 2 : 0) + 6;
    double rw = *rn;
    // candidate phi (phi_prev + alpha x, or alpha x) and its FP64 residual, in the level-0 FP64 scratch
    double* cand = from_prev ? l0.t64 : phi;
    double* cres = from_prev ? l0.r64 : res;
    if (alpha != 0.0) {
        rc = from_prev ? nn::axpy_to64(l0.g.count, phi, l0.x32, alpha, cand, st)
                       : nn::scale_to64(l0.g.count, l0.x32, alpha, cand, st);
        if (rc) return rc;
        GBP_CUDA(cudaMemsetAsync(dnorm + 2, 0, sizeof(unsigned long long), st));
        resid0(cand, rhs0, cres, dnorm + 2, st);
        if (launch_rc) return launch_rc;
        nk += 2;
        GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        rw = bits_to_double(hnorm[2]);
    }
    // taken when its residual is below the start it would replace, and (once a solve has measured the
    // V-cycle contraction and cost) when the V-cycles that smaller residual saves cost more than the
    // network's device time so far
    bool take = alpha != 0.0 && isfinite(rw) && rw < *rn;
    double saved_ms = 0.0, spent_ms = 0.0;
    if (take && vc_rho > 0.0 && vc_rho < 1.0 && vc_ms > 0.0) {
        GBP_CUDA(cudaEventRecord(ev2, st));
        GBP_CUDA(cudaEventSynchronize(ev2));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, evw, ev2);
        spent_ms = ms;
        saved_ms = log(rw / *rn) / log(vc_rho) * vc_ms;
        take = saved_ms > spent_ms;
    }
    // two bypasses in a row: skip the next 16 attempts, then try again
    warm_streak = take ? 0 : warm_streak + 1;
    if (warm_streak >= 2) {
        warm_skip = 16;
        warm_streak = 0;
    }
    if (take) {
        if (from_prev) {
            GBP_CUDA(cudaMemcpyAsync(phi, cand, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
            GBP_CUDA(cudaMemcpyAsync(res, cres, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
        }
        GBP_CUDA(cudaMemcpyAsync(dnorm + 1, dnorm + 2, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
        *rn = rw;
    } else if (!from_prev) {
        // bypass: back to the zero start (the previous-phi start was left in phi / res untouched)
        GBP_CUDA(cudaMemsetAsync(phi, 0, sizeof(double) * l0.g.count, st));
        GBP_CUDA(cudaMemcpyAsync(res, rhs0, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
        GBP_CUDA(cudaMemcpyAsync(dnorm + 1, dnorm, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    }
    GBP_CUDA(cudaEventRecord(ev2, st));
    GBP_CUDA(cudaEventSynchronize(ev2));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, evw, ev2);
        stats->warm_start = take ? 1 : 2;
        stats->warm_rel_resid = bnorm > 0.0 ? rw / bnorm : rw;
        stats->ms_warm = ms;
    }
    if (opt.verbose)
        fprintf(stderr, "gbp nodal: warm start (%s) alpha %.4e, rel resid %.3e, saves %.3f ms of V-cycles for %.3f ms (%s)\n",
                from_prev ? "increment" : "phi", alpha, bnorm > 0 ? rw / bnorm : rw, saved_ms, spent_ms,
                take ? "used" : "bypassed");
    return GBP_OK;
}

int NodalSolver::project(const RhsArgs& rhs, const CorrArgs& corr, gbp_array4* phi_out, int phi_accumulate,
                         const gbp_array4* phi_guess, gbp_stats* stats, const HostCopy* phi_copy,
                         const HostSlabs* out_slabs, const RhsGroups* rhs_groups)
{
    if (!sigma_ready) {
        set_error("nodal project: sigma was never set on this plan");
        return GBP_BAD_ARG;
    }
    const NodalLevel& l0 = L[0];
    GBP_CUDA(cudaEventRecord(ev0, st));
    GBP_CUDA(cudaMemsetAsync(dnorm, 0, sizeof(unsigned long long), st));
    RhsArgs ra = rhs;
    if (eb.on) ra.cmask = eb.e.reg;  // cut and covered cells: the cut-cell table below
    if (rhs_groups && rhs_groups->n > 0 && !eb.on) {
        // each group of z chunks as soon as the cells it reads are on the device
        const RhsGroups& G = *rhs_groups;
        for (int q = 0; q < G.n; ++q) {
            GBP_CUDA(cudaStreamWaitEvent(st, G.ev[q], 0));
            if (q == 0 && l0.g.per[2]) GBP_CUDA(cudaStreamWaitEvent(st, G.ev[G.n - 1], 0));
            nodal_rhs(l0.g, ra, l0.s64, rhs0, singular ? partials : nullptr, st, G.zb[q], G.zb[q + 1]);
            ++nk;
        }
    } else {
        nodal_rhs(l0.g, ra, l0.s64, rhs0, singular ? partials : nullptr, st);
        ++nk;
    }
    if (eb.on) eb_rhs(l0.g, eb.e, ra, rhs0, st);
    if (singular) {
        // consistent right-hand side, and its max norm (the relative-tolerance reference; with cut
        // cells taken again below over the fluid volumes)
        // (the cut cells' int u . grad N sum to zero over each cell's corners, an EB inflow does not:
        // then the sums are taken again over the assembled right-hand side)
        const bool fresh = eb.on && eb.e.inflow != nullptr;
        nodal_remove_mean(l0.g, rhs0, partials, dscal, 0, fresh ? 0 : 1, nodal_rhs_partials(l0.g), dnorm, st);
        nk += fresh ? 3 : 2;
    } else {
        nodal_norm(l0.g, rhs0, dnorm, st);
        ++nk;
    }
    if (eb.on) {
        GBP_CUDA(cudaMemsetAsync(dnorm, 0, sizeof(unsigned long long), st));
        eb_norm(l0.g, rhs0, eb.ivol, dnorm, st);
    }
    if (phi_guess) {
        nodal_load_phi(l0.g, *phi_guess, phi, st);
        ++nk;
    }
    // initial_guess = previous: the last solution of this plan is the start (unless the caller gave one)
    const bool from_prev = !phi_guess && opt.initial_guess == 1 && have_last;
    if (from_prev) GBP_CUDA(cudaMemcpyAsync(phi, phi_last, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
    GBP_CUDA(cudaGetLastError());
    int status = solve(phi_guess != nullptr || from_prev, stats, from_prev);
    if (status != GBP_OK && status != GBP_NOT_CONVERGED) return status;
    if (opt.initial_guess == 1) {
        if (!phi_last) GBP_CUDA(cudaMalloc(&phi_last, sizeof(double) * l0.g.count));
        GBP_CUDA(cudaMemcpyAsync(phi_last, phi, sizeof(double) * l0.g.count, cudaMemcpyDeviceToDevice, st));
        have_last = status == GBP_OK;
    }
    // p_nd first: its copy-out can then overlap the velocity correction
    if (phi_out && phi_out->data) {
        nodal_store_phi(l0.g, *phi_out, phi, phi_accumulate, st);
        ++nk;
        if (phi_copy && phi_copy->dst) {
            GBP_CUDA(cudaEventRecord(phi_copy->ev, st));
            GBP_CUDA(cudaStreamWaitEvent(phi_copy->stream, phi_copy->ev, 0));
            GBP_CUDA(cudaMemcpyAsync(phi_copy->dst, phi_copy->src, phi_copy->bytes, cudaMemcpyDeviceToHost,
                                     phi_copy->stream));
        }
    }
    CorrArgs ca = corr;
    if (eb.on) ca.cmask = eb.e.reg;
    if (out_slabs && out_slabs->nslabs > 0 && !eb.on) {
        // correction by z-slabs, each slab's velocity and gp copied out while the next is corrected
        const HostSlabs& o = *out_slabs;
        const int nz = l0.g.n[2];
        for (int q = 0; q < o.nslabs; ++q) {
            const int k0 = (int)((long long)nz * q / o.nslabs), k1 = (int)((long long)nz * (q + 1) / o.nslabs);
            if (k1 <= k0) continue;
            nodal_correct(l0.g, ca, l0.s64, phi, st, k0, k1);
            ++nk;
            GBP_CUDA(cudaEventRecord(o.ev[q], st));
            GBP_CUDA(cudaStreamWaitEvent(o.stream, o.ev[q], 0));
            const size_t off = (size_t)k0 * o.plane, cnt = (size_t)(k1 - k0) * o.plane;
            for (int c = 0; c < 3; ++c) {
                GBP_CUDA(cudaMemcpyAsync(o.hvel + c * o.ncell + off, o.dvel + c * o.ncell + off, cnt * sizeof(double),
                                         cudaMemcpyDeviceToHost, o.stream));
                GBP_CUDA(cudaMemcpyAsync(o.hgp + c * o.ncell + off, o.dgp + c * o.ncell + off, cnt * sizeof(double),
                                         cudaMemcpyDeviceToHost, o.stream));
            }
        }
    } else {
        nodal_correct(l0.g, ca, l0.s64, phi, st);
        ++nk;
        if (eb.on) eb_correct(l0.g, eb.e, corr, phi, st);
        if (out_slabs && out_slabs->nslabs > 0) {
            // cut cells: one copy after the whole correction
            const HostSlabs& o = *out_slabs;
            GBP_CUDA(cudaEventRecord(o.ev[0], st));
            GBP_CUDA(cudaStreamWaitEvent(o.stream, o.ev[0], 0));
            GBP_CUDA(cudaMemcpyAsync(o.hvel, o.dvel, 3 * o.ncell * sizeof(double), cudaMemcpyDeviceToHost, o.stream));
            GBP_CUDA(cudaMemcpyAsync(o.hgp, o.dgp, 3 * o.ncell * sizeof(double), cudaMemcpyDeviceToHost, o.stream));
        }
    }
    GBP_CUDA(cudaEventRecord(ev2, st));
    GBP_CUDA(cudaGetLastError());
    if (stats) {
        GBP_CUDA(cudaEventSynchronize(ev2));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev2);
        stats->ms_total = ms;
        stats->kernel_launches = nk;
    }
    return status;
}

}  // namespace gbp

namespace gbp {

int NodalSolver::time_kernel(int which, int reps, double* ms, double* bytes)
{
    if (which < 0 || which > 9 || reps < 1 || !sigma_ready || (which >= 6 && L.size() < 2)) {
        set_error("time_kernel: which must be 0..9 (6..9 need two levels), reps >= 1, and sigma must be set");
        return GBP_BAD_ARG;
    }
    if (which >= 8 && !(use_tma && vsweep32_transfer_supported(L[0].g, L[1].g))) {
        set_error("time_kernel: the fused transfer sweeps (8, 9) do not apply to this level");
        return GBP_BAD_ARG;
    }
    const NodalLevel& l0 = L[0];
    const NodalGeom& g = l0.g;
    const bool f32 = (which & 1) || which >= 4;
    const double w = f32 ? 4.0 : 8.0;
    const double nn = (double)g.nu[0] * g.nu[1] * g.nu[2];
    const double nc = (double)g.n[0] * g.n[1] * g.n[2];
    // Jacobi: x, b read + x written per node, sigma read per cell; residual: x, b read, r written;
    // triad (which 4): three padded arrays read, one written
    *bytes = which == 4 ? 4.0 * 4.0 * (double)g.count : w * (3.0 * nn + nc);
    // prolongation (which 6): fine x read and written, coarse x read; restriction (7): fine r read,
    // coarse b written
    if (which == 6) *bytes = 4.0 * (2.0 * nn + nn / 8.0);
    if (which == 7) *bytes = 4.0 * (nn + nn / 8.0);
    // fused residual + restriction (8): x, b read per node, sigma per cell, coarse b written; fused
    // prolongation + Jacobi (9): x, b read and the result written per node, sigma per cell, coarse x read
    if (which == 8) *bytes = 4.0 * (2.0 * nn + nc + nn / 8.0);
    if (which == 9) *bytes = 4.0 * (3.0 * nn + nc + nn / 8.0);
    if (f32) nodal_to_f32(g, res, l0.b32, scale32, st);
    GBP_CUDA(cudaEventRecord(ev0, st));
    for (int r = 0; r < reps; ++r) {
        switch (which) {
        case 0: jacobi<double>(g, l0.s64, (r & 1) ? l0.t64 : l0.x64, res, (r & 1) ? l0.x64 : l0.t64, omega_eff, st); break;
        case 1: jacobi<float>(g, l0.s32, (r & 1) ? l0.t32 : l0.x32, l0.b32, (r & 1) ? l0.x32 : l0.t32, omega_eff, st);
                break;
        case 2: resid<double>(g, l0.s64, phi, rhs0, l0.r64, nullptr, st); break;
        case 3: resid<float>(g, l0.s32, l0.x32, l0.b32, l0.r32, nullptr, st); break;
        case 4: stream_triad(l0.x32, l0.s32, l0.b32, l0.r32, g.count, st); break;
        case 6: nodal_prolong_add<float>(g, L[1].g, L[1].x32, l0.x32, st); break;
        case 7: nodal_restrict<float>(g, L[1].g, l0.r32, L[1].b32, st); break;
        case 8: {
            int rc = vsweep32_resid_restrict(g, L[1].g, l0.s32, l0.x32, l0.b32, L[1].b32, derr, st);
            if (rc) return rc;
            break;
        }
        case 9: {
            int rc = vsweep32_prolong_jacobi(g, L[1].g, l0.s32, l0.x32, L[1].x32, l0.b32, l0.t32, (float)omega_eff,
                                             derr, st);
            if (rc) return rc;
            break;
        }
        default:
            nodal_jacobi<float>(g, l0.s32, (r & 1) ? l0.t32 : l0.x32, l0.b32, (r & 1) ? l0.x32 : l0.t32, omega_eff,
                                false, st);
            break;
        }
    }
    GBP_CUDA(cudaEventRecord(ev1, st));
    GBP_CUDA(cudaEventSynchronize(ev1));
    float t = 0.f;
    GBP_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
    *ms = t / reps;
    return GBP_OK;
}

int NodalSolver::divergence(const RhsArgs& rhs, const gbp_array4* out, double* max_norm)
{
    const NodalLevel& l0 = L[0];
    GBP_CUDA(cudaMemsetAsync(dnorm, 0, sizeof(unsigned long long), st));
    RhsArgs ra = rhs;
    if (eb.on) ra.cmask = eb.e.reg;
    nodal_rhs(l0.g, ra, l0.s64, rhs0, singular ? partials : nullptr, st);
    if (eb.on) eb_rhs(l0.g, eb.e, ra, rhs0, st);
    if (singular)
        nodal_remove_mean(l0.g, rhs0, partials, dscal, 0, (eb.on && eb.e.inflow) ? 0 : 1, nodal_rhs_partials(l0.g),
                          dnorm, st);
    else
        nodal_norm(l0.g, rhs0, dnorm, st);
    if (out && out->data) nodal_store_div(l0.g, *out, rhs0, st);
    GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    GBP_CUDA(cudaGetLastError());
    if (max_norm) *max_norm = bits_to_double(hnorm[0]);
    return GBP_OK;
}

}  // namespace gbp

namespace gbp {

namespace {

__global__ void k_maxdiff(const float* __restrict__ a, const float* __restrict__ ref, long long n,
                          unsigned long long* out)
{
    double d = 0.0, m = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        d = nanmax(d, fabs((double)a[p] - (double)ref[p]));
        m = nanmax(m, fabs((double)ref[p]));
    }
    d = block_max(d);
    __syncthreads();
    m = block_max(m);
    if (threadIdx.x == 0) {
        atomic_max_nonneg(out, d);
        atomic_max_nonneg(out + 1, m);
    }
}

// seeded values in [-1, 1) on the unique nodes (with their periodic aliases when `aliases`)
__global__ void k_fill_seeded(NodalGeom g, float* __restrict__ a, unsigned seed, int aliases)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= g.nu[0]) return;
    unsigned h = (unsigned)(i + 7919 * j + 104729 * k) * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const float v = (float)(h & 0xffffff) * (2.0f / 16777216.0f) - 1.0f;
    if (aliases)
        store_node(a, g, i, j, k, v);
    else
        a[pidx(g.sy, g.sz, i, j, k)] = v;
}

}  // namespace

int NodalSolver::check_level_kernels(double diff[4])
{
    if (L.size() < 3 || !sigma_ready || !vsweep32_supported(L[0].g)) {
        set_error("check_level_kernels: needs a level that the whole-row FP32 sweeps handle, and sigma");
        return GBP_BAD_ARG;
    }
    const NodalLevel& l0 = L[0];
    const NodalLevel& l1 = L[1];
    const NodalGeom& g = l0.g;
    // scratch of its own (a test hook may allocate): the plan's FP64 arrays must keep their zero padding
    float *A = nullptr, *C = nullptr;
    GBP_CUDA(cudaMalloc(&A, sizeof(float) * g.count));
    if (cudaMalloc(&C, sizeof(float) * g.count) != cudaSuccess) {
        cudaFree(A);
        set_error("check_level_kernels: cudaMalloc failed");
        return GBP_CUDA_ERROR;
    }
    int rc = check_level_kernels_on(A, C, diff);
    cudaStreamSynchronize(st);
    cudaFree(A);
    cudaFree(C);
    // leave the FP32 level arrays as a fresh plan has them (the next solve refills what it reads)
    const size_t f0 = sizeof(float) * g.count, f1 = sizeof(float) * l1.g.count;
    for (float* p : {l0.x32, l0.t32, l0.b32, l0.r32}) GBP_CUDA(cudaMemsetAsync(p, 0, f0, st));
    for (float* p : {l1.x32, l1.b32, l1.r32}) GBP_CUDA(cudaMemsetAsync(p, 0, f1, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    return rc;
}

int NodalSolver::check_level_kernels_on(float* A, float* C, double diff[4])
{
    const NodalLevel& l0 = L[0];
    const NodalLevel& l1 = L[1];
    const NodalGeom& g = l0.g;
    unsigned long long* dm = reinterpret_cast<unsigned long long*>(dscal + 4);
    auto compare = [&](const float* a, const float* ref, long long n, double* out) -> int {
        GBP_CUDA(cudaMemsetAsync(dm, 0, 2 * sizeof(unsigned long long), st));
        k_maxdiff<<<592, 256, 0, st>>>(a, ref, n, dm);
        unsigned long long h[2];
        GBP_CUDA(cudaMemcpyAsync(h, dm, sizeof(h), cudaMemcpyDeviceToHost, st));
        GBP_CUDA(cudaStreamSynchronize(st));
        double d, m;
        memcpy(&d, &h[0], 8);
        memcpy(&m, &h[1], 8);
        *out = m > 0 ? d / m : d;
        return GBP_OK;
    };
    const size_t f0 = sizeof(float) * g.count, f1 = sizeof(float) * l1.g.count;
    int rc = GBP_OK;
    GBP_CUDA(cudaMemsetAsync(derr, 0, sizeof(unsigned), st));
    // seeded inputs, so that residuals are of the size of their terms: x and the coarse correction
    // with their periodic aliases (as the level sweeps write them), b on the unique nodes only
    GBP_CUDA(cudaMemsetAsync(l0.x32, 0, f0, st));
    GBP_CUDA(cudaMemsetAsync(l0.b32, 0, f0, st));
    GBP_CUDA(cudaMemsetAsync(l1.x32, 0, f1, st));
    k_fill_seeded<<<dim3((g.nu[0] + 127) / 128, g.nu[1], g.nu[2]), 128, 0, st>>>(g, l0.x32, 17u, 1);
    k_fill_seeded<<<dim3((g.nu[0] + 127) / 128, g.nu[1], g.nu[2]), 128, 0, st>>>(g, l0.b32, 29u, 0);
    k_fill_seeded<<<dim3((l1.g.nu[0] + 127) / 128, l1.g.nu[1], l1.g.nu[2]), 128, 0, st>>>(l1.g, l1.x32, 41u, 1);
    // [0] Jacobi
    GBP_CUDA(cudaMemsetAsync(l0.t32, 0, f0, st));
    GBP_CUDA(cudaMemsetAsync(A, 0, f0, st));
    nodal_jacobi<float>(g, l0.s32, l0.x32, l0.b32, l0.t32, omega_eff, false, st);
    rc = vsweep32(g, 0, l0.s32, l0.x32, l0.b32, A, (float)omega_eff, derr, st);
    if (!rc) rc = compare(A, l0.t32, g.count, &diff[0]);
    // [1] residual
    if (!rc) {
        GBP_CUDA(cudaMemsetAsync(l0.r32, 0, f0, st));
        GBP_CUDA(cudaMemsetAsync(A, 0, f0, st));
        nodal_resid<float>(g, l0.s32, l0.x32, l0.b32, l0.r32, nullptr, st);
        rc = vsweep32(g, 1, l0.s32, l0.x32, l0.b32, A, 0.f, derr, st);
    }
    if (!rc) rc = compare(A, l0.r32, g.count, &diff[1]);
    // [2] residual + restriction (l0.r32 holds the reference residual); [2] and [3] are -1 where the
    // fused transfers do not run (an overset mask)
    diff[2] = diff[3] = -1.0;
    if (!vsweep32_transfer_supported(g, l1.g)) return rc;
    if (!rc) {
        GBP_CUDA(cudaMemsetAsync(l1.b32, 0, f1, st));
        GBP_CUDA(cudaMemsetAsync(l1.r32, 0, f1, st));
        nodal_restrict<float>(g, l1.g, l0.r32, l1.b32, st);
        rc = vsweep32_resid_restrict(g, l1.g, l0.s32, l0.x32, l0.b32, l1.r32, derr, st);
    }
    if (!rc) rc = compare(l1.r32, l1.b32, l1.g.count, &diff[2]);
    // [3] prolongation + Jacobi: reference x' = x + P e in C, then a Jacobi sweep
    if (!rc) {
        GBP_CUDA(cudaMemcpyAsync(C, l0.x32, f0, cudaMemcpyDeviceToDevice, st));
        nodal_prolong_add<float>(g, l1.g, l1.x32, C, st);
        GBP_CUDA(cudaMemsetAsync(l0.t32, 0, f0, st));
        GBP_CUDA(cudaMemsetAsync(A, 0, f0, st));
        nodal_jacobi<float>(g, l0.s32, C, l0.b32, l0.t32, omega_eff, false, st);
        rc = vsweep32_prolong_jacobi(g, l1.g, l0.s32, l0.x32, l1.x32, l0.b32, A, (float)omega_eff, derr, st);
    }
    if (!rc) rc = compare(A, l0.t32, g.count, &diff[3]);
    if (rc) return rc;
    unsigned herr = 0;
    GBP_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    GBP_CUDA(cudaGetLastError());
    if (herr) {
        set_error("check_level_kernels: a bounded device wait ran out");
        return GBP_TIMEOUT;
    }
    return GBP_OK;
}

int NodalSolver::check_coarse_cycle(double* diff)
{
    const int lc = coarse_first();
    if (lc < 1 || !sigma_ready) {
        set_error("check_coarse_cycle: the plan has no cluster-cycled levels (levels " + std::to_string(L.size()) +
                  ", dense bottom " + std::to_string((int)dense_bottom) + " of " + std::to_string(nbottom) +
                  " nodes, cluster path " + std::to_string((int)use_coarse) + ") or no sigma (" +
                  std::to_string((int)sigma_ready) + ")");
        return GBP_BAD_ARG;
    }
    const NodalLevel& v = L[lc];
    const NodalGeom& g = v.g;
    const size_t bytes = sizeof(float) * g.count;
    float* C = nullptr;
    GBP_CUDA(cudaMalloc(&C, bytes));
    cap_or_st = st;
    // the same seeded right-hand side through the per-level launches and through the cluster kernel
    GBP_CUDA(cudaMemsetAsync(v.b32, 0, bytes, st));
    k_fill_seeded<<<dim3((g.nu[0] + 127) / 128, g.nu[1], g.nu[2]), 128, 0, st>>>(g, v.b32, 53u, 0);
    use_coarse = false;
    vcycle<float>(lc, v.b32, true);
    cudaMemcpyAsync(C, xres[lc], bytes, cudaMemcpyDeviceToDevice, st);
    use_coarse = true;
    vcycle<float>(lc, v.b32, true);
    unsigned long long* dm = reinterpret_cast<unsigned long long*>(dscal + 4);
    cudaMemsetAsync(dm, 0, 2 * sizeof(unsigned long long), st);
    k_maxdiff<<<592, 256, 0, st>>>((const float*)xres[lc], C, (long long)g.count, dm);
    unsigned long long h[2] = {0, 0};
    cudaMemcpyAsync(h, dm, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(C);
    const int rc = launch_rc;
    launch_rc = 0;
    if (e != cudaSuccess) return cuda_fail(e, "check_coarse_cycle");
    if (rc) return rc;
    double d, m;
    memcpy(&d, &h[0], 8);
    memcpy(&m, &h[1], 8);
    *diff = m > 0 ? d / m : d;
    return GBP_OK;
}

}  // namespace gbp
