// MAC multigrid driver (host side): the same residual-correction / iterative-refinement loop as
// the nodal driver, on the cell-centred 7-point operator with red-black Gauss-Seidel smoothing.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <unordered_map>
#include <vector>

#include "mac_solver.h"

namespace gbp {

static CellGeom make_cgeom(const int n[3], const double h[3], const int per[3], const int dlo[3], const int dhi[3])
{
    CellGeom g;
    memset(&g, 0, sizeof(g));
    for (int d = 0; d < 3; ++d) {
        g.n[d] = n[d];
        g.per[d] = per[d];
        g.dlo[d] = per[d] ? 0 : dlo[d];
        g.dhi[d] = per[d] ? 0 : dhi[d];
        g.h[d] = h[d];
        g.ih[d] = 1.0 / h[d];
    }
    const long long P0 = padded_row(n[0]);
    g.sy = P0;
    g.sz = P0 * (long long)(n[1] + 2);
    g.count = g.sz * (long long)(n[2] + 2);
    g.vol = h[0] * h[1] * h[2];
    for (int d = 0; d < 3; ++d) g.w[d] = g.vol / (h[d] * h[d]);
    return g;
}

void MacSolver::destroy()
{
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    if (hnorm) cudaFreeHost(hnorm);
    hnorm = nullptr;
    if (cap) cudaStreamDestroy(cap);
    cap = nullptr;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev2) cudaEventDestroy(ev2);
    ev0 = ev1 = ev2 = nullptr;
    pool.release();
    apool.release();
    dpool.release();
    dmat = nullptr;
    dact = nullptr;
    dense_bottom = false;
    abec = false;
    eb.pool.release();
    eb = EbState{};
    L.clear();
    beta_ready = false;
}

int MacSolver::set_options(const gbp_options& o)
{
    if (o.nu1 < 0 || o.nu2 < 0 || o.nu1 + o.nu2 < 1 || o.ir_inner_cycles < 1 || o.maxiter < 0) {
        set_error("mac options: need nu1+nu2 >= 1, ir_inner_cycles >= 1, maxiter >= 0");
        return GBP_BAD_ARG;
    }
    const int maxc = opt.max_coarsening_level;
    opt = o;
    opt.max_coarsening_level = maxc;
    if (gexec) {
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    return GBP_OK;
}

int MacSolver::init(const gbp_geometry& geom, const int bc_lo[3], const int bc_hi[3], const gbp_options& o,
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
        bclo[d] = bc_lo[d];
        bchi[d] = bc_hi[d];
        if (n[d] < 2) {
            set_error("mac plan: every direction needs at least 2 cells");
            return GBP_BAD_ARG;
        }
        h[d] = (geom.prob_hi[d] - geom.prob_lo[d]) / n[d];
        if (!(h[d] > 0.0)) {
            set_error("mac plan: prob_hi must exceed prob_lo");
            return GBP_BAD_ARG;
        }
        if ((bc_lo[d] == GBP_BC_PERIODIC) != (bc_hi[d] == GBP_BC_PERIODIC)) {
            set_error("mac plan: a periodic direction must be periodic on both sides");
            return GBP_BAD_ARG;
        }
        for (int s = 0; s < 2; ++s) {
            int b = s ? bc_hi[d] : bc_lo[d];
            if (b < GBP_BC_PERIODIC || b > GBP_BC_ROBIN) {
                set_error("mac plan: unknown boundary type");
                return GBP_BAD_ARG;
            }
        }
        per[d] = bc_lo[d] == GBP_BC_PERIODIC;
        if (per[d] && (n[d] & 1)) {
            set_error("mac plan: a periodic direction needs an even cell count (red-black ordering)");
            return GBP_BAD_ARG;
        }
        dlo[d] = bc_lo[d] == GBP_BC_DIRICHLET;
        dhi[d] = bc_hi[d] == GBP_BC_DIRICHLET;
        if (dlo[d] || dhi[d]) singular = false;
    }
    any_dirichlet = !singular;
    robin_ready = true;
    for (int d = 0; d < 3; ++d)
        if (bc_lo[d] == GBP_BC_ROBIN || bc_hi[d] == GBP_BC_ROBIN) robin_ready = false;
    int rc = set_options(o);
    if (rc) return rc;
    opt.max_coarsening_level = o.max_coarsening_level;
    L.clear();
    int cn[3] = {n[0], n[1], n[2]};
    double ch[3] = {h[0], h[1], h[2]};
    for (;;) {
        MacLevel lv;
        lv.g = make_cgeom(cn, ch, per, dlo, dhi);
        L.push_back(lv);
        bool ok = (int)L.size() <= opt.max_coarsening_level && (int)L.size() < kMaxLevels;
        for (int d = 0; d < 3; ++d) ok = ok && (cn[d] % 2 == 0) && (cn[d] / 2 >= 2);
        if (!ok) break;
        for (int d = 0; d < 3; ++d) {
            cn[d] /= 2;
            ch[d] *= 2.0;
        }
    }
    const MacLevel& B = L.back();
    if ((long long)B.g.n[0] * B.g.n[1] * B.g.n[2] > 200000) {
        set_error("mac plan: the coarsest level is too large for the single-CTA bottom solver");
        return GBP_BAD_ARG;
    }
    size_t need = 0;
    auto add = [&](size_t cnt, size_t sz) { need = ((need + 255) & ~size_t(255)) + cnt * sz; };
    for (auto& lv : L) {
        for (int q = 0; q < 6; ++q) add(lv.g.count, 8);
        for (int q = 0; q < 6; ++q) add(lv.g.count, 4);
    }
    const CellGeom& G0 = L[0].g;
    for (int q = 0; q < 3; ++q) add(G0.count, 8);
    add(mac_partials_needed(G0) + 64, 8);
    add(5 * B.g.count, 8);
    add(8, 8);
    add(8, 4);
    for (int q = 0; q < 6; ++q) {
        const int d = q >> 1, d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
        if ((q & 1 ? bc_hi[d] : bc_lo[d]) == GBP_BC_ROBIN) {
            add((size_t)n[d1] * n[d2], 8);
            add((size_t)n[d1] * n[d2], 8);
        }
    }
    need += 4096;
    rc = pool.reserve(need);
    if (rc) return rc;
    for (auto& lv : L) {
        for (int d = 0; d < 3; ++d) lv.b64[d] = pool.take<double>(lv.g.count);
        lv.x64 = pool.take<double>(lv.g.count);
        lv.rhs64 = pool.take<double>(lv.g.count);
        lv.r64 = pool.take<double>(lv.g.count);
        for (int d = 0; d < 3; ++d) lv.b32[d] = pool.take<float>(lv.g.count);
        lv.x32 = pool.take<float>(lv.g.count);
        lv.rhs32 = pool.take<float>(lv.g.count);
        lv.r32 = pool.take<float>(lv.g.count);
    }
    phi = pool.take<double>(G0.count);
    rhs0 = pool.take<double>(G0.count);
    res = pool.take<double>(G0.count);
    partials = pool.take<double>(mac_partials_needed(G0) + 64);
    bscr = pool.take<double>(5 * B.g.count);
    dnorm = pool.take<unsigned long long>(8);
    dflags = pool.take<unsigned>(8);
    rb = RobinFaces{};
    for (int q = 0; q < 6; ++q) {
        const int d = q >> 1, d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
        if ((q & 1 ? bc_hi[d] : bc_lo[d]) == GBP_BC_ROBIN) {
            rb.rfac[q] = pool.take<double>((size_t)n[d1] * n[d2]);
            rb.braw[q] = pool.take<double>((size_t)n[d1] * n[d2]);
        }
    }
    GBP_CUDA(cudaMallocHost(&hnorm, 8 * sizeof(unsigned long long)));
    memset(hnorm, 0, 8 * sizeof(unsigned long long));
    GBP_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    GBP_CUDA(cudaEventCreate(&ev0));
    GBP_CUDA(cudaEventCreate(&ev1));
    GBP_CUDA(cudaEventCreate(&ev2));
    return GBP_OK;
}

int MacSolver::set_beta(int source, const gbp_array4* src[3], double cval)
{
    for (int d = 0; d < 3; ++d) {
        const gbp_array4* s = source == 0 ? src[d] : (source == 2 ? src[0] : nullptr);
        mac_set_beta(L[0].g, d, source, s, cval, bclo[d], bchi[d], L[0].b64[d], L[0].b32[d], st, &rb,
                     eb.on ? eb.m.ap[d] : nullptr);
    }
    for (size_t l = 1; l < L.size(); ++l)
        for (int d = 0; d < 3; ++d)
            mac_coarsen_beta(L[l - 1].g, L[l].g, d, L[l - 1].b64[d], L[l].b64[d], L[l].b32[d], st);
    eb_refresh_beta();
    GBP_CUDA(cudaGetLastError());
    beta_ready = true;
    return build_dense_bottom();
}

int MacSolver::set_abec(double alpha, const gbp_array4* a, double a0, double beta, const gbp_array4* const b[3],
                        double b0, const gbp_array4* eta_cc, const double* bscale)
{
    if (eb.on) {
        set_error("abec: cut cells are not supported by the ABecLaplacian form");
        return GBP_BAD_ARG;
    }
    for (int d = 0; d < 3; ++d)
        if (bclo[d] == GBP_BC_ROBIN || bchi[d] == GBP_BC_ROBIN) {
            set_error("abec: Robin sides are not supported by the ABecLaplacian form");
            return GBP_BAD_ARG;
        }
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    if (alpha != 0.0) {
        if (!apool.base) {
            size_t need = 0;
            for (auto& lv : L) need += ((lv.g.count * 12 + 255) & ~size_t(255)) + 512;
            int rc = apool.reserve(need + 4096);
            if (rc) return rc;
            for (auto& lv : L) {
                double* p64 = apool.take<double>(lv.g.count);
                float* p32 = apool.take<float>(lv.g.count);
                GBP_CUDA(cudaMemsetAsync(p64, 0, sizeof(double) * lv.g.count, st));
                GBP_CUDA(cudaMemsetAsync(p32, 0, sizeof(float) * lv.g.count, st));
                lv.g.a64 = p64;
                lv.g.a32 = p32;
            }
        }
        abec_acoef(L[0].g, a, alpha, a0, const_cast<double*>(L[0].g.a64), const_cast<float*>(L[0].g.a32), st);
        for (size_t l = 1; l < L.size(); ++l)
            abec_acoarsen(L[l - 1].g, L[l].g, L[l - 1].g.a64, const_cast<double*>(L[l].g.a64),
                          const_cast<float*>(L[l].g.a32), st);
        abec = true;
    } else {
        for (auto& lv : L) {
            lv.g.a64 = nullptr;
            lv.g.a32 = nullptr;
        }
        apool.release();
        abec = false;
    }
    // face coefficients beta b (b arrays or the constant b0)
    const bool arrays = b && b[0];
    for (int d = 0; d < 3; ++d) {
        const double f = bscale ? bscale[d] : 1.0;
        if (eta_cc)
            mac_set_beta(L[0].g, d, 3, eta_cc, 0.0, bclo[d], bchi[d], L[0].b64[d], L[0].b32[d], st, &rb, nullptr,
                         beta * f);
        else
            mac_set_beta(L[0].g, d, arrays ? 0 : 1, arrays ? b[d] : nullptr, arrays ? 0.0 : beta * b0 * f, bclo[d],
                         bchi[d], L[0].b64[d], L[0].b32[d], st, &rb, nullptr, arrays ? beta * f : 1.0);
    }
    for (size_t l = 1; l < L.size(); ++l)
        for (int d = 0; d < 3; ++d)
            mac_coarsen_beta(L[l - 1].g, L[l].g, d, L[l - 1].b64[d], L[l].b64[d], L[l].b32[d], st);
    GBP_CUDA(cudaGetLastError());
    beta_ready = true;
    singular = !any_dirichlet && !abec;
    return build_dense_bottom();
}

int MacSolver::abec_solve(const gbp_array4* rhs, gbp_array4* phi_io, gbp_stats* stats)
{
    if (!beta_ready) {
        set_error("abec solve: coefficients were never set on this plan");
        return GBP_BAD_ARG;
    }
    const MacLevel& l0 = L[0];
    GBP_CUDA(cudaEventRecord(ev0, st));
    abec_rhs(l0.g, *rhs, rhs0, st);
    for (int d = 0; d < 3; ++d) {
        if (bclo[d] == GBP_BC_DIRICHLET) abec_dirichlet(l0.g, d, 0, l0.b64[d], *phi_io, rhs0, st);
        if (bchi[d] == GBP_BC_DIRICHLET) abec_dirichlet(l0.g, d, 1, l0.b64[d], *phi_io, rhs0, st);
    }
    if (singular) mac_remove_mean(l0.g, rhs0, partials, 0, st);
    GBP_CUDA(cudaMemsetAsync(phi, 0, sizeof(double) * l0.g.count, st));
    mac_load_phi(l0.g, *phi_io, phi, st);
    GBP_CUDA(cudaGetLastError());
    int status = solve(true, stats);
    if (status != GBP_OK && status != GBP_NOT_CONVERGED) return status;
    mac_store_phi(l0.g, *phi_io, phi, st);
    GBP_CUDA(cudaEventRecord(ev2, st));
    GBP_CUDA(cudaGetLastError());
    if (stats) {
        GBP_CUDA(cudaEventSynchronize(ev2));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev2);
        stats->ms_total = ms;
    }
    return status;
}

// Dense inverse of the coarsest level's operator, assembled on the host from its face coefficients
// (boundary factors included: 0 on walls, doubled on Dirichlet faces) and alpha a V: the same matrix the
// smoother and the CG see. Cells whose row is empty (covered by an embedded boundary) carry no
// equation and stay 0; a singular system is regularised with c 1 1^T over the other cells.
int MacSolver::build_dense_bottom()
{
    const MacLevel& B = L.back();
    const CellGeom& g = B.g;
    const int N = g.n[0] * g.n[1] * g.n[2];
    const bool was = dense_bottom;
    dense_bottom = false;
    // (a one-level hierarchy with cut cells has terms outside the face coefficients: keep the CG)
    if (N > kMacDenseBottomMax || (L.size() == 1 && eb.on)) {
        if (was && gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        return GBP_OK;
    }
    if (!dmat) {
        int rc = dpool.reserve(sizeof(double) * (size_t)N * N + (size_t)N + 1024);
        if (rc) return rc;
        dmat = dpool.take<double>((size_t)N * N);
        dact = dpool.take<unsigned char>((size_t)N);
    }
    std::vector<double> bf[3], av;
    for (int d = 0; d < 3; ++d) {
        bf[d].resize((size_t)g.count);
        GBP_CUDA(cudaMemcpyAsync(bf[d].data(), B.b64[d], sizeof(double) * g.count, cudaMemcpyDeviceToHost, st));
    }
    if (g.a64) {
        av.resize((size_t)g.count);
        GBP_CUDA(cudaMemcpyAsync(av.data(), g.a64, sizeof(double) * g.count, cudaMemcpyDeviceToHost, st));
    }
    GBP_CUDA(cudaStreamSynchronize(st));
    auto cid = [&](int i, int j, int k) { return i + g.n[0] * (j + g.n[1] * k); };
    std::vector<double> A((size_t)N * N, 0.0);
    const long long sd[3] = {1, g.sy, g.sz};
    for (int k = 0; k < g.n[2]; ++k)
        for (int j = 0; j < g.n[1]; ++j)
            for (int i = 0; i < g.n[0]; ++i) {
                const int c = cid(i, j, k);
                const long long p = pidx(g.sy, g.sz, i, j, k);
                double diag = av.empty() ? 0.0 : av[(size_t)p];
                const int ijk[3] = {i, j, k};
                for (int d = 0; d < 3; ++d)
                    for (int side = 0; side < 2; ++side) {
                        const double coef = g.w[d] * bf[d][(size_t)(side ? p + sd[d] : p)];
                        diag += coef;
                        int nb[3] = {ijk[0], ijk[1], ijk[2]};
                        nb[d] += side ? 1 : -1;
                        if (nb[d] < 0 || nb[d] >= g.n[d]) {
                            if (!g.per[d]) continue;  // ghost value 0 (Dirichlet) or no flux
                            nb[d] = (nb[d] + g.n[d]) % g.n[d];
                        }
                        A[(size_t)c * N + cid(nb[0], nb[1], nb[2])] -= coef;
                    }
                A[(size_t)c * N + c] += diag;
            }
    std::vector<unsigned char> act((size_t)N);
    int na = 0;
    double tr = 0.0;
    for (int c = 0; c < N; ++c) {
        act[(size_t)c] = A[(size_t)c * N + c] != 0.0;
        na += act[(size_t)c];
        tr += A[(size_t)c * N + c];
    }
    if (singular && na > 0) {
        const double cr = tr / ((double)na * na);
        for (int u = 0; u < N; ++u)
            for (int v = 0; v < N; ++v)
                if (act[(size_t)u] && act[(size_t)v]) A[(size_t)u * N + v] += cr;
    }
    for (int c = 0; c < N; ++c)
        if (!act[(size_t)c]) A[(size_t)c * N + c] = 1.0;
    // Gauss-Jordan inverse with partial pivoting
    std::vector<double> M((size_t)N * N, 0.0);
    for (int u = 0; u < N; ++u) M[(size_t)u * N + u] = 1.0;
    for (int col = 0; col < N; ++col) {
        int piv = col;
        for (int r = col + 1; r < N; ++r)
            if (fabs(A[(size_t)r * N + col]) > fabs(A[(size_t)piv * N + col])) piv = r;
        if (A[(size_t)piv * N + col] == 0.0) {  // not invertible: keep the CG bottom
            if (was && gexec) {
                cudaGraphExecDestroy(gexec);
                gexec = nullptr;
            }
            return GBP_OK;
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
    for (int u = 0; u < N; ++u)
        if (!act[(size_t)u])
            for (int q = 0; q < N; ++q) M[(size_t)u * N + q] = M[(size_t)q * N + u] = 0.0;
    std::vector<double> Mt((size_t)N * N);
    for (int u = 0; u < N; ++u)
        for (int v = 0; v < N; ++v) Mt[(size_t)v * N + u] = M[(size_t)u * N + v];
    GBP_CUDA(cudaMemcpyAsync(dmat, Mt.data(), sizeof(double) * Mt.size(), cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaMemcpyAsync(dact, act.data(), (size_t)N, cudaMemcpyHostToDevice, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    dense_bottom = true;
    if (!was && gexec) {  // a captured step holds the other bottom kernel
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    return GBP_OK;
}

void MacSolver::add_vcycle_correction(const double* r, double* e, double sc)
{
    const MacLevel& l0 = L[0];
    cap_or_st = st;
    if (opt.precision == GBP_PREC_MIXED) {
        mac_to_f32(l0.g, r, l0.rhs32, sc, st);
        vcycle<float>(0, l0.rhs32, true);
        for (int c = 1; c < opt.ir_inner_cycles; ++c) vcycle<float>(0, l0.rhs32, false);
        mac_add_correction<float>(l0.g, e, l0.x32, 1.0 / sc, st);
    } else {
        vcycle<double>(0, r, true);
        for (int c = 1; c < opt.ir_inner_cycles; ++c) vcycle<double>(0, r, false);
        mac_add_correction<double>(l0.g, e, l0.x64, 1.0, st);
    }
}

void MacSolver::vcycles32(const float* b32)
{
    cap_or_st = st;
    vcycle<float>(0, b32, true);
    for (int c = 1; c < opt.ir_inner_cycles; ++c) vcycle<float>(0, b32, false);
}

void MacSolver::eb_refresh_beta()
{
    if (!eb.on) return;
    const double* b[3] = {L[0].b64[0], L[0].b64[1], L[0].b64[2]};
    const double* a[3] = {eb.m.ap[0], eb.m.ap[1], eb.m.ap[2]};
    eb_table_beta(eb.faces, eb.nfaces, b, a, eb.cb64, eb.cb32, st);
}

// Cut-face table of the finest level. For a cut face (0 < ap < 1) off the non-periodic domain sides,
// the normal derivative at its centroid is the bilinear blend of the face-centre differences of the face
// and of its neighbours f1, f2, f12 one cell towards the centroid in the two tangential directions
// (weights |offset|); a neighbour enters only if open, the corner only with both f1 and f2 (else the
// second weight drops). This is the face-centroid gradient of the cut-cell finite-volume method that
// AMReX's MLEBABecLap uses for the MAC projection (Location::FaceCentroid, src/incflo.cpp:286-292).
int MacSolver::set_eb(const gbp_array4* vfrac, const gbp_array4* const area[3], const gbp_array4* const fcent[3])
{
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    beta_ready = false;
    GBP_CUDA(cudaStreamSynchronize(st));
    eb.pool.release();
    eb = EbState{};
    if (!vfrac) return GBP_OK;
    for (int d = 0; d < 3; ++d)
        if (!area || !fcent || !area[d] || !fcent[d] || !area[d]->data || !fcent[d]->data || fcent[d]->ncomp < 2) {
            set_error("mac_set_eb: need the volume fractions, 3 area-fraction arrays and 3 face-centroid arrays "
                      "(2 components)");
            return GBP_BAD_ARG;
        }
    if (!vfrac->data) {
        set_error("mac_set_eb: null volume-fraction data");
        return GBP_BAD_ARG;
    }
    const CellGeom& g = L[0].g;
    const int* n = g.n;
    // every array must cover its index space
    auto covers = [&](const gbp_array4& a, int d) {
        for (int e = 0; e < 3; ++e) {
            const int hi = n[e] - 1 + (e == d ? 1 : 0);
            if (a.lo[e] > 0 || a.hi[e] < hi) return false;
        }
        return true;
    };
    bool ok = covers(*vfrac, -1);
    for (int d = 0; d < 3; ++d) ok = ok && covers(*area[d], d) && covers(*fcent[d], d);
    if (!ok) {
        set_error("mac_set_eb: an EB array does not cover the cells / faces of the level");
        return GBP_BAD_ARG;
    }
    // host copies (dense, x fastest)
    long long fnum[3];
    int fn[3][3];
    for (int d = 0; d < 3; ++d) {
        for (int e = 0; e < 3; ++e) fn[d][e] = n[e] + (e == d ? 1 : 0);
        fnum[d] = (long long)fn[d][0] * fn[d][1] * fn[d][2];
    }
    const long long ncell = (long long)n[0] * n[1] * n[2];
    long long mx = ncell;
    for (int d = 0; d < 3; ++d) mx = std::max(mx, fnum[d]);
    double* tmp = nullptr;
    GBP_CUDA(cudaMalloc(&tmp, sizeof(double) * (size_t)mx));
    std::vector<double> kapH((size_t)ncell), apH[3], fcH[3][2];
    auto fetch = [&](const gbp_array4& a, int d, int c, std::vector<double>& out) -> int {
        const long long cnt = d < 0 ? ncell : fnum[d];
        out.resize((size_t)cnt);
        mac_pack_faces(g, d, a, c, tmp, st);
        cudaError_t e = cudaMemcpyAsync(out.data(), tmp, sizeof(double) * (size_t)cnt, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? GBP_OK : cuda_fail(e, "mac_set_eb: copy of the EB arrays");
    };
    int rc = fetch(*vfrac, -1, 0, kapH);
    for (int d = 0; d < 3 && !rc; ++d) {
        rc = fetch(*area[d], d, 0, apH[d]);
        for (int c = 0; c < 2 && !rc; ++c) rc = fetch(*fcent[d], d, c, fcH[d][c]);
    }
    cudaFree(tmp);
    if (rc) return rc;
    auto cid = [&](int i, int j, int k) { return i + (long long)n[0] * (j + (long long)n[1] * k); };
    auto fid = [&](int d, int i, int j, int k) { return i + (long long)fn[d][0] * (j + (long long)fn[d][1] * k); };
    double ksum = 0.0;
    for (long long c = 0; c < ncell; ++c) {
        const double v = kapH[(size_t)c];
        if (!(v >= 0.0 && v <= 1.0)) {
            set_error("mac_set_eb: volume fractions must lie in [0, 1]");
            return GBP_BAD_ARG;
        }
        ksum += v;
    }
    if (!(ksum > 0.0)) {
        set_error("mac_set_eb: every cell is covered");
        return GBP_BAD_ARG;
    }
    for (int d = 0; d < 3; ++d)
        for (int k = 0; k < fn[d][2]; ++k)
            for (int j = 0; j < fn[d][1]; ++j)
                for (int i = 0; i < fn[d][0]; ++i) {
                    const long long q = fid(d, i, j, k);
                    const double a = apH[d][(size_t)q];
                    const double o0 = fcH[d][0][(size_t)q], o1 = fcH[d][1][(size_t)q];
                    if (!(a >= 0.0 && a <= 1.0) || !(fabs(o0) <= 0.5 + 1e-12) || !(fabs(o1) <= 0.5 + 1e-12)) {
                        set_error("mac_set_eb: area fractions must lie in [0, 1] and centroid offsets in [-0.5, 0.5]");
                        return GBP_BAD_ARG;
                    }
                    if (a > 0.0) {
                        int c[3] = {i, j, k};
                        const int fd = c[d];
                        for (int side = 0; side < 2; ++side) {
                            int cc[3] = {c[0], c[1], c[2]};
                            cc[d] = fd - 1 + side;
                            if (g.per[d]) cc[d] = (cc[d] + n[d]) % n[d];
                            if (cc[d] < 0 || cc[d] >= n[d]) continue;
                            if (!(kapH[(size_t)cid(cc[0], cc[1], cc[2])] > 0.0)) {
                                set_error("mac_set_eb: an open face (area fraction > 0) touches a covered cell");
                                return GBP_BAD_ARG;
                            }
                        }
                    }
                }
    // cut-face table
    std::vector<EbFace> F;
    std::unordered_map<long long, int> cell_of;
    std::vector<EbCell> C;
    const long long sd[3] = {1, g.sy, g.sz};
    auto add_slot = [&](int i, int j, int k, int slot, int e) {
        const long long key = cid(i, j, k);
        auto it = cell_of.find(key);
        int ci;
        if (it == cell_of.end()) {
            EbCell ec;
            ec.p = pidx(g.sy, g.sz, i, j, k);
            for (int s = 0; s < 6; ++s) ec.slot[s] = -1;
            ci = (int)C.size();
            C.push_back(ec);
            cell_of.emplace(key, ci);
        } else {
            ci = it->second;
        }
        C[(size_t)ci].slot[slot] = e;
    };
    for (int d = 0; d < 3; ++d) {
        const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
        for (int k = 0; k < fn[d][2]; ++k)
            for (int j = 0; j < fn[d][1]; ++j)
                for (int i = 0; i < fn[d][0]; ++i) {
                    const long long q = fid(d, i, j, k);
                    const double a = apH[d][(size_t)q];
                    if (!(a > 0.0 && a < 1.0)) continue;
                    int f[3] = {i, j, k};
                    const int fd = f[d];
                    if (!g.per[d] && (fd == 0 || fd == n[d])) continue;  // no blend on domain sides
                    const double o[2] = {fcH[d][0][(size_t)q], fcH[d][1][(size_t)q]};
                    const int s1 = o[0] >= 0.0 ? 1 : -1, s2 = o[1] >= 0.0 ? 1 : -1;
                    auto shift = [&](const int* in, int t, int s, int* out) {
                        for (int e = 0; e < 3; ++e) out[e] = in[e];
                        out[t] += s;
                        if (g.per[t]) out[t] = (out[t] + n[t]) % n[t];
                        return out[t] >= 0 && out[t] < n[t];
                    };
                    auto open = [&](const int* ff) { return apH[d][(size_t)fid(d, ff[0], ff[1], ff[2])] > 0.0; };
                    int f1[3], f2[3], f12[3];
                    const bool h1 = shift(f, t1, s1, f1) && open(f1);
                    const bool h2 = shift(f, t2, s2, f2) && open(f2);
                    double w1 = h1 ? fabs(o[0]) : 0.0, w2 = h2 ? fabs(o[1]) : 0.0;
                    bool h12 = false;
                    if (w1 > 0.0 && w2 > 0.0) {
                        h12 = shift(f1, t2, s2, f12) && open(f12);
                        if (!h12) w2 = 0.0;
                    }
                    if (w1 == 0.0 && w2 == 0.0) continue;
                    EbFace e{};
                    e.d = d;
                    for (int c = 0; c < 3; ++c) e.f[c] = f[c];
                    const double wd = g.w[d], hd = g.h[d];
                    auto put = [&](const int* ff, double wt) {
                        const int m = e.nm++;
                        e.pf[m] = pidx(g.sy, g.sz, ff[0], ff[1], ff[2]);
                        e.coef[m] = a * wd * wt;
                        e.vcoef[m] = wt / hd;
                    };
                    put(f, (1.0 - w1) * (1.0 - w2) - 1.0);
                    if (w1 > 0.0) put(f1, w1 * (1.0 - w2));
                    if (w2 > 0.0) put(f2, (1.0 - w1) * w2);
                    if (w1 > 0.0 && w2 > 0.0) put(f12, w1 * w2);
                    (void)sd;
                    const int ei = (int)F.size();
                    F.push_back(e);
                    // the face is the low face of cell f (if inside) and the high face of cell f - e_d
                    if (fd < n[d]) add_slot(f[0], f[1], f[2], 2 * d, ei);
                    if (fd >= 1) {
                        int c[3] = {f[0], f[1], f[2]};
                        c[d] -= 1;
                        add_slot(c[0], c[1], c[2], 2 * d + 1, ei);
                    }
                }
    }
    // device storage
    size_t need = 0;
    auto add = [&](size_t cnt, size_t sz) { need = ((need + 255) & ~size_t(255)) + cnt * sz; };
    for (int q = 0; q < 6; ++q) add(g.count, 8);
    add(g.count, 4);
    add(F.size() + 1, sizeof(EbFace));
    add(C.size() + 1, sizeof(EbCell));
    add(4 * F.size() + 4, 8);
    add(4 * F.size() + 4, 4);
    need += 4096;
    rc = eb.pool.reserve(need);
    if (rc) return rc;
    eb.m.kap = eb.pool.take<double>(g.count);
    for (int d = 0; d < 3; ++d) eb.m.ap[d] = eb.pool.take<double>(g.count);
    eb.flux = eb.pool.take<double>(g.count);
    eb.beff64 = eb.pool.take<double>(g.count);
    eb.beff32 = eb.pool.take<float>(g.count);
    eb.faces = eb.pool.take<EbFace>(F.size() + 1);
    eb.cells = eb.pool.take<EbCell>(C.size() + 1);
    eb.cb64 = eb.pool.take<double>(4 * F.size() + 4);
    eb.cb32 = eb.pool.take<float>(4 * F.size() + 4);
    eb.nfaces = (int)F.size();
    eb.ncells = (int)C.size();
    eb.kap_sum = ksum;
    if (!F.empty()) GBP_CUDA(cudaMemcpyAsync(eb.faces, F.data(), sizeof(EbFace) * F.size(), cudaMemcpyHostToDevice, st));
    if (!C.empty()) GBP_CUDA(cudaMemcpyAsync(eb.cells, C.data(), sizeof(EbCell) * C.size(), cudaMemcpyHostToDevice, st));
    mac_load_eb(g, *vfrac, area, eb.m, st);
    GBP_CUDA(cudaGetLastError());
    GBP_CUDA(cudaStreamSynchronize(st));  // the host tables go out of scope
    eb.on = true;
    return GBP_OK;
}

int MacSolver::set_eb_inflow(const gbp_array4* eb_vel)
{
    if (!eb_vel) {
        eb.m.ebflux = nullptr;
        return GBP_OK;
    }
    if (!eb.on) {
        set_error("mac_set_eb_inflow: the plan has no embedded boundary (mac_set_eb first)");
        return GBP_BAD_ARG;
    }
    mac_eb_inflow_flux(L[0].g, *eb_vel, eb.m, eb.flux, st);
    GBP_CUDA(cudaGetLastError());
    eb.m.ebflux = eb.flux;
    return GBP_OK;
}

int MacSolver::set_robin(const gbp_array4* a, const gbp_array4* b, const gbp_array4* f)
{
    bool any = false;
    for (int q = 0; q < 6; ++q) any = any || rb.rfac[q];
    if (!any) {
        set_error("mac_set_robin: the plan has no Robin (GBP_BC_ROBIN) side");
        return GBP_BAD_ARG;
    }
    GBP_CUDA(cudaMemsetAsync(dflags, 0, sizeof(unsigned), st));
    for (int q = 0; q < 6; ++q)
        if (rb.rfac[q])
            mac_robin_factors(L[0].g, q >> 1, q & 1, *a, *b, f, const_cast<double*>(rb.rfac[q]), dflags, st);
    unsigned fl = 0;
    GBP_CUDA(cudaMemcpyAsync(&fl, dflags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    if (fl & 2u) {
        set_error("mac_set_robin: Robin data needs a >= 0, b >= 0, a h / 2 + b > 0 and f = 0 on every Robin face");
        robin_ready = false;
        return GBP_BAD_ARG;
    }
    robin_ready = true;
    if (beta_ready) {
        for (int q = 0; q < 6; ++q)
            if (rb.rfac[q]) {
                const int d = q >> 1;
                mac_robin_apply(L[0].g, d, q & 1, rb.braw[q], rb.rfac[q], L[0].b64[d], L[0].b32[d], st,
                                eb.on ? eb.m.ap[d] : nullptr);
            }
        for (size_t l = 1; l < L.size(); ++l)
            for (int d = 0; d < 3; ++d)
                mac_coarsen_beta(L[l - 1].g, L[l].g, d, L[l - 1].b64[d], L[l].b64[d], L[l].b32[d], st);
        eb_refresh_beta();
        GBP_CUDA(cudaGetLastError());
    }
    // a Robin face with a > 0 pins phi like a Dirichlet face
    const bool sing = !(any_dirichlet || (fl & 1u));
    if (sing != singular) {
        singular = sing;
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    return beta_ready ? build_dense_bottom() : GBP_OK;
}

template <typename T>
struct MacBufs;
template <>
struct MacBufs<double> {
    template <typename E>
    static double* beff(const E& e) { return e.beff64; }
    template <typename E>
    static const double* cb(const E& e) { return e.cb64; }
    static double* const* b(const MacLevel& l) { return l.b64; }
    static double* x(const MacLevel& l) { return l.x64; }
    static double* rhs(const MacLevel& l) { return l.rhs64; }
    static double* r(const MacLevel& l) { return l.r64; }
};
template <>
struct MacBufs<float> {
    template <typename E>
    static float* beff(const E& e) { return e.beff32; }
    template <typename E>
    static const float* cb(const E& e) { return e.cb32; }
    static float* const* b(const MacLevel& l) { return l.b32; }
    static float* x(const MacLevel& l) { return l.x32; }
    static float* rhs(const MacLevel& l) { return l.rhs32; }
    static float* r(const MacLevel& l) { return l.r32; }
};

// First level cycled by the cluster kernel: the first level below the finest with at most kCoarseCells
// cells, when the bottom is the dense inverse and the tail fits the kernel's table; -1 otherwise.
int MacSolver::coarse_first() const
{
    if (!dense_bottom || !use_coarse) return -1;
    for (int l = 1; l + 1 < (int)L.size(); ++l) {
        const CellGeom& g = L[l].g;
        if ((long long)g.n[0] * g.n[1] * g.n[2] <= kCoarseCells)
            return ((int)L.size() - l <= kMacCoarseMaxLevels) ? l : -1;
    }
    return -1;
}

template <typename T>
void MacSolver::vcycle(int l, const T* b, bool zero)
{
    using B = MacBufs<T>;
    const MacLevel& lv = L[l];
    const cudaStream_t s = cap_or_st;
    T* x = B::x(lv);
    // the small levels (this one down to the bottom) in one cluster-resident launch
    if (sizeof(T) == 4 && zero && l >= 1 && l == coarse_first()) {
        MacCoarseCycle<T> c{};
        c.nl = (int)L.size() - l;
        for (int q = 0; q < c.nl; ++q) {
            const MacLevel& v = L[l + q];
            c.g[q] = v.g;
            c.bx[q] = B::b(v)[0];
            c.by[q] = B::b(v)[1];
            c.bz[q] = B::b(v)[2];
            c.x[q] = B::x(v);
            c.b[q] = B::rhs(v);
            c.r[q] = B::r(v);
        }
        c.b[0] = const_cast<T*>(b);
        c.M = dmat;
        c.act = dact;
        c.singular = singular ? 1 : 0;
        c.nu1 = opt.nu1;
        c.nu2 = opt.nu2;
        int rc = mac_coarse_vcycle<T>(c, mac_coarse_cluster_size(), s);
        if (rc && !launch_rc) launch_rc = rc;
        return;
    }
    if (l == (int)L.size() - 1) {
        if (dense_bottom)
            mac_bottom_dense<T>(lv.g, dmat, dact, b, x, singular ? 1 : 0, s);
        else
            mac_bottom<T>(lv.g, lv.b64[0], lv.b64[1], lv.b64[2], b, x, bscr, opt.bottom_maxiter, opt.bottom_rtol,
                          opt.bottom_atol, singular ? 1 : 0, s);
        return;
    }
    T* const* be = B::b(lv);
    if (zero) cudaMemsetAsync(x, 0, sizeof(T) * lv.g.count, s);
    // cut cells on the finest level: the smoother sees b minus the cut-face terms of the current x
    // (lagged by one red-black pair), the residual carries them exactly
    const bool cut = l == 0 && eb.on;
    const T* bs = b;
    if (cut) {
        T* beff = B::beff(eb);
        cudaMemcpyAsync(beff, b, sizeof(T) * lv.g.count, cudaMemcpyDeviceToDevice, s);
        bs = beff;
    }
    auto lag = [&]() {
        if (cut) eb_cells<T>(lv.g, eb.cells, eb.ncells, eb.faces, B::cb(eb), x, b, B::beff(eb), s);
    };
    for (int q = 0; q < opt.nu1; ++q) {
        lag();
        mac_rbgs<T>(lv.g, be[0], be[1], be[2], bs, x, 0, s);
        mac_rbgs<T>(lv.g, be[0], be[1], be[2], bs, x, 1, s);
    }
    mac_resid<T>(lv.g, be[0], be[1], be[2], x, b, B::r(lv), nullptr, s);
    if (cut) eb_cells<T>(lv.g, eb.cells, eb.ncells, eb.faces, B::cb(eb), x, B::r(lv), B::r(lv), s);
    const MacLevel& cv = L[l + 1];
    mac_restrict<T>(lv.g, cv.g, B::r(lv), B::rhs(cv), s);
    vcycle<T>(l + 1, B::rhs(cv), true);
    mac_prolong_add<T>(lv.g, cv.g, B::x(cv), x, s);
    for (int q = 0; q < opt.nu2; ++q) {
        lag();
        mac_rbgs<T>(lv.g, be[0], be[1], be[2], bs, x, 1, s);
        mac_rbgs<T>(lv.g, be[0], be[1], be[2], bs, x, 0, s);
    }
}

void MacSolver::resid64(const double* x, const double* b, double* r, unsigned long long* norm, cudaStream_t s)
{
    const MacLevel& l0 = L[0];
    if (!eb.on) {
        mac_resid<double>(l0.g, l0.b64[0], l0.b64[1], l0.b64[2], x, b, r, norm, s);
        return;
    }
    mac_resid<double>(l0.g, l0.b64[0], l0.b64[1], l0.b64[2], x, b, r, nullptr, s);
    eb_cells<double>(l0.g, eb.cells, eb.ncells, eb.faces, eb.cb64, x, r, r, s);
    mac_norm(l0.g, r, norm, s, eb.m.kap);
}

void MacSolver::record_iteration(int m)
{
    const MacLevel& l0 = L[0];
    const cudaStream_t s = cap_or_st;
    if (opt.precision == GBP_PREC_MIXED) {
        mac_to_f32(l0.g, res, l0.rhs32, scale32, s);
        vcycle<float>(0, l0.rhs32, true);
        for (int c = 1; c < m; ++c) vcycle<float>(0, l0.rhs32, false);
        mac_add_correction<float>(l0.g, phi, l0.x32, 1.0 / scale32, s);
    } else {
        vcycle<double>(0, res, true);
        mac_add_correction<double>(l0.g, phi, l0.x64, 1.0, s);
    }
    cudaMemsetAsync(dnorm + 1, 0, sizeof(unsigned long long), s);
    resid64(phi, rhs0, res, dnorm + 1, s);
    cudaMemcpyAsync(hnorm + 1, dnorm + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
}

int MacSolver::run_iteration(int m)
{
    // the captured step holds ir_inner_cycles V-cycles; a shortened last step is launched directly
    launch_rc = 0;
    if (!opt.use_graphs || m != opt.ir_inner_cycles) {
        cap_or_st = st;
        record_iteration(m);
        if (launch_rc) return launch_rc;
        GBP_CUDA(cudaGetLastError());
        return GBP_OK;
    }
    if (!gexec || gexec_prec != opt.precision || gexec_scale != scale32) {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        cudaGraph_t graph = nullptr;
        cap_or_st = cap;
        GBP_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        record_iteration(opt.ir_inner_cycles);
        cudaError_t e = cudaStreamEndCapture(cap, &graph);
        cap_or_st = st;
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(mac refinement step)");
        if (launch_rc) {
            cudaGraphDestroy(graph);
            return launch_rc;
        }
        e = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            gexec = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate(mac refinement step)");
        }
        gexec_prec = opt.precision;
        gexec_scale = scale32;
    }
    GBP_CUDA(cudaGraphLaunch(gexec, st));
    return GBP_OK;
}

static inline double bits_to_double(unsigned long long b)
{
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
}

int MacSolver::solve(bool have_guess, gbp_stats* stats)
{
    const MacLevel& l0 = L[0];
    cap_or_st = st;
    GBP_CUDA(cudaEventRecord(ev1, st));
    if (!have_guess) GBP_CUDA(cudaMemsetAsync(phi, 0, sizeof(double) * l0.g.count, st));
    GBP_CUDA(cudaMemsetAsync(dnorm, 0, 4 * sizeof(unsigned long long), st));
    mac_norm(l0.g, rhs0, dnorm, st, eb.on ? eb.m.kap : nullptr);
    resid64(phi, rhs0, res, dnorm + 1, st);
    GBP_CUDA(cudaMemcpyAsync(hnorm, dnorm, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GBP_CUDA(cudaStreamSynchronize(st));
    const double bnorm = bits_to_double(hnorm[0]);
    double rn = bits_to_double(hnorm[1]);
    if (!isfinite(bnorm) || !isfinite(rn)) {
        set_error("mac solve: right-hand side or initial residual is not finite");
        if (stats) stats->status = GBP_NAN;
        return GBP_NAN;
    }
    const double ref = opt.always_use_bnorm ? bnorm : rn;
    const double target = std::max(opt.rtol * ref, opt.atol);
    if (bnorm > 0.0) {
        int ex = 0;
        frexp(bnorm * l0.g.vol, &ex);
        scale32 = ldexp(1.0, -ex);
    }
    int it = 0, status = GBP_OK, vcycles = 0;
    const double r0 = rn;
    const bool mixed = opt.precision == GBP_PREC_MIXED;
    int m = mixed ? opt.ir_inner_cycles : 1;
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
            // next inner solve: the V-cycles the observed per-cycle contraction says the remaining
            // reduction needs (+1/4 cycle of margin), capped by ir_inner_cycles and by what an FP32
            // inner solve delivers (about 1e-6 of its right-hand side)
            const double rho = std::min(0.9, std::max(1e-3, pow(rn / rprev, 1.0 / m)));
            const double need = log(std::max(target / rn, 1e-6)) / log(rho);
            m = std::max(1, std::min(opt.ir_inner_cycles, (int)ceil(need + 0.25)));
        }
        if (opt.verbose > 1) fprintf(stderr, "gbp mac: iter %d rel resid %.3e\n", it, bnorm > 0 ? rn / bnorm : rn);
        if (!isfinite(rn)) {
            status = GBP_NAN;
            set_error("mac solve: residual became NaN/Inf");
            break;
        }
    }
    if (singular)
        mac_remove_mean(l0.g, phi, partials, 1, st, eb.on ? eb.m.kap : nullptr, eb.kap_sum);
    else if (eb.on)
        eb_zero_covered(l0.g, eb.m.kap, phi, st);
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
        fprintf(stderr, "gbp mac: %s after %d steps, rel resid %.3e\n", status == GBP_OK ? "converged" : "stopped", it,
                bnorm > 0 ? rn / bnorm : rn);
    return status;
}

int MacSolver::get_fluxes(const gbp_array4& phi_in, gbp_array4* flux[3])
{
    if (!beta_ready || !robin_ready) {
        set_error("mac get_fluxes: beta (and Robin data on Robin sides) must be set on the plan");
        return GBP_BAD_ARG;
    }
    const MacLevel& l0 = L[0];
    mac_load_phi(l0.g, phi_in, phi, st);
    // the correction of project() applied to zero face values: 0 - beta grad phi
    for (int d = 0; d < 3; ++d) mac_zero_faces(l0.g, d, *flux[d], st);
    for (int d = 0; d < 3; ++d) mac_correct(l0.g, d, *flux[d], l0.b64[d], phi, st, eb.on ? eb.m.ap[d] : nullptr);
    if (eb.on) {
        const double* b[3] = {l0.b64[0], l0.b64[1], l0.b64[2]};
        const double* a[3] = {eb.m.ap[0], eb.m.ap[1], eb.m.ap[2]};
        eb_correct_u(l0.g, eb.faces, eb.nfaces, b, a, phi, flux, st);
    }
    GBP_CUDA(cudaGetLastError());
    return GBP_OK;
}

int MacSolver::project(gbp_array4* u[3], gbp_array4* phi_io, int phi_guess, gbp_stats* stats)
{
    if (!beta_ready || !robin_ready) {
        set_error(beta_ready ? "mac project: the plan has Robin sides but no Robin data (mac_set_robin)"
                             : "mac project: beta was never set on this plan");
        return GBP_BAD_ARG;
    }
    const MacLevel& l0 = L[0];
    GBP_CUDA(cudaEventRecord(ev0, st));
    mac_rhs(l0.g, *u[0], *u[1], *u[2], rhs0, st, eb.on ? &eb.m : nullptr);
    if (singular) mac_remove_mean(l0.g, rhs0, partials, 0, st, eb.on ? eb.m.kap : nullptr, eb.kap_sum);
    const bool guess = phi_guess && phi_io && phi_io->data;
    if (guess) mac_load_phi(l0.g, *phi_io, phi, st);
    GBP_CUDA(cudaGetLastError());
    int status = solve(guess, stats);
    if (status != GBP_OK && status != GBP_NOT_CONVERGED) return status;
    for (int d = 0; d < 3; ++d) mac_correct(l0.g, d, *u[d], l0.b64[d], phi, st, eb.on ? eb.m.ap[d] : nullptr);
    if (eb.on) {
        const double* b[3] = {l0.b64[0], l0.b64[1], l0.b64[2]};
        const double* a[3] = {eb.m.ap[0], eb.m.ap[1], eb.m.ap[2]};
        eb_correct_u(l0.g, eb.faces, eb.nfaces, b, a, phi, u, st);
    }
    if (phi_io && phi_io->data) mac_store_phi(l0.g, *phi_io, phi, st);
    GBP_CUDA(cudaEventRecord(ev2, st));
    GBP_CUDA(cudaGetLastError());
    if (stats) {
        GBP_CUDA(cudaEventSynchronize(ev2));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev2);
        stats->ms_total = ms;
        // kernels per V-cycle: 2 sweeps (red, black) per smoothing step, residual, restriction and
        // prolongation on every level above the bottom, one bottom solve
        const int cut = eb.on ? 1 : 0;
        // with cut cells the finest level adds one cut-cell pass per smoothing step and one for its residual
        const long long per_v =
            (long long)(L.size() - 1) * (2LL * (opt.nu1 + opt.nu2) + 3) + 1 + cut * (opt.nu1 + opt.nu2 + 1);
        const int mixed = opt.precision == GBP_PREC_MIXED;
        const long long per_step = (mixed ? opt.ir_inner_cycles : 1) * per_v + 2 + mixed + 2 * cut;
        const int steps = stats->outer_iters - 1;
        stats->kernel_launches = 1 + (singular ? 4 : 0) + (guess ? 1 : 0) + 2 + 2 * cut + steps * per_step + 3 +
                                 2 * cut + ((phi_io && phi_io->data) ? 1 : 0);
    }
    return status;
}

namespace {

__global__ void k_mac_fill_seeded(CellGeom g, float* __restrict__ a, unsigned seed)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nc = (long long)g.n[0] * g.n[1] * g.n[2];
    if (t >= nc) return;
    const int i = (int)(t % g.n[0]), j = (int)((t / g.n[0]) % g.n[1]), k = (int)(t / ((long long)g.n[0] * g.n[1]));
    unsigned h = (unsigned)t * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    a[pidx(g.sy, g.sz, i, j, k)] = (float)(h & 0xffffff) / 16777216.f - 0.5f;
}

__global__ void k_mac_maxdiff(const float* __restrict__ a, const float* __restrict__ ref, long long n,
                              unsigned long long* out)
{
    double d = 0.0, m = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        d = fmax(d, fabs((double)a[t] - (double)ref[t]));
        m = fmax(m, fabs((double)ref[t]));
    }
    atomicMax(out, (unsigned long long)__double_as_longlong(d));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong(m));
}

}  // namespace

int MacSolver::check_coarse_cycle(double* diff)
{
    const int lc = coarse_first();
    if (lc < 1 || !beta_ready) {
        set_error("check_coarse_cycle: the MAC plan has no cluster-cycled levels (levels " + std::to_string(L.size()) +
                  ", dense bottom " + std::to_string((int)dense_bottom) + ") or no beta");
        return GBP_BAD_ARG;
    }
    const MacLevel& v = L[lc];
    const CellGeom& g = v.g;
    const size_t bytes = sizeof(float) * g.count;
    float *B = nullptr, *C = nullptr;
    unsigned long long* dm = nullptr;
    GBP_CUDA(cudaMalloc(&B, bytes));
    GBP_CUDA(cudaMalloc(&C, bytes));
    GBP_CUDA(cudaMalloc(&dm, 2 * sizeof(unsigned long long)));
    cap_or_st = st;
    launch_rc = 0;
    GBP_CUDA(cudaMemsetAsync(B, 0, bytes, st));
    const long long nc = (long long)g.n[0] * g.n[1] * g.n[2];
    k_mac_fill_seeded<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(g, B, 77u);
    use_coarse = false;
    vcycle<float>(lc, B, true);
    cudaMemcpyAsync(C, v.x32, bytes, cudaMemcpyDeviceToDevice, st);
    use_coarse = true;
    vcycle<float>(lc, B, true);
    cudaMemsetAsync(dm, 0, 2 * sizeof(unsigned long long), st);
    k_mac_maxdiff<<<592, 256, 0, st>>>(v.x32, C, (long long)g.count, dm);
    unsigned long long h[2] = {0, 0};
    cudaMemcpyAsync(h, dm, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(B);
    cudaFree(C);
    cudaFree(dm);
    const int rc = launch_rc;
    launch_rc = 0;
    if (e != cudaSuccess) return cuda_fail(e, "check_coarse_cycle (MAC)");
    if (rc) return rc;
    double d, m;
    memcpy(&d, &h[0], 8);
    memcpy(&m, &h[1], 8);
    *diff = m > 0 ? d / m : d;
    return GBP_OK;
}

}  // namespace gbp
