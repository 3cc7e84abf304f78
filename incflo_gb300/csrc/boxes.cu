// Multi-box levels at the C ABI: a level whose MultiFabs hold several FABs (incflo's
// amr.max_grid_size split) passes one gbp_array4 per FAB with the level's BoxArray. One batched kernel
// per field gathers every FAB's valid region into the plan's single-box staging arrays (plus the ghost
// cells the solve reads across domain sides), the single-box entry point runs on them, and the outputs
// are scattered back to every FAB. Reference call sites: the MFIter loops over the level MultiFabs of
// src/projection/incflo_apply_nodal_projection.cpp:58-93, 124-192, 221-257 and
// src/convection/incflo_compute_MAC_projected_velocities.cpp:82-90, 272-299.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gbp_internal.cuh"
#include "plan.h"

using namespace gbp;

namespace {

// one FAB region copied between the FAB and the staging array (inclusive bounds, level index space)
struct BoxXfer {
    gbp_array4 fab;
    int lo[3], hi[3];
    long long count;
};

__device__ __forceinline__ double* at(const gbp_array4& a, int i, int j, int k, int c)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride +
           (long long)(k - a.lo[2]) * a.kstride + (long long)c * a.nstride;
}

// mode 0: staging <- FAB; mode 1: FAB <- staging. blockIdx.y = the box.
__global__ void __launch_bounds__(256) k_box_xfer(const BoxXfer* __restrict__ tab, gbp_array4 stage, int ncomp,
                                                  int mode)
{
    const BoxXfer& b = tab[blockIdx.y];
    const int ex = b.hi[0] - b.lo[0] + 1, ey = b.hi[1] - b.lo[1] + 1;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < b.count;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = q / ex;
        const int i = b.lo[0] + (int)(q - r * ex);
        const int j = b.lo[1] + (int)(r % ey);
        const int k = b.lo[2] + (int)(r / ey);
        for (int c = 0; c < ncomp; ++c) {
            double* s = at(stage, i, j, k, c);
            double* f = at(b.fab, i, j, k, c);
            if (mode == 0)
                *s = *f;
            else
                *f = *s;
        }
    }
}

int box_fail(const std::string& what)
{
    set_error(what);
    return GBP_BAD_ARG;
}

// The BoxArray must tile the level: every box inside the domain, pairwise disjoint, volumes adding up.
int check_boxes(const gbp_plan* p, int nbox, const int* boxes, const char* fn)
{
    if (nbox < 1 || !boxes) return box_fail(std::string(fn) + ": need at least one box");
    const int* n = p->geom.n_cell;
    long long vol = 0;
    for (int b = 0; b < nbox; ++b) {
        const int* B = boxes + 6 * b;
        for (int d = 0; d < 3; ++d)
            if (B[d] < 0 || B[3 + d] >= n[d] || B[d] > B[3 + d])
                return box_fail(std::string(fn) + ": box " + std::to_string(b) + " is empty or leaves the domain");
        vol += (long long)(B[3] - B[0] + 1) * (B[4] - B[1] + 1) * (B[5] - B[2] + 1);
        for (int c = 0; c < b; ++c) {
            const int* C = boxes + 6 * c;
            bool overlap = true;
            for (int d = 0; d < 3; ++d) overlap = overlap && B[d] <= C[3 + d] && C[d] <= B[3 + d];
            if (overlap)
                return box_fail(std::string(fn) + ": boxes " + std::to_string(c) + " and " + std::to_string(b) +
                                " overlap");
        }
    }
    if (vol != (long long)n[0] * n[1] * n[2]) return box_fail(std::string(fn) + ": the boxes do not cover the domain");
    return GBP_OK;
}

// A field of the level: per-FAB arrays, the region of each box it moves (valid cells, nodes or faces,
// widened by one ghost on chosen domain sides), and the staging array it maps to.
struct Field {
    gbp_array4 stage{};
    std::vector<BoxXfer> xf;
    int ncomp = 1;
};

// staging array over [lo, hi] (inclusive) with ncomp components, carved from the plan's buffer
gbp_array4 stage_array(double* base, const int lo[3], const int hi[3], int ncomp)
{
    gbp_array4 a{};
    a.data = base;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = lo[d];
        a.hi[d] = hi[d];
    }
    a.ncomp = ncomp;
    a.jstride = hi[0] - lo[0] + 1;
    a.kstride = a.jstride * (long long)(hi[1] - lo[1] + 1);
    a.nstride = a.kstride * (long long)(hi[2] - lo[2] + 1);
    return a;
}

long long stage_count(const gbp_array4& a) { return a.nstride * a.ncomp; }

// box b's region: cells lo..hi (+1 on the high side in direction `face`, or on every side for nodes),
// widened by `ghost` cells on the domain sides flagged in widen_lo / widen_hi
void region(const gbp_plan* p, const int* B, int face, bool nodes, int ghost, const bool widen_lo[3],
            const bool widen_hi[3], int lo[3], int hi[3])
{
    for (int d = 0; d < 3; ++d) {
        lo[d] = B[d];
        hi[d] = B[3 + d] + ((nodes || d == face) ? 1 : 0);
        if (ghost && widen_lo[d] && B[d] == 0) lo[d] -= ghost;
        if (ghost && widen_hi[d] && B[3 + d] == p->geom.n_cell[d] - 1) hi[d] += ghost;
    }
}

int add_field(const gbp_plan* p, int nbox, const int* boxes, const gbp_array4* const* fabs, int ncomp, int face,
              bool nodes, int ghost, const bool widen_lo[3], const bool widen_hi[3], const char* what, Field& f)
{
    f.ncomp = ncomp;
    f.xf.resize((size_t)nbox);
    for (int b = 0; b < nbox; ++b) {
        const gbp_array4* a = fabs[b];
        BoxXfer& x = f.xf[(size_t)b];
        region(p, boxes + 6 * b, face, nodes, ghost, widen_lo, widen_hi, x.lo, x.hi);
        if (!a || !a->data || a->ncomp < ncomp || a->jstride <= 0 || a->kstride <= 0 || (ncomp > 1 && a->nstride <= 0))
            return box_fail(std::string(what) + ": FAB " + std::to_string(b) + " is missing or has too few components");
        for (int d = 0; d < 3; ++d)
            if (x.lo[d] < a->lo[d] || x.hi[d] > a->hi[d])
                return box_fail(std::string(what) + ": FAB " + std::to_string(b) +
                                " does not cover its box (and the ghost cells read across domain sides)");
        x.fab = *a;
        x.count = (long long)(x.hi[0] - x.lo[0] + 1) * (x.hi[1] - x.lo[1] + 1) * (x.hi[2] - x.lo[2] + 1);
    }
    return GBP_OK;
}

// staging memory of the plan for `fields` (grown when needed) and the device transfer table
int reserve(gbp_plan* p, std::vector<Field*>& fields, const std::vector<std::pair<const int*, const int*>>& ranges)
{
    size_t need = 0;
    for (size_t q = 0; q < fields.size(); ++q) {
        const int* lo = ranges[q].first;
        const int* hi = ranges[q].second;
        long long c = fields[q]->ncomp;
        for (int d = 0; d < 3; ++d) c *= (long long)(hi[d] - lo[d] + 1);
        need += ((size_t)c * sizeof(double) + 255) & ~size_t(255);
    }
    if (p->boxbuf_bytes < need) {
        GBP_CUDA(cudaStreamSynchronize(p->stream));
        if (p->boxbuf) cudaFree(p->boxbuf);
        p->boxbuf = nullptr;
        p->boxbuf_bytes = 0;
        GBP_CUDA(cudaMalloc(&p->boxbuf, need));
        p->boxbuf_bytes = need;
        // ghost cells no FAB supplies (sides the solve never reads) stay 0, never uninitialised
        GBP_CUDA(cudaMemsetAsync(p->boxbuf, 0, need, p->stream));
    }
    size_t off = 0;
    for (size_t q = 0; q < fields.size(); ++q) {
        fields[q]->stage =
            stage_array(reinterpret_cast<double*>(reinterpret_cast<char*>(p->boxbuf) + off), ranges[q].first,
                        ranges[q].second, fields[q]->ncomp);
        off += ((size_t)stage_count(fields[q]->stage) * sizeof(double) + 255) & ~size_t(255);
    }
    size_t tab = 0;
    for (Field* f : fields) tab += f->xf.size() * sizeof(BoxXfer);
    if (p->boxtab_bytes < tab) {
        GBP_CUDA(cudaStreamSynchronize(p->stream));
        if (p->boxtab) cudaFree(p->boxtab);
        p->boxtab = nullptr;
        p->boxtab_bytes = 0;
        GBP_CUDA(cudaMalloc(&p->boxtab, tab));
        p->boxtab_bytes = tab;
    }
    // one table upload for every field; the host vectors are staged by the copy (pageable source)
    std::vector<BoxXfer> all;
    for (Field* f : fields) all.insert(all.end(), f->xf.begin(), f->xf.end());
    GBP_CUDA(cudaMemcpyAsync(p->boxtab, all.data(), all.size() * sizeof(BoxXfer), cudaMemcpyHostToDevice, p->stream));
    GBP_CUDA(cudaStreamSynchronize(p->stream));
    return GBP_OK;
}

// launch the transfer of field q (its table entries start after those of the fields before it)
void xfer(gbp_plan* p, const std::vector<Field*>& fields, size_t q, int mode)
{
    size_t first = 0;
    for (size_t r = 0; r < q; ++r) first += fields[r]->xf.size();
    const Field& f = *fields[q];
    long long mx = 1;
    for (const BoxXfer& x : f.xf) mx = std::max(mx, x.count);
    const unsigned gx = (unsigned)std::min<long long>((mx + 255) / 256, 1024);
    k_box_xfer<<<dim3(gx, (unsigned)f.xf.size()), 256, 0, p->stream>>>(
        reinterpret_cast<const BoxXfer*>(p->boxtab) + first, f.stage, f.ncomp, mode);
}

}  // namespace

extern "C" {

int gbp_apply_nodal_projection_boxes(gbp_plan* p, int nbox, const int* boxes, gbp_array4* const* vel,
                                     const gbp_array4* const* vel_old, const gbp_array4* const* rho, double rho0,
                                     gbp_array4* const* gp, gbp_array4* const* p_nd, double time, double dt,
                                     double prev_dt, double scaling_factor, int incremental, int set_inflow_bc,
                                     gbp_stats* stats)
{
    const char* fn = "gbp_apply_nodal_projection_boxes";
    if (!p || !p->nodal) return box_fail(std::string(fn) + ": not a nodal plan");
    int rc = check_boxes(p, nbox, boxes, fn);
    if (rc) return rc;
    if (!vel) return box_fail(std::string(fn) + ": vel is required");
    const bool small_dt = time > 0.0 && dt < 0.1 * prev_dt;
    const bool sub_old = small_dt || incremental;
    if (sub_old && !vel_old) return box_fail(std::string(fn) + ": vel_old is required (incremental / small dt)");
    if (!incremental && !gp) return box_fail(std::string(fn) + ": gp is required");
    const int* n = p->geom.n_cell;
    // the velocity's ghost cells are read across inflow sides only
    bool in_lo[3], in_hi[3], none[3] = {false, false, false};
    for (int d = 0; d < 3; ++d) {
        in_lo[d] = p->bc_lo[d] == GBP_BC_INFLOW;
        in_hi[d] = p->bc_hi[d] == GBP_BC_INFLOW;
    }
    Field fv, fo, fr, fg, fp;
    std::vector<Field*> fields;
    std::vector<std::pair<const int*, const int*>> ranges;
    const int c_lo[3] = {0, 0, 0}, c_hi[3] = {n[0] - 1, n[1] - 1, n[2] - 1};
    const int g_lo[3] = {-1, -1, -1}, g_hi[3] = {n[0], n[1], n[2]};
    const int n_hi[3] = {n[0], n[1], n[2]};
    if ((rc = add_field(p, nbox, boxes, vel, 3, -1, false, 1, in_lo, in_hi, "vel", fv))) return rc;
    fields.push_back(&fv);
    ranges.push_back({g_lo, g_hi});
    if (sub_old) {
        if ((rc = add_field(p, nbox, boxes, vel_old, 3, -1, false, 0, none, none, "vel_old", fo))) return rc;
        fields.push_back(&fo);
        ranges.push_back({c_lo, c_hi});
    }
    if (rho) {
        if ((rc = add_field(p, nbox, boxes, rho, 1, -1, false, 0, none, none, "rho", fr))) return rc;
        fields.push_back(&fr);
        ranges.push_back({c_lo, c_hi});
    }
    if (gp) {
        if ((rc = add_field(p, nbox, boxes, const_cast<const gbp_array4* const*>(gp), 3, -1, false, 0, none, none,
                            "gp", fg)))
            return rc;
        fields.push_back(&fg);
        ranges.push_back({c_lo, c_hi});
    }
    if (p_nd) {
        if ((rc = add_field(p, nbox, boxes, const_cast<const gbp_array4* const*>(p_nd), 1, -1, true, 0, none, none,
                            "p_nd", fp)))
            return rc;
        fields.push_back(&fp);
        ranges.push_back({c_lo, n_hi});
    }
    if ((rc = reserve(p, fields, ranges))) return rc;
    // inputs in (p_nd too when it accumulates: the incremental form adds phi to it)
    for (size_t q = 0; q < fields.size(); ++q)
        if (fields[q] != &fp || incremental) xfer(p, fields, q, 0);
    GBP_CUDA(cudaGetLastError());
    rc = gbp_apply_nodal_projection(p, &fv.stage, sub_old ? &fo.stage : nullptr, rho ? &fr.stage : nullptr, rho0,
                                    gp ? &fg.stage : nullptr, p_nd ? &fp.stage : nullptr, time, dt, prev_dt,
                                    scaling_factor, incremental, set_inflow_bc, stats);
    if (rc != GBP_OK && rc != GBP_NOT_CONVERGED) return rc;
    // outputs back to every FAB: the velocity (valid cells), gp and p_nd (each box's nodes)
    for (size_t q = 0; q < fields.size(); ++q)
        if (fields[q] == &fv || fields[q] == &fg || fields[q] == &fp) xfer(p, fields, q, 1);
    GBP_CUDA(cudaGetLastError());
    GBP_CUDA(cudaStreamSynchronize(p->stream));
    return rc;
}

int gbp_mac_set_beta_from_density_boxes(gbp_plan* p, int nbox, const int* boxes, const gbp_array4* const* rho,
                                        double dt)
{
    const char* fn = "gbp_mac_set_beta_from_density_boxes";
    if (!p || !p->mac) return box_fail(std::string(fn) + ": not a MAC plan");
    int rc = check_boxes(p, nbox, boxes, fn);
    if (rc) return rc;
    if (!rho) return box_fail(std::string(fn) + ": rho is required");
    const int* n = p->geom.n_cell;
    // rho is read one cell across Dirichlet sides
    bool d_lo[3], d_hi[3];
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        d_lo[d] = p->bc_lo[d] == GBP_BC_DIRICHLET;
        d_hi[d] = p->bc_hi[d] == GBP_BC_DIRICHLET;
        lo[d] = d_lo[d] ? -1 : 0;
        hi[d] = n[d] - 1 + (d_hi[d] ? 1 : 0);
    }
    Field fr;
    if ((rc = add_field(p, nbox, boxes, rho, 1, -1, false, 1, d_lo, d_hi, "rho", fr))) return rc;
    std::vector<Field*> fields{&fr};
    std::vector<std::pair<const int*, const int*>> ranges{{lo, hi}};
    if ((rc = reserve(p, fields, ranges))) return rc;
    xfer(p, fields, 0, 0);
    GBP_CUDA(cudaGetLastError());
    rc = gbp_mac_set_beta_from_density(p, &fr.stage, dt);
    if (rc) return rc;
    GBP_CUDA(cudaStreamSynchronize(p->stream));
    return GBP_OK;
}

int gbp_mac_project_boxes(gbp_plan* p, int nbox, const int* boxes, gbp_array4* const* ux, gbp_array4* const* uy,
                          gbp_array4* const* uz, gbp_array4* const* phi, int phi_guess, gbp_stats* stats)
{
    const char* fn = "gbp_mac_project_boxes";
    if (!p || !p->mac) return box_fail(std::string(fn) + ": not a MAC plan");
    int rc = check_boxes(p, nbox, boxes, fn);
    if (rc) return rc;
    if (!ux || !uy || !uz) return box_fail(std::string(fn) + ": umac is required");
    const int* n = p->geom.n_cell;
    const bool none[3] = {false, false, false};
    Field fu[3], fphi;
    std::vector<Field*> fields;
    std::vector<std::pair<const int*, const int*>> ranges;
    const int c_lo[3] = {0, 0, 0}, c_hi[3] = {n[0] - 1, n[1] - 1, n[2] - 1};
    int f_hi[3][3];
    gbp_array4* const* u[3] = {ux, uy, uz};
    for (int d = 0; d < 3; ++d) {
        for (int e = 0; e < 3; ++e) f_hi[d][e] = n[e] - 1 + (e == d ? 1 : 0);
        if ((rc = add_field(p, nbox, boxes, const_cast<const gbp_array4* const*>(u[d]), 1, d, false, 0, none, none,
                            "umac", fu[d])))
            return rc;
        fields.push_back(&fu[d]);
        ranges.push_back({c_lo, f_hi[d]});
    }
    if (phi) {
        if ((rc = add_field(p, nbox, boxes, const_cast<const gbp_array4* const*>(phi), 1, -1, false, 0, none, none,
                            "phi", fphi)))
            return rc;
        fields.push_back(&fphi);
        ranges.push_back({c_lo, c_hi});
    }
    if ((rc = reserve(p, fields, ranges))) return rc;
    for (size_t q = 0; q < fields.size(); ++q)
        if (fields[q] != &fphi || phi_guess) xfer(p, fields, q, 0);
    GBP_CUDA(cudaGetLastError());
    rc = gbp_mac_project(p, &fu[0].stage, &fu[1].stage, &fu[2].stage, phi ? &fphi.stage : nullptr, phi_guess, stats);
    if (rc != GBP_OK && rc != GBP_NOT_CONVERGED) return rc;
    for (size_t q = 0; q < fields.size(); ++q) xfer(p, fields, q, 1);
    GBP_CUDA(cudaGetLastError());
    GBP_CUDA(cudaStreamSynchronize(p->stream));
    return rc;
}

}  // extern "C"
