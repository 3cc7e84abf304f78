// The C ABI (include/incflo_gb300.h): plans, options (the nodal_proj.* / mac_proj.* inputs surface),
// and the projection entry points. Never aborts; every failure is a status code plus a message
// retrievable with gbp_last_error().
#include <ctype.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "gbp_internal.cuh"
#include "mac_solver.h"
#include "nodal_solver.h"
#include "plan.h"
#include "amr.h"
#include "tensor.h"
#include "cc_projection.h"
#include "solvability.h"

namespace gbp {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GBP_CUDA_ERROR;
}

}  // namespace gbp

using namespace gbp;


static bool valid_array(const gbp_array4* a, int ncomp_min)
{
    return a && a->data && a->ncomp >= ncomp_min && a->jstride > 0 && a->kstride > 0 &&
           (a->ncomp == 1 || a->nstride > 0);
}

// the region [lo,hi] (inclusive, per direction) must lie inside the array's allocated bounds
static bool covers(const gbp_array4* a, const int lo[3], const int hi[3])
{
    for (int d = 0; d < 3; ++d)
        if (lo[d] < a->lo[d] || hi[d] > a->hi[d]) return false;
    return true;
}

extern "C" {

int gbp_abi_version(void) { return GBP_ABI_VERSION; }

const char* gbp_status_string(int status)
{
    switch (status) {
    case GBP_OK: return "ok";
    case GBP_NOT_CONVERGED: return "not converged";
    case GBP_NAN: return "residual is NaN or Inf";
    case GBP_BAD_ARG: return "bad argument";
    case GBP_CUDA_ERROR: return "CUDA error";
    case GBP_TIMEOUT: return "device wait timed out";
    case GBP_NO_DEVICE: return "no usable CUDA device";
    default: return "unknown status";
    }
}

const char* gbp_last_error(void) { return g_last_error.c_str(); }

int gbp_device_check(void)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error("no CUDA device visible");
        return GBP_NO_DEVICE;
    }
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3) {
        set_error("this library is built for sm_103 (GB300) only; device is sm_" + std::to_string(major) +
                  std::to_string(minor));
        return GBP_NO_DEVICE;
    }
    return GBP_OK;
}

int gbp_options_default(int kind, gbp_options* o)
{
    if (!o) return GBP_BAD_ARG;
    memset(o, 0, sizeof(*o));
    o->rtol = 1.0e-11;
    o->atol = 1.0e-14;
    o->max_coarsening_level = 100;
    o->maxiter = kind == GBP_MAC ? 200 : 100;
    o->bottom_maxiter = 200;
    o->bottom_rtol = 1.0e-4;
    o->bottom_atol = -1.0;
    o->verbose = 0;
    o->bottom_verbose = 0;
    o->precision = GBP_PREC_FP64;
    o->nu1 = 2;
    o->nu2 = 2;
    o->omega = 0.85;
    o->ir_inner_cycles = 5;
    o->use_graphs = 1;
    o->always_use_bnorm = 1;
    o->initial_guess = 0;
    return GBP_OK;
}

static bool parse_double(const char* v, double* out)
{
    char* end = nullptr;
    double x = strtod(v, &end);
    if (end == v) return false;
    while (*end && isspace((unsigned char)*end)) ++end;
    if (*end) return false;
    *out = x;
    return true;
}

static bool parse_int(const char* v, int* out)
{
    double x;
    if (!parse_double(v, &x) || x != floor(x)) return false;
    *out = (int)x;
    return true;
}

int gbp_options_set(gbp_options* o, const char* key, const char* value)
{
    if (!o || !key || !value) return GBP_BAD_ARG;
    std::string k(key);
    std::string v(value);
    while (!v.empty() && isspace((unsigned char)v.back())) v.pop_back();
    size_t a = 0;
    while (a < v.size() && isspace((unsigned char)v[a])) ++a;
    v = v.substr(a);
    if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
    const char* s = v.c_str();
    bool ok = true;
    if (k == "mg_rtol")
        ok = parse_double(s, &o->rtol);
    else if (k == "mg_atol")
        ok = parse_double(s, &o->atol);
    else if (k == "mg_max_coarsening_level")
        ok = parse_int(s, &o->max_coarsening_level);
    else if (k == "maxiter")
        ok = parse_int(s, &o->maxiter);
    else if (k == "bottom_maxiter")
        ok = parse_int(s, &o->bottom_maxiter);
    else if (k == "bottom_rtol")
        ok = parse_double(s, &o->bottom_rtol);
    else if (k == "bottom_atol")
        ok = parse_double(s, &o->bottom_atol);
    else if (k == "verbose")
        ok = parse_int(s, &o->verbose);
    else if (k == "bottom_verbose")
        ok = parse_int(s, &o->bottom_verbose);
    else if (k == "bottom_solver")
        // the coarsest level is always solved by conjugate gradients in one CTA; every MLMG bottom
        // solver name incflo decks use is accepted (InputsMultigrid.rst)
        ok = v == "bicgstab" || v == "bicgcg" || v == "cg" || v == "cgbicg" || v == "smoother" || v == "hypre" ||
             v == "petsc" || v == "default";
    else if (k == "precision") {
        if (v == "fp64" || v == "double")
            o->precision = GBP_PREC_FP64;
        else if (v == "mixed" || v == "fp32-ir")
            o->precision = GBP_PREC_MIXED;
        else
            ok = false;
    } else if (k == "num_pre_smooth")
        ok = parse_int(s, &o->nu1);
    else if (k == "num_post_smooth")
        ok = parse_int(s, &o->nu2);
    else if (k == "jacobi_weight")
        ok = parse_double(s, &o->omega);
    else if (k == "ir_inner_cycles")
        ok = parse_int(s, &o->ir_inner_cycles);
    else if (k == "use_graphs")
        ok = parse_int(s, &o->use_graphs);
    else if (k == "always_use_bnorm")
        ok = parse_int(s, &o->always_use_bnorm);
    else if (k == "smoother")
        ok = v == "jacobi" || v == "rbgs" || v == "default";
    else if (k == "initial_guess") {
        if (v == "zero" || v == "0")
            o->initial_guess = 0;
        else if (v == "previous" || v == "1")
            o->initial_guess = 1;
        else
            ok = false;
    }
    else {
        set_error("unknown projection option '" + k + "'");
        return GBP_BAD_ARG;
    }
    if (!ok) {
        set_error("bad value '" + v + "' for projection option '" + k + "'");
        return GBP_BAD_ARG;
    }
    return GBP_OK;
}

int gbp_options_parse(gbp_options* o, const char* prefix, const char* text)
{
    if (!o || !prefix || !text) return GBP_BAD_ARG;
    const std::string pre = std::string(prefix) + ".";
    const char* p = text;
    while (*p) {
        const char* e = strchr(p, '\n');
        std::string line = e ? std::string(p, e - p) : std::string(p);
        p = e ? e + 1 : p + strlen(p);
        size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = line.substr(0, eq);
        std::string val = line.substr(eq + 1);
        while (!key.empty() && isspace((unsigned char)key.back())) key.pop_back();
        size_t a = 0;
        while (a < key.size() && isspace((unsigned char)key[a])) ++a;
        key = key.substr(a);
        if (key.compare(0, pre.size(), pre) != 0) continue;
        int rc = gbp_options_set(o, key.substr(pre.size()).c_str(), val.c_str());
        if (rc) return rc;
    }
    return GBP_OK;
}

int gbp_plan_create(const gbp_geometry* geom, int kind, const int bc_lo[3], const int bc_hi[3],
                    const gbp_options* opt, void* stream, gbp_plan** plan)
{
    if (!geom || !bc_lo || !bc_hi || !plan || (kind != GBP_NODAL && kind != GBP_MAC)) {
        set_error("gbp_plan_create: null argument or unknown kind");
        return GBP_BAD_ARG;
    }
    *plan = nullptr;
    int rc = gbp_device_check();
    if (rc) return rc;
    gbp_options o;
    if (opt)
        o = *opt;
    else
        gbp_options_default(kind, &o);
    gbp_plan* p = new (std::nothrow) gbp_plan();
    if (!p) return GBP_BAD_ARG;
    p->kind = kind;
    p->stream = (cudaStream_t)stream;
    p->geom = *geom;
    for (int d = 0; d < 3; ++d) {
        p->bc_lo[d] = bc_lo[d];
        p->bc_hi[d] = bc_hi[d];
    }
    if (kind == GBP_NODAL) {
        p->nodal = new NodalSolver();
        rc = p->nodal->init(*geom, bc_lo, bc_hi, o, p->stream);
    } else {
        p->mac = new MacSolver();
        rc = p->mac->init(*geom, bc_lo, bc_hi, o, p->stream);
    }
    if (rc) {
        gbp_plan_destroy(p);
        return rc;
    }
    *plan = p;
    return GBP_OK;
}

int gbp_plan_destroy(gbp_plan* p)
{
    if (!p) return GBP_OK;
    if (p->stream) cudaStreamSynchronize(p->stream);
    delete p->nodal;
    delete p->mac;
    if (p->hbuf) cudaFree(p->hbuf);
    if (p->copy_stream) {
        cudaStreamSynchronize(p->copy_stream);
        cudaStreamDestroy(p->copy_stream);
    }
    if (p->ev_in) cudaEventDestroy(p->ev_in);
    if (p->ev_phi) cudaEventDestroy(p->ev_phi);
    if (p->ev_out) cudaEventDestroy(p->ev_out);
    for (auto e : p->ev_slab)
        if (e) cudaEventDestroy(e);
    for (auto e : p->ev_rhs)
        if (e) cudaEventDestroy(e);
    if (p->dflux) cudaFree(p->dflux);
    if (p->ccbuf) cudaFree(p->ccbuf);
    if (p->boxbuf) cudaFree(p->boxbuf);
    if (p->boxtab) cudaFree(p->boxtab);
    delete p;
    return GBP_OK;
}

int gbp_plan_set_options(gbp_plan* p, const gbp_options* opt)
{
    if (!p || !opt) return GBP_BAD_ARG;
    return p->nodal ? p->nodal->set_options(*opt) : p->mac->set_options(*opt);
}

size_t gbp_plan_device_bytes(const gbp_plan* p)
{
    if (!p) return 0;
    size_t b = p->hbuf_bytes + p->boxbuf_bytes + p->boxtab_bytes;
    b += p->nodal ? p->nodal->device_bytes() : p->mac->device_bytes();
    return b;
}

int gbp_nodal_set_sigma_from_density(gbp_plan* p, const gbp_array4* rho, double scaling_factor, double rho0)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_set_sigma_from_density: not a nodal plan");
        return GBP_BAD_ARG;
    }
    if (rho) {
        const int lo[3] = {0, 0, 0};
        const int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        if (!valid_array(rho, 1) || !covers(rho, lo, hi)) {
            set_error("gbp_nodal_set_sigma_from_density: rho must cover the valid cells");
            return GBP_BAD_ARG;
        }
    }
    return p->nodal->set_sigma_from_density(rho, scaling_factor, rho0);
}

int gbp_nodal_set_sigma(gbp_plan* p, const gbp_array4* sigma, double const_sigma)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_set_sigma: not a nodal plan");
        return GBP_BAD_ARG;
    }
    if (sigma) {
        const int lo[3] = {0, 0, 0};
        const int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        if (!valid_array(sigma, 1) || !covers(sigma, lo, hi)) {
            set_error("gbp_nodal_set_sigma: sigma must cover the valid cells");
            return GBP_BAD_ARG;
        }
    }
    return p->nodal->set_sigma(sigma, const_sigma);
}

static int check_vel(const gbp_plan* p, const gbp_array4* vel, bool need_ghost)
{
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const bool inflow = p->bc_lo[d] == GBP_BC_INFLOW || p->bc_hi[d] == GBP_BC_INFLOW;
        const int g = (need_ghost && inflow) ? 1 : 0;
        lo[d] = -g;
        hi[d] = p->geom.n_cell[d] - 1 + g;
    }
    if (!valid_array(vel, 3) || !covers(vel, lo, hi)) {
        set_error("velocity array must hold 3 components over the valid cells (plus one ghost cell "
                  "across inflow faces)");
        return GBP_BAD_ARG;
    }
    return GBP_OK;
}

static int check_cells(const gbp_plan* p, const gbp_array4* a, int ncomp, const char* what)
{
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
    if (!valid_array(a, ncomp) || !covers(a, lo, hi)) {
        set_error(std::string(what) + " must cover the valid cells with enough components");
        return GBP_BAD_ARG;
    }
    return GBP_OK;
}

static int check_nodes(const gbp_plan* p, const gbp_array4* a, const char* what)
{
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {p->geom.n_cell[0], p->geom.n_cell[1], p->geom.n_cell[2]};
    if (!valid_array(a, 1) || !covers(a, lo, hi)) {
        set_error(std::string(what) + " must cover nodes 0..n in every direction");
        return GBP_BAD_ARG;
    }
    return GBP_OK;
}

static void fill_rhs_corr(const gbp_plan* p, RhsArgs& ra, CorrArgs& ca)
{
    const NodalGeom& g = p->nodal->geom0();
    for (int d = 0; d < 3; ++d) {
        ra.inflow_lo[d] = p->bc_lo[d] == GBP_BC_INFLOW;
        ra.inflow_hi[d] = p->bc_hi[d] == GBP_BC_INFLOW;
        ca.inv4h[d] = 1.0 / (4.0 * g.h[d]);
    }
    ra.cf[0] = 0.25 * g.h[1] * g.h[2];
    ra.cf[1] = 0.25 * g.h[0] * g.h[2];
    ra.cf[2] = 0.25 * g.h[0] * g.h[1];
}

int gbp_nodal_project(gbp_plan* p, gbp_array4* vel, gbp_array4* phi, gbp_array4* gradphi, int phi_guess,
                      gbp_stats* stats)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_project: not a nodal plan");
        return GBP_BAD_ARG;
    }
    int rc = check_vel(p, vel, true);
    if (rc) return rc;
    if (phi && phi->data && (rc = check_nodes(p, phi, "phi"))) return rc;
    if (gradphi && gradphi->data && (rc = check_cells(p, gradphi, 3, "gradphi"))) return rc;
    if (phi_guess && !(phi && phi->data)) {
        set_error("gbp_nodal_project: phi_guess set without phi");
        return GBP_BAD_ARG;
    }
    RhsArgs ra{};
    CorrArgs ca{};
    fill_rhs_corr(p, ra, ca);
    ra.vel = *vel;
    ca.vel = *vel;
    if (gradphi) ca.gradphi = *gradphi;
    if (stats) memset(stats, 0, sizeof(*stats));
    p->nodal->reset_count();
    return p->nodal->project(ra, ca, phi, 0, phi_guess ? phi : nullptr, stats);
}

int gbp_nodal_set_overset_mask(gbp_plan* p, const gbp_iarray4* m)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_set_overset_mask: not a nodal plan");
        return GBP_BAD_ARG;
    }
    if (m && m->data) {
        for (int d = 0; d < 3; ++d)
            if (m->lo[d] > 0 || m->hi[d] < p->geom.n_cell[d] || m->jstride <= 0 || m->kstride <= 0) {
                set_error("gbp_nodal_set_overset_mask: the mask must cover nodes 0..n");
                return GBP_BAD_ARG;
            }
    }
    return p->nodal->set_mask(m);
}

int gbp_nodal_divergence(gbp_plan* p, const gbp_array4* vel, int use_inflow, gbp_array4* div_out, double* max_norm)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_divergence: not a nodal plan");
        return GBP_BAD_ARG;
    }
    int rc = check_vel(p, vel, use_inflow != 0);
    if (rc) return rc;
    if (div_out && div_out->data && (rc = check_nodes(p, div_out, "div_out"))) return rc;
    RhsArgs ra{};
    CorrArgs ca{};
    fill_rhs_corr(p, ra, ca);
    ra.vel = *vel;
    if (!use_inflow)
        for (int d = 0; d < 3; ++d) ra.inflow_lo[d] = ra.inflow_hi[d] = 0;
    return p->nodal->divergence(ra, div_out, max_norm);
}

static int apply_nodal_impl(gbp_plan* p, gbp_array4* vel, const gbp_array4* vel_old, const gbp_array4* rho,
                            double rho0, gbp_array4* gp, gbp_array4* p_nd, double time, double dt, double prev_dt,
                            double scaling_factor, int incremental, int set_inflow_bc, gbp_stats* stats,
                            cudaEvent_t wait_before_rhs, const gbp::HostCopy* phi_copy,
                            const gbp::HostSlabs* out_slabs = nullptr, const gbp::RhsGroups* rhs_groups = nullptr);

int gbp_apply_nodal_projection(gbp_plan* p, gbp_array4* vel, const gbp_array4* vel_old, const gbp_array4* rho,
                               double rho0, gbp_array4* gp, gbp_array4* p_nd, double time, double dt, double prev_dt,
                               double scaling_factor, int incremental, int set_inflow_bc, gbp_stats* stats)
{
    return apply_nodal_impl(p, vel, vel_old, rho, rho0, gp, p_nd, time, dt, prev_dt, scaling_factor, incremental,
                            set_inflow_bc, stats, nullptr, nullptr);
}

// wait_before_rhs: an event the plan's stream waits on after sigma is set and before the right-hand
// side (the host path uploads the velocities meanwhile); phi_copy: a copy issued once p_nd is stored;
// out_slabs: the corrected velocity and gp copied out slab by slab behind the correction
static int apply_nodal_impl(gbp_plan* p, gbp_array4* vel, const gbp_array4* vel_old, const gbp_array4* rho,
                            double rho0, gbp_array4* gp, gbp_array4* p_nd, double time, double dt, double prev_dt,
                            double scaling_factor, int incremental, int set_inflow_bc, gbp_stats* stats,
                            cudaEvent_t wait_before_rhs, const gbp::HostCopy* phi_copy,
                            const gbp::HostSlabs* out_slabs, const gbp::RhsGroups* rhs_groups)
{
    if (!p || !p->nodal) {
        set_error("gbp_apply_nodal_projection: not a nodal plan");
        return GBP_BAD_ARG;
    }
    // incflo_apply_nodal_projection.cpp:36: the small-dt form projects (U* - U^n + dt Gp)
    const bool small_dt = time > 0.0 && dt < 0.1 * prev_dt;
    const bool sub_old = small_dt || incremental;
    int rc = check_vel(p, vel, set_inflow_bc != 0);
    if (rc) return rc;
    if (sub_old && (rc = check_cells(p, vel_old, 3, "vel_old"))) return rc;
    if (gp && (rc = check_cells(p, gp, 3, "gp"))) return rc;
    if (p_nd && (rc = check_nodes(p, p_nd, "p_nd"))) return rc;
    if (!incremental && !gp) {
        set_error("gbp_apply_nodal_projection: gp is required (its add-back is part of the projection)");
        return GBP_BAD_ARG;
    }
    p->nodal->reset_count();
    rc = gbp_nodal_set_sigma_from_density(p, rho, scaling_factor, rho0);
    if (rc) return rc;
    RhsArgs ra{};
    CorrArgs ca{};
    fill_rhs_corr(p, ra, ca);
    ra.vel = *vel;
    if (gp) ra.gp = *gp;
    if (sub_old) ra.vel_old = *vel_old;
    ra.add_gp = !incremental;
    ra.sub_old = sub_old;
    if (!(set_inflow_bc && !small_dt && !incremental))
        for (int d = 0; d < 3; ++d) ra.inflow_lo[d] = ra.inflow_hi[d] = 0;
    ca.vel = *vel;
    if (gp) ca.gp = *gp;
    ca.add_gp = !incremental;
    ca.incremental = incremental;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (wait_before_rhs) GBP_CUDA(cudaStreamWaitEvent(p->stream, wait_before_rhs, 0));
    return p->nodal->project(ra, ca, p_nd, incremental, nullptr, stats, phi_copy, out_slabs, rhs_groups);
}

int gbp_mac_set_beta(gbp_plan* p, const gbp_array4* bx, const gbp_array4* by, const gbp_array4* bz,
                     double const_beta)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_set_beta: not a MAC plan");
        return GBP_BAD_ARG;
    }
    const gbp_array4* src[3] = {bx, by, bz};
    const bool arrays = bx || by || bz;
    if (arrays) {
        for (int d = 0; d < 3; ++d) {
            int lo[3] = {0, 0, 0};
            int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
            hi[d] += 1;
            if (!valid_array(src[d], 1) || !covers(src[d], lo, hi)) {
                set_error("gbp_mac_set_beta: each beta array must cover its faces 0..n");
                return GBP_BAD_ARG;
            }
        }
    }
    return p->mac->set_beta(arrays ? 0 : 1, src, const_beta);
}

int gbp_mac_set_beta_from_density(gbp_plan* p, const gbp_array4* rho, double dt)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_set_beta_from_density: not a MAC plan");
        return GBP_BAD_ARG;
    }
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const bool dir = p->bc_lo[d] == GBP_BC_DIRICHLET || p->bc_hi[d] == GBP_BC_DIRICHLET;
        lo[d] = (dir && p->bc_lo[d] == GBP_BC_DIRICHLET) ? -1 : 0;
        hi[d] = p->geom.n_cell[d] - 1 + ((dir && p->bc_hi[d] == GBP_BC_DIRICHLET) ? 1 : 0);
    }
    if (!valid_array(rho, 1) || !covers(rho, lo, hi)) {
        set_error("gbp_mac_set_beta_from_density: rho must cover the valid cells and one ghost cell "
                  "across Dirichlet faces");
        return GBP_BAD_ARG;
    }
    const gbp_array4* src[3] = {rho, nullptr, nullptr};
    return p->mac->set_beta(2, src, dt);
}

int gbp_mac_set_robin(gbp_plan* p, const gbp_array4* robin_a, const gbp_array4* robin_b, const gbp_array4* robin_f)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_set_robin: not a MAC plan");
        return GBP_BAD_ARG;
    }
    const int lo[3] = {-1, -1, -1};
    const int hi[3] = {p->geom.n_cell[0], p->geom.n_cell[1], p->geom.n_cell[2]};
    for (const gbp_array4* a : {robin_a, robin_b}) {
        if (!valid_array(a, 1) || !covers(a, lo, hi)) {
            set_error("gbp_mac_set_robin: robin_a and robin_b must be cell arrays with one ghost layer");
            return GBP_BAD_ARG;
        }
    }
    if (robin_f && robin_f->data && !(valid_array(robin_f, 1) && covers(robin_f, lo, hi))) {
        set_error("gbp_mac_set_robin: robin_f must be a cell array with one ghost layer");
        return GBP_BAD_ARG;
    }
    return p->mac->set_robin(robin_a, robin_b, (robin_f && robin_f->data) ? robin_f : nullptr);
}

int gbp_mac_set_eb(gbp_plan* p, const gbp_array4* vfrac, const gbp_array4* ax, const gbp_array4* ay,
                   const gbp_array4* az, const gbp_array4* fx, const gbp_array4* fy, const gbp_array4* fz)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_set_eb: not a MAC plan");
        return GBP_BAD_ARG;
    }
    if (!vfrac || !vfrac->data) return p->mac->set_eb(nullptr, nullptr, nullptr);
    const gbp_array4* area[3] = {ax, ay, az};
    const gbp_array4* fc[3] = {fx, fy, fz};
    if (!valid_array(vfrac, 1)) {
        set_error("gbp_mac_set_eb: bad volume-fraction array");
        return GBP_BAD_ARG;
    }
    for (int d = 0; d < 3; ++d)
        if (!valid_array(area[d], 1) || !valid_array(fc[d], 2)) {
            set_error("gbp_mac_set_eb: need 3 area-fraction arrays and 3 face-centroid arrays with 2 components");
            return GBP_BAD_ARG;
        }
    return p->mac->set_eb(vfrac, area, fc);
}

int gbp_mac_set_eb_inflow(gbp_plan* p, const gbp_array4* eb_vel)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_set_eb_inflow: not a MAC plan");
        return GBP_BAD_ARG;
    }
    if (!eb_vel || !eb_vel->data) return p->mac->set_eb_inflow(nullptr);
    int rc = check_cells(p, eb_vel, 3, "gbp_mac_set_eb_inflow: eb_vel");
    if (rc) return rc;
    return p->mac->set_eb_inflow(eb_vel);
}

int gbp_mac_project(gbp_plan* p, gbp_array4* ux, gbp_array4* uy, gbp_array4* uz, gbp_array4* phi, int phi_guess,
                    gbp_stats* stats)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_project: not a MAC plan");
        return GBP_BAD_ARG;
    }
    gbp_array4* u[3] = {ux, uy, uz};
    for (int d = 0; d < 3; ++d) {
        int lo[3] = {0, 0, 0};
        int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        hi[d] += 1;
        if (!valid_array(u[d], 1) || !covers(u[d], lo, hi)) {
            set_error("gbp_mac_project: each umac array must cover its faces 0..n");
            return GBP_BAD_ARG;
        }
    }
    if (phi && phi->data) {
        int rc = check_cells(p, phi, 1, "phi");
        if (rc) return rc;
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    return p->mac->project(u, phi, phi_guess, stats);
}

int gbp_mac_get_fluxes(gbp_plan* p, const gbp_array4* phi, gbp_array4* fx, gbp_array4* fy, gbp_array4* fz)
{
    if (!p || !p->mac) {
        set_error("gbp_mac_get_fluxes: not a MAC plan");
        return GBP_BAD_ARG;
    }
    gbp_array4* f[3] = {fx, fy, fz};
    for (int d = 0; d < 3; ++d) {
        int lo[3] = {0, 0, 0};
        int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        hi[d] += 1;
        if (!valid_array(f[d], 1) || !covers(f[d], lo, hi)) {
            set_error("gbp_mac_get_fluxes: each flux array must cover its faces 0..n");
            return GBP_BAD_ARG;
        }
    }
    int rc = check_cells(p, phi, 1, "phi");
    if (rc) return rc;
    return p->mac->get_fluxes(*phi, f);
}

int gbp_apply_cc_projection(gbp_plan* p, gbp_array4* vel, const gbp_array4* vel_old, const gbp_array4* rho,
                            double rho0, gbp_array4* gp, gbp_array4* p_cc, gbp_array4* umac_x, gbp_array4* umac_y,
                            gbp_array4* umac_z, double time, double dt, double prev_dt, double scaling_factor,
                            int incremental, int set_inflow_bc, gbp_stats* stats)
{
    if (!p || !p->mac) {
        set_error("gbp_apply_cc_projection: not a MAC plan");
        return GBP_BAD_ARG;
    }
    // incflo_apply_cc_projection.cpp:212: the small-dt form projects (U* - U^n + dt Gp)
    const bool small_dt = time > 0.0 && dt < 0.1 * prev_dt;
    const bool sub_old = small_dt || incremental;
    int rc = check_vel(p, vel, true);
    if (rc) return rc;
    if (sub_old && (rc = check_cells(p, vel_old, 3, "vel_old"))) return rc;
    if (gp && (rc = check_cells(p, gp, 3, "gp"))) return rc;
    if (p_cc && (rc = check_cells(p, p_cc, 1, "p_cc"))) return rc;
    if (!incremental && !gp) {
        set_error("gbp_apply_cc_projection: gp is required (its add-back is part of the projection)");
        return GBP_BAD_ARG;
    }
    if (!(scaling_factor > 0.0) || (!rho && !(rho0 > 0.0))) {
        set_error("gbp_apply_cc_projection: scaling_factor and rho0 must be positive");
        return GBP_BAD_ARG;
    }
    if (rho) {
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = p->bc_lo[d] == GBP_BC_DIRICHLET ? -1 : 0;
            hi[d] = p->geom.n_cell[d] - 1 + (p->bc_hi[d] == GBP_BC_DIRICHLET ? 1 : 0);
        }
        if (!valid_array(rho, 1) || !covers(rho, lo, hi)) {
            set_error("gbp_apply_cc_projection: rho must cover the cells and one ghost across Dirichlet faces");
            return GBP_BAD_ARG;
        }
    }
    gbp_array4* u[3] = {umac_x, umac_y, umac_z};
    for (int d = 0; d < 3; ++d) {
        int lo[3] = {0, 0, 0};
        int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        hi[d] += 1;
        if (!valid_array(u[d], 1) || !covers(u[d], lo, hi)) {
            set_error("gbp_apply_cc_projection: each umac array must cover its faces 0..n");
            return GBP_BAD_ARG;
        }
    }
    if (!p->ccbuf) GBP_CUDA(cudaMalloc(&p->ccbuf, cc_scratch_doubles(p->geom) * sizeof(double)));
    CcArgs a{};
    a.vel = *vel;
    if (sub_old) a.vel_old = *vel_old;
    if (rho) a.rho = *rho;
    if (gp) a.gp = *gp;
    if (p_cc) a.p_cc = *p_cc;
    a.rho0 = rho0;
    a.s = scaling_factor;
    a.add_gp = !incremental;
    a.sub_old = sub_old;
    a.use_inflow = set_inflow_bc && !sub_old;
    a.incremental = incremental;
    if (stats) memset(stats, 0, sizeof(*stats));
    return cc_projection(p->geom, p->bc_lo, p->bc_hi, a, u, p->ccbuf, *p->mac, stats, p->stream);
}

static int plan_flux(gbp_plan* p)
{
    if (!p->dflux) GBP_CUDA(cudaMalloc(&p->dflux, 2 * sizeof(double)));
    return GBP_OK;
}

int gbp_enforce_inout_solvability(gbp_plan* p, gbp_array4* vel, const int dd_lo[3], const int dd_hi[3],
                                  double* inflow_outflow)
{
    if (!p || !dd_lo || !dd_hi || !valid_array(vel, 3)) {
        set_error("gbp_enforce_inout_solvability: plan, 3-component vel and dd_lo/dd_hi are required");
        return GBP_BAD_ARG;
    }
    const int lo[3] = {-1, -1, -1};
    const int hi[3] = {p->geom.n_cell[0], p->geom.n_cell[1], p->geom.n_cell[2]};
    if (!covers(vel, lo, hi)) {
        set_error("gbp_enforce_inout_solvability: vel must hold one ghost layer");
        return GBP_BAD_ARG;
    }
    int rc = plan_flux(p);
    if (!rc) rc = enforce_inout_cell(p->geom, dd_lo, dd_hi, *vel, p->dflux, p->stream);
    if (!rc && inflow_outflow) {
        GBP_CUDA(cudaMemcpyAsync(inflow_outflow, p->dflux, 2 * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        GBP_CUDA(cudaStreamSynchronize(p->stream));
    }
    return rc;
}

int gbp_mac_enforce_inout_solvability(gbp_plan* p, gbp_array4* ux, gbp_array4* uy, gbp_array4* uz,
                                      const int dd_lo[3], const int dd_hi[3], double* inflow_outflow)
{
    gbp_array4* u[3] = {ux, uy, uz};
    if (!p || !dd_lo || !dd_hi) {
        set_error("gbp_mac_enforce_inout_solvability: plan and dd_lo/dd_hi are required");
        return GBP_BAD_ARG;
    }
    gbp_array4 uu[3];
    for (int d = 0; d < 3; ++d) {
        int lo[3] = {0, 0, 0};
        int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
        hi[d] += 1;
        if (!valid_array(u[d], 1) || !covers(u[d], lo, hi)) {
            set_error("gbp_mac_enforce_inout_solvability: face arrays must cover faces 0..n");
            return GBP_BAD_ARG;
        }
        uu[d] = *u[d];
    }
    int rc = plan_flux(p);
    if (!rc) rc = enforce_inout_faces(p->geom, dd_lo, dd_hi, uu, p->dflux, p->stream);
    if (!rc && inflow_outflow) {
        GBP_CUDA(cudaMemcpyAsync(inflow_outflow, p->dflux, 2 * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        GBP_CUDA(cudaStreamSynchronize(p->stream));
    }
    return rc;
}

int gbp_average_down(const gbp_array4* fine, gbp_array4* crse, const int ratio[3], int ncomp, const int crse_lo[3],
                     const int crse_hi[3], void* stream)
{
    if (!fine || !crse || !ratio || !crse_lo || !crse_hi || ncomp < 1 || !valid_array(fine, ncomp) ||
        !valid_array(crse, ncomp)) {
        set_error("gbp_average_down: fine / coarse arrays with ncomp components and the coarse box are required");
        return GBP_BAD_ARG;
    }
    int flo[3], fhi[3];
    for (int d = 0; d < 3; ++d) {
        if (ratio[d] < 1 || crse_hi[d] < crse_lo[d]) {
            set_error("gbp_average_down: ratio must be >= 1 and the coarse box non-empty");
            return GBP_BAD_ARG;
        }
        flo[d] = crse_lo[d] * ratio[d];
        fhi[d] = crse_hi[d] * ratio[d] + ratio[d] - 1;
    }
    if (!covers(crse, crse_lo, crse_hi) || !covers(fine, flo, fhi)) {
        set_error("gbp_average_down: the arrays do not cover the coarse box / its refinement");
        return GBP_BAD_ARG;
    }
    return average_down(*fine, *crse, ratio, ncomp, crse_lo, crse_hi, static_cast<cudaStream_t>(stream));
}

int gbp_plan_time_kernel(gbp_plan* p, int which, int reps, double* ms_per_launch, double* bytes_per_launch)
{
    if (!p || !p->nodal || !ms_per_launch || !bytes_per_launch) {
        set_error("gbp_plan_time_kernel: needs a nodal plan and output pointers");
        return GBP_BAD_ARG;
    }
    return p->nodal->time_kernel(which, reps, ms_per_launch, bytes_per_launch);
}

int gbp_plan_check_level_kernels(gbp_plan* p, double diff[4])
{
    if (!p || !p->nodal || !diff) {
        set_error("gbp_plan_check_level_kernels: needs a nodal plan and an output array");
        return GBP_BAD_ARG;
    }
    return p->nodal->check_level_kernels(diff);
}

int gbp_plan_check_coarse_cycle(gbp_plan* p, double* diff)
{
    if (!p || !diff || (!p->nodal && !p->mac)) {
        set_error("gbp_plan_check_coarse_cycle: needs a nodal or MAC plan and an output");
        return GBP_BAD_ARG;
    }
    return p->nodal ? p->nodal->check_coarse_cycle(diff) : p->mac->check_coarse_cycle(diff);
}

int gbp_nodal_set_eb(gbp_plan* p, const gbp_array4* moments)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_set_eb: not a nodal plan");
        return GBP_BAD_ARG;
    }
    if (moments && moments->data && !valid_array(moments, 27)) {
        set_error("gbp_nodal_set_eb: the moments array needs 27 components");
        return GBP_BAD_ARG;
    }
    return p->nodal->set_eb((moments && moments->data) ? moments : nullptr);
}

int gbp_nodal_set_eb_inflow(gbp_plan* p, const gbp_array4* eb_vel, const gbp_array4* eb_dap,
                            const gbp_array4* eb_bcent)
{
    if (!p || !p->nodal) {
        set_error("gbp_nodal_set_eb_inflow: not a nodal plan");
        return GBP_BAD_ARG;
    }
    if (!eb_vel || !eb_vel->data) return p->nodal->set_eb_inflow(nullptr, nullptr, nullptr);
    int rc = check_cells(p, eb_vel, 3, "gbp_nodal_set_eb_inflow: eb_vel");
    if (!rc) rc = check_cells(p, eb_dap, 3, "gbp_nodal_set_eb_inflow: eb_dap");
    if (!rc) rc = check_cells(p, eb_bcent, 3, "gbp_nodal_set_eb_inflow: eb_bcent");
    if (rc) return rc;
    return p->nodal->set_eb_inflow(eb_vel, eb_dap, eb_bcent);
}

int gbp_abec_set_coeffs(gbp_plan* p, double alpha, const gbp_array4* a, double a0, double beta,
                        const gbp_array4* bx, const gbp_array4* by, const gbp_array4* bz, double b0)
{
    if (!p || !p->mac) {
        set_error("gbp_abec_set_coeffs: not a MAC plan");
        return GBP_BAD_ARG;
    }
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
    if (a && !(valid_array(a, 1) && covers(a, lo, hi))) {
        set_error("gbp_abec_set_coeffs: a must cover the cells");
        return GBP_BAD_ARG;
    }
    const gbp_array4* b[3] = {bx, by, bz};
    if (bx || by || bz)
        for (int d = 0; d < 3; ++d) {
            int fhi[3] = {hi[0], hi[1], hi[2]};
            fhi[d] += 1;
            if (!valid_array(b[d], 1) || !covers(b[d], lo, fhi)) {
                set_error("gbp_abec_set_coeffs: each b array must cover its faces 0..n");
                return GBP_BAD_ARG;
            }
        }
    return p->mac->set_abec(alpha, a, a0, beta, (bx || by || bz) ? b : nullptr, b0);
}

int gbp_abec_set_coeffs_eta(gbp_plan* p, double alpha, const gbp_array4* a, double a0, double beta,
                            const gbp_array4* eta)
{
    if (!p || !p->mac) {
        set_error("gbp_abec_set_coeffs_eta: not a MAC plan");
        return GBP_BAD_ARG;
    }
    const int lo[3] = {0, 0, 0};
    const int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
    if ((a && !(valid_array(a, 1) && covers(a, lo, hi))) || !valid_array(eta, 1) || !covers(eta, lo, hi)) {
        set_error("gbp_abec_set_coeffs_eta: a and eta must cover the cells");
        return GBP_BAD_ARG;
    }
    return p->mac->set_abec(alpha, a, a0, beta, nullptr, 0.0, eta);
}

int gbp_abec_solve(gbp_plan* p, const gbp_array4* rhs, gbp_array4* phi, gbp_stats* stats)
{
    if (!p || !p->mac) {
        set_error("gbp_abec_solve: not a MAC plan");
        return GBP_BAD_ARG;
    }
    int lo[3] = {0, 0, 0};
    int hi[3] = {p->geom.n_cell[0] - 1, p->geom.n_cell[1] - 1, p->geom.n_cell[2] - 1};
    if (!valid_array(rhs, 1) || !covers(rhs, lo, hi)) {
        set_error("gbp_abec_solve: rhs must cover the cells");
        return GBP_BAD_ARG;
    }
    for (int d = 0; d < 3; ++d) {
        if (p->bc_lo[d] == GBP_BC_DIRICHLET) lo[d] = -1;
        if (p->bc_hi[d] == GBP_BC_DIRICHLET) hi[d] += 1;
    }
    if (!valid_array(phi, 1) || !covers(phi, lo, hi)) {
        set_error("gbp_abec_solve: phi must cover the cells and one ghost layer on the Dirichlet sides");
        return GBP_BAD_ARG;
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    return p->mac->abec_solve(rhs, phi, stats);
}

struct gbp_tensor {
    gbp::TensorSolver* t = nullptr;
};

int gbp_tensor_create(const gbp_geometry* geom, const int bc_lo[9], const int bc_hi[9], const gbp_options* opt,
                      void* stream, gbp_tensor** out)
{
    if (!geom || !bc_lo || !bc_hi || !out) {
        set_error("gbp_tensor_create: geometry, boundary types and the output handle are required");
        return GBP_BAD_ARG;
    }
    *out = nullptr;
    gbp_options o;
    if (opt)
        o = *opt;
    else
        gbp_options_default(GBP_MAC, &o);
    gbp_tensor* h = new (std::nothrow) gbp_tensor;
    if (!h) return GBP_BAD_ARG;
    h->t = new (std::nothrow) gbp::TensorSolver;
    if (!h->t) {
        delete h;
        return GBP_BAD_ARG;
    }
    int rc = h->t->init(*geom, bc_lo, bc_hi, o, static_cast<cudaStream_t>(stream));
    if (rc) {
        gbp_tensor_destroy(h);
        return rc;
    }
    *out = h;
    return GBP_OK;
}

int gbp_tensor_destroy(gbp_tensor* h)
{
    if (!h) return GBP_OK;
    delete h->t;
    delete h;
    return GBP_OK;
}

int gbp_tensor_set_options(gbp_tensor* h, const gbp_options* opt)
{
    if (!h || !opt) return GBP_BAD_ARG;
    return h->t->set_options(*opt);
}

size_t gbp_tensor_device_bytes(const gbp_tensor* h) { return h ? h->t->device_bytes() : 0; }

int gbp_tensor_set_coeffs(gbp_tensor* h, double alpha, const gbp_array4* a, double a0, double beta,
                          const gbp_array4* eta_cc, const gbp_array4* eta_x, const gbp_array4* eta_y,
                          const gbp_array4* eta_z, double eta0)
{
    if (!h) {
        set_error("gbp_tensor_set_coeffs: null handle");
        return GBP_BAD_ARG;
    }
    if ((a && !valid_array(a, 1)) || (eta_cc && !valid_array(eta_cc, 1))) {
        set_error("gbp_tensor_set_coeffs: invalid a or eta array");
        return GBP_BAD_ARG;
    }
    const bool faces = eta_x && eta_y && eta_z;
    if (!eta_cc && (eta_x || eta_y || eta_z) && !(faces && valid_array(eta_x, 1) && valid_array(eta_y, 1) &&
                                                   valid_array(eta_z, 1))) {
        set_error("gbp_tensor_set_coeffs: give all three eta face arrays or none");
        return GBP_BAD_ARG;
    }
    const gbp_array4* ef[3] = {eta_x, eta_y, eta_z};
    return h->t->set_coeffs(alpha, a, a0, beta, eta_cc, (!eta_cc && faces) ? ef : nullptr, eta0);
}

int gbp_tensor_solve(gbp_tensor* h, const gbp_array4* rhs, gbp_array4* vel, gbp_stats* stats)
{
    if (!h || !rhs || !vel) {
        set_error("gbp_tensor_solve: handle, rhs and vel are required");
        return GBP_BAD_ARG;
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    return h->t->solve(*rhs, *vel, stats);
}

int gbp_tensor_apply(gbp_tensor* h, const gbp_array4* vel, gbp_array4* divtau)
{
    if (!h || !vel || !divtau) {
        set_error("gbp_tensor_apply: handle, vel and divtau are required");
        return GBP_BAD_ARG;
    }
    return h->t->apply(*vel, *divtau);
}

struct gbp_amr {
    gbp::CompositeNodal* c = nullptr;
    gbp_geometry geom{};
};

int gbp_amr_create(const gbp_geometry* coarse, const int bc_lo[3], const int bc_hi[3], const int* fine_boxes,
                   int nbox, const gbp_options* opt, void* stream, gbp_amr** amr)
{
    if (!coarse || !bc_lo || !bc_hi || !fine_boxes || nbox < 1 || !amr) {
        set_error("gbp_amr_create: geometry, boundary types, fine boxes and the output handle are required");
        return GBP_BAD_ARG;
    }
    *amr = nullptr;
    gbp_options o;
    if (opt)
        o = *opt;
    else
        gbp_options_default(GBP_NODAL, &o);
    gbp_amr* a = new (std::nothrow) gbp_amr;
    if (!a) return GBP_BAD_ARG;
    a->geom = *coarse;
    a->c = new (std::nothrow) gbp::CompositeNodal;
    if (!a->c) {
        delete a;
        return GBP_BAD_ARG;
    }
    int rc = a->c->init(*coarse, bc_lo, bc_hi, fine_boxes, nbox, o, static_cast<cudaStream_t>(stream));
    if (rc) {
        gbp_amr_destroy(a);
        return rc;
    }
    *amr = a;
    return GBP_OK;
}

int gbp_amr_destroy(gbp_amr* a)
{
    if (!a) return GBP_OK;
    delete a->c;
    delete a;
    return GBP_OK;
}

int gbp_amr_set_options(gbp_amr* a, const gbp_options* opt)
{
    if (!a || !opt) return GBP_BAD_ARG;
    return a->c->set_options(*opt);
}

size_t gbp_amr_device_bytes(const gbp_amr* a) { return a ? a->c->device_bytes() : 0; }

int gbp_amr_apply_nodal_projection(gbp_amr* a, gbp_array4* vel_c, const gbp_array4* vel_old_c,
                                   const gbp_array4* rho_c, gbp_array4* gp_c, gbp_array4* p_c,
                                   gbp_array4* const* vel_f, const gbp_array4* const* vel_old_f,
                                   const gbp_array4* const* rho_f, gbp_array4* const* gp_f, gbp_array4* const* p_f,
                                   double rho0, double scaling_factor, int incremental, gbp_stats* stats)
{
    if (!a) {
        set_error("gbp_amr_apply_nodal_projection: null handle");
        return GBP_BAD_ARG;
    }
    const int lo[3] = {0, 0, 0};
    const int hic[3] = {a->geom.n_cell[0] - 1, a->geom.n_cell[1] - 1, a->geom.n_cell[2] - 1};
    const int hin[3] = {a->geom.n_cell[0], a->geom.n_cell[1], a->geom.n_cell[2]};
    if (!valid_array(vel_c, 3) || !covers(vel_c, lo, hic) || !valid_array(gp_c, 3) || !covers(gp_c, lo, hic)) {
        set_error("gbp_amr_apply_nodal_projection: coarse vel and gp must cover the cells with 3 components");
        return GBP_BAD_ARG;
    }
    if (rho_c && !(valid_array(rho_c, 1) && covers(rho_c, lo, hic))) {
        set_error("gbp_amr_apply_nodal_projection: coarse rho must cover the cells");
        return GBP_BAD_ARG;
    }
    if (p_c && p_c->data && !(valid_array(p_c, 1) && covers(p_c, lo, hin))) {
        set_error("gbp_amr_apply_nodal_projection: coarse p_nd must cover the nodes");
        return GBP_BAD_ARG;
    }
    if ((rho_c == nullptr) != (rho_f == nullptr)) {
        set_error("gbp_amr_apply_nodal_projection: rho must be given on both levels or on neither");
        return GBP_BAD_ARG;
    }
    if (incremental && ((vel_old_c == nullptr) != (vel_old_f == nullptr))) {
        set_error("gbp_amr_apply_nodal_projection: vel_old must be given on both levels or on neither");
        return GBP_BAD_ARG;
    }
    if (vel_old_c && !(valid_array(vel_old_c, 3) && covers(vel_old_c, lo, hic))) {
        set_error("gbp_amr_apply_nodal_projection: coarse vel_old must cover the cells with 3 components");
        return GBP_BAD_ARG;
    }
    gbp::AmrFields f{};
    f.vel_c = vel_c;
    f.vel_old_c = incremental ? vel_old_c : nullptr;
    f.rho_c = rho_c;
    f.gp_c = gp_c;
    f.p_c = (p_c && p_c->data) ? p_c : nullptr;
    f.vel_f = vel_f;
    f.vel_old_f = incremental ? vel_old_f : nullptr;
    f.rho_f = rho_f;
    f.gp_f = gp_f;
    f.p_f = p_f;
    f.rho0 = rho0;
    f.scale = scaling_factor;
    f.incremental = incremental;
    return a->c->project(f, stats);
}

int gbp_apply_nodal_projection_host(gbp_plan* p, double* vel, const double* rho, double rho0, double* gp,
                                    double* p_nd, double scaling_factor, int incremental, gbp_stats* stats)
{
    if (!p || !p->nodal || !vel || !gp) {
        set_error("gbp_apply_nodal_projection_host: nodal plan, vel and gp are required");
        return GBP_BAD_ARG;
    }
    const int nx = p->geom.n_cell[0], ny = p->geom.n_cell[1], nz = p->geom.n_cell[2];
    const size_t nc = (size_t)nx * ny * nz;
    const size_t nn = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    const size_t need = (3 * nc + (rho ? nc : 0) + 3 * nc + (p_nd ? nn : 0)) * sizeof(double);
    if (p->hbuf_bytes < need) {
        if (p->hbuf) cudaFree(p->hbuf);
        p->hbuf = nullptr;
        p->hbuf_bytes = 0;
        GBP_CUDA(cudaMalloc(&p->hbuf, need));
        p->hbuf_bytes = need;
    }
    if (!p->copy_stream) {
        GBP_CUDA(cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
        GBP_CUDA(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming));
        GBP_CUDA(cudaEventCreateWithFlags(&p->ev_phi, cudaEventDisableTiming));
        GBP_CUDA(cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming));
    }
    double* dvel = p->hbuf;
    double* dgp = dvel + 3 * nc;
    double* drho = dgp + 3 * nc;
    double* dp = drho + (rho ? nc : 0);
    const cudaStream_t s = p->stream, c = p->copy_stream;
    // the copy stream starts after the work already queued on the plan's stream (earlier users of
    // the staging buffers)
    GBP_CUDA(cudaEventRecord(p->ev_out, s));
    GBP_CUDA(cudaStreamWaitEvent(c, p->ev_out, 0));
    // density first on the plan's stream (sigma and its edge weights are computed from it while the
    // velocities and gp upload on the copy stream)
    if (rho) GBP_CUDA(cudaMemcpyAsync(drho, rho, nc * sizeof(double), cudaMemcpyHostToDevice, s));
    // velocity and gp by z-slabs matched to the right-hand side's z chunks: each group of chunks starts
    // as soon as the cells it reads have arrived (not with a p_nd to upload: the incremental form)
    const bool grouped = !(p_nd && incremental) && !p->nodal->has_eb();
    gbp::RhsGroups rg{};
    if (grouped) {
        if (!p->ev_rhs[0])
            for (auto& e : p->ev_rhs) GBP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        int kc = 1;
        const int nzc = gbp::nodal_rhs_zchunks(p->nodal->geom0(), &kc);
        rg.n = std::min(gbp::kRhsGroups, nzc);
        const size_t plane = (size_t)nx * ny;
        int cs = 0;
        for (int q = 0; q < rg.n; ++q) {
            rg.zb[q] = (int)((long long)nzc * q / rg.n);
            rg.zb[q + 1] = (int)((long long)nzc * (q + 1) / rg.n);
            const int ce = q == rg.n - 1 ? nz : std::min(nz, rg.zb[q + 1] * kc);
            if (ce > cs)
                for (int comp = 0; comp < 3; ++comp) {
                    const size_t off = comp * nc + (size_t)cs * plane, cnt = (size_t)(ce - cs) * plane;
                    GBP_CUDA(cudaMemcpyAsync(dvel + off, vel + off, cnt * sizeof(double), cudaMemcpyHostToDevice, c));
                    GBP_CUDA(cudaMemcpyAsync(dgp + off, gp + off, cnt * sizeof(double), cudaMemcpyHostToDevice, c));
                }
            cs = std::max(cs, ce);
            rg.ev[q] = p->ev_rhs[q];
            GBP_CUDA(cudaEventRecord(rg.ev[q], c));
        }
    } else {
        GBP_CUDA(cudaMemcpyAsync(dvel, vel, 3 * nc * sizeof(double), cudaMemcpyHostToDevice, c));
        GBP_CUDA(cudaMemcpyAsync(dgp, gp, 3 * nc * sizeof(double), cudaMemcpyHostToDevice, c));
    }
    if (p_nd && incremental) GBP_CUDA(cudaMemcpyAsync(dp, p_nd, nn * sizeof(double), cudaMemcpyHostToDevice, c));
    GBP_CUDA(cudaEventRecord(p->ev_in, c));
    auto cells = [&](double* d, int nc_) {
        gbp_array4 a{};
        a.data = d;
        a.hi[0] = nx - 1;
        a.hi[1] = ny - 1;
        a.hi[2] = nz - 1;
        a.ncomp = nc_;
        a.jstride = nx;
        a.kstride = (long long)nx * ny;
        a.nstride = (long long)nx * ny * nz;
        return a;
    };
    gbp_array4 av = cells(dvel, 3), ag = cells(dgp, 3), ar = cells(drho, 1);
    gbp_array4 ap{};
    ap.data = dp;
    ap.hi[0] = nx;
    ap.hi[1] = ny;
    ap.hi[2] = nz;
    ap.ncomp = 1;
    ap.jstride = nx + 1;
    ap.kstride = (long long)(nx + 1) * (ny + 1);
    ap.nstride = (long long)nn;
    // p_nd goes back on the copy stream as soon as it is stored, then the velocity and gp slab by slab
    // while the correction of the next slab runs
    gbp::HostCopy pc{p_nd, dp, nn * sizeof(double), c, p->ev_phi};
    if (!p->ev_slab[0])
        for (auto& e : p->ev_slab) GBP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const int nslabs = std::min(kHostSlabs, std::max(1, nz / 16));
    gbp::HostSlabs os{vel, gp, dvel, dgp, (size_t)nx * ny, nc, nslabs, c, p->ev_slab};
    int rc = apply_nodal_impl(p, &av, nullptr, rho ? &ar : nullptr, rho0, &ag, p_nd ? &ap : nullptr, 0.0, 1.0, 1.0,
                              scaling_factor, incremental, 0, stats, grouped ? nullptr : p->ev_in,
                              p_nd ? &pc : nullptr, &os, grouped ? &rg : nullptr);
    if (rc != GBP_OK && rc != GBP_NOT_CONVERGED) {
        cudaStreamSynchronize(c);
        return rc;
    }
    GBP_CUDA(cudaStreamSynchronize(s));
    GBP_CUDA(cudaStreamSynchronize(c));
    return rc;
}

}  // extern "C"
