// Header-only C++ shim over the C ABI of incflo_gb300.h with the method names of the AMReX-Hydro
// projectors that incflo drives, so incflo's call sites change by a type swap:
//
//   Hydro::NodalProjector  (used in src/projection/incflo_apply_nodal_projection.cpp:181-219)
//   Hydro::MacProjector    (used in src/convection/incflo_compute_MAC_projected_velocities.cpp:93-299)
//
// One box per level: an AMReX MultiFab FAB converts to gbp_array4 with gb::view() (its data
// pointer, its box including ghost cells, and its strides), with zero copies. Errors throw
// gb::Error carrying the gbp_status code (the reference aborts instead).
#pragma once

#include <stdexcept>
#include <string>
#include <utility>

#include "incflo_gb300.h"

namespace gb {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& where)
        : std::runtime_error(where + ": " + gbp_status_string(s) + " (" + gbp_last_error() + ")"), status(s)
    {
    }
};

inline void check(int s, const char* where)
{
    if (s != GBP_OK) throw Error(s, where);
}

// Array4-like view: data, inclusive index bounds of the allocation (ghost cells included),
// contiguous x, jstride / kstride / nstride in elements.
inline gbp_array4 view(double* data, const int lo[3], const int hi[3], int ncomp = 1)
{
    gbp_array4 a{};
    a.data = data;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = lo[d];
        a.hi[d] = hi[d];
    }
    a.ncomp = ncomp;
    a.jstride = (long long)(hi[0] - lo[0] + 1);
    a.kstride = a.jstride * (long long)(hi[1] - lo[1] + 1);
    a.nstride = a.kstride * (long long)(hi[2] - lo[2] + 1);
    return a;
}

struct Geometry {
    int n_cell[3];
    double prob_lo[3];
    double prob_hi[3];
    gbp_geometry c() const
    {
        gbp_geometry g{};
        for (int d = 0; d < 3; ++d) {
            g.n_cell[d] = n_cell[d];
            g.prob_lo[d] = prob_lo[d];
            g.prob_hi[d] = prob_hi[d];
        }
        return g;
    }
};

struct LPInfo {
    int max_coarsening_level = 100;
    LPInfo& setMaxCoarseningLevel(int n)
    {
        max_coarsening_level = n;
        return *this;
    }
};

class Plan {
public:
    Plan() = default;
    Plan(const Plan&) = delete;
    Plan& operator=(const Plan&) = delete;
    Plan(Plan&& o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
    ~Plan() { gbp_plan_destroy(p_); }
    void create(const Geometry& geom, int kind, const int lo[3], const int hi[3], const gbp_options& opt, void* stream)
    {
        gbp_plan_destroy(p_);
        p_ = nullptr;
        const gbp_geometry g = geom.c();
        check(gbp_plan_create(&g, kind, lo, hi, &opt, stream, &p_), "gbp_plan_create");
    }
    gbp_plan* get() const { return p_; }
    explicit operator bool() const { return p_ != nullptr; }

private:
    gbp_plan* p_ = nullptr;
};

// Hydro::NodalProjector(vel, sigma, geom, info): setDomainBC, project(rtol, atol), getPhi, getGradPhi.
// Unlike the reference, the plan (multigrid hierarchy) survives across projections: keep the
// projector alive and call setVelocity / setSigma before each project.
class NodalProjector {
public:
    NodalProjector(gbp_array4 vel, gbp_array4 sigma, const Geometry& geom, LPInfo info = {}, void* stream = nullptr,
                   const char* inputs = nullptr)
        : vel_(vel), sigma_(sigma), have_sigma_(true), geom_(geom), stream_(stream)
    {
        init(info, inputs);
    }
    NodalProjector(gbp_array4 vel, double sigma, const Geometry& geom, LPInfo info = {}, void* stream = nullptr,
                   const char* inputs = nullptr)
        : vel_(vel), const_sigma_(sigma), geom_(geom), stream_(stream)
    {
        init(info, inputs);
    }

    void setDomainBC(const int lo[3], const int hi[3])
    {
        plan_.create(geom_, GBP_NODAL, lo, hi, opt_, stream_);
    }
    void setVelocity(gbp_array4 vel) { vel_ = vel; }
    void setSigma(gbp_array4 sigma)
    {
        sigma_ = sigma;
        have_sigma_ = true;
    }
    // output storage of getPhi() / getGradPhi(): nodal phi, 3-component cell gradient
    void setOutputs(gbp_array4 phi, gbp_array4 gradphi)
    {
        phi_ = phi;
        gradphi_ = gradphi;
    }
    // getLinOp().setOversetMask(lev, mask): 0 = phi held at 0 (incflo::make_nodalBC_mask)
    void setOversetMask(gbp_iarray4 mask)
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "NodalProjector::setOversetMask before setDomainBC");
        check(gbp_nodal_set_overset_mask(plan_.get(), &mask), "gbp_nodal_set_overset_mask");
    }

    // the EB factory's volume moments of the level (27 components; gbp_nodal_set_eb)
    void setEB(const gbp_array4& moments)
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "NodalProjector::setEB before setDomainBC");
        check(gbp_nodal_set_eb(plan_.get(), &moments), "gbp_nodal_set_eb");
    }
    // getLinOp().setEBInflowVelocity(lev, eb_vel), with the EB factory's boundary area vector (area
    // fraction differences) and boundary centroid of the level, 3 components each
    void setEBInflowVelocity(int lev, const gbp_array4& eb_vel, const gbp_array4& eb_dap, const gbp_array4& eb_bcent)
    {
        if (lev != 0) throw Error(GBP_BAD_ARG, "NodalProjector::setEBInflowVelocity: single level");
        if (!plan_) throw Error(GBP_BAD_ARG, "NodalProjector::setEBInflowVelocity before setDomainBC");
        check(gbp_nodal_set_eb_inflow(plan_.get(), &eb_vel, &eb_dap, &eb_bcent), "gbp_nodal_set_eb_inflow");
    }

    gbp_stats project(double rtol, double atol)
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "NodalProjector::project before setDomainBC");
        opt_.rtol = rtol;
        opt_.atol = atol;
        check(gbp_plan_set_options(plan_.get(), &opt_), "gbp_plan_set_options");
        check(gbp_nodal_set_sigma(plan_.get(), have_sigma_ ? &sigma_ : nullptr, const_sigma_), "gbp_nodal_set_sigma");
        gbp_stats st{};
        check(gbp_nodal_project(plan_.get(), &vel_, phi_.data ? &phi_ : nullptr, gradphi_.data ? &gradphi_ : nullptr, 0,
                                &st),
              "gbp_nodal_project");
        return st;
    }
    const gbp_array4& getPhi() const { return phi_; }
    const gbp_array4& getGradPhi() const { return gradphi_; }
    gbp_options& options() { return opt_; }
    gbp_plan* plan() const { return plan_.get(); }

private:
    void init(const LPInfo& info, const char* inputs)
    {
        check(gbp_options_default(GBP_NODAL, &opt_), "gbp_options_default");
        if (inputs) check(gbp_options_parse(&opt_, "nodal_proj", inputs), "gbp_options_parse(nodal_proj)");
        opt_.max_coarsening_level = info.max_coarsening_level;
    }
    gbp_array4 vel_{}, sigma_{}, phi_{}, gradphi_{};
    double const_sigma_ = 0.0;
    bool have_sigma_ = false;
    Geometry geom_;
    void* stream_;
    gbp_options opt_{};
    Plan plan_;
};

// Hydro::MacProjector(geom): needInitialization, initProjector(info, beta) / initProjector(info, beta0),
// setDomainBC, updateBeta / updateCoeffs, setUMAC, project(rtol, atol), project(phi, rtol, atol).
class MacProjector {
public:
    explicit MacProjector(const Geometry& geom, void* stream = nullptr, const char* inputs = nullptr)
        : geom_(geom), stream_(stream)
    {
        check(gbp_options_default(GBP_MAC, &opt_), "gbp_options_default");
        if (inputs) check(gbp_options_parse(&opt_, "mac_proj", inputs), "gbp_options_parse(mac_proj)");
    }
    bool needInitialization() const { return !plan_; }
    void initProjector(const LPInfo& info, const gbp_array4 beta[3])
    {
        opt_.max_coarsening_level = info.max_coarsening_level;
        for (int d = 0; d < 3; ++d) beta_[d] = beta[d];
        have_beta_ = true;
    }
    void initProjector(const LPInfo& info, double beta)
    {
        opt_.max_coarsening_level = info.max_coarsening_level;
        const_beta_ = beta;
        have_beta_ = false;
    }
    void setDomainBC(const int lo[3], const int hi[3])
    {
        plan_.create(geom_, GBP_MAC, lo, hi, opt_, stream_);
        push_beta();
    }
    void updateBeta(double beta)
    {
        const_beta_ = beta;
        have_beta_ = false;
        push_beta();
    }
    void updateCoeffs(const gbp_array4 beta[3])
    {
        for (int d = 0; d < 3; ++d) beta_[d] = beta[d];
        have_beta_ = true;
        push_beta();
    }
    void setUMAC(const gbp_array4 umac[3])
    {
        for (int d = 0; d < 3; ++d) umac_[d] = umac[d];
    }
    // setLevelBC(lev, nullptr, robin_a, robin_b, robin_f) for the Robin sides (f = 0)
    void setLevelBC(int lev, const gbp_array4* levelbcdata, const gbp_array4* robin_a, const gbp_array4* robin_b,
                    const gbp_array4* robin_f)
    {
        if (lev != 0 || levelbcdata) throw Error(GBP_BAD_ARG, "MacProjector::setLevelBC: single level, zero Dirichlet");
        if (!plan_) throw Error(GBP_BAD_ARG, "MacProjector::setLevelBC before setDomainBC");
        check(gbp_mac_set_robin(plan_.get(), robin_a, robin_b, robin_f), "gbp_mac_set_robin");
    }
    // the EB factory's volume fractions, area fractions and face centroids (what the reference's
    // MacProjector reads from the factory of its MultiFabs); beta is pushed again afterwards
    void setEB(const gbp_array4& vfrac, const gbp_array4 area[3], const gbp_array4 fcent[3])
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "MacProjector::setEB before setDomainBC");
        check(gbp_mac_set_eb(plan_.get(), &vfrac, &area[0], &area[1], &area[2], &fcent[0], &fcent[1], &fcent[2]),
              "gbp_mac_set_eb");
        push_beta();
    }
    // setEBInflowVelocity(lev, eb_vel): the velocity on the embedded boundary (3 components)
    void setEBInflowVelocity(int lev, const gbp_array4& eb_vel)
    {
        if (lev != 0) throw Error(GBP_BAD_ARG, "MacProjector::setEBInflowVelocity: single level");
        if (!plan_) throw Error(GBP_BAD_ARG, "MacProjector::setEBInflowVelocity before setDomainBC");
        check(gbp_mac_set_eb_inflow(plan_.get(), &eb_vel), "gbp_mac_set_eb_inflow");
    }
    gbp_stats project(double rtol, double atol) { return run(nullptr, rtol, atol); }
    gbp_stats project(gbp_array4 phi, double rtol, double atol) { return run(&phi, rtol, atol); }
    // MacProjector::getFluxes(fluxes, phi, loc): fluxes[d] = -beta grad phi on the faces (face centroids
    // of cut faces), the correction project() applied to umac
    void getFluxes(gbp_array4 fluxes[3], const gbp_array4& phi)
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "MacProjector::getFluxes before setDomainBC");
        check(gbp_mac_get_fluxes(plan_.get(), &phi, &fluxes[0], &fluxes[1], &fluxes[2]), "gbp_mac_get_fluxes");
    }
    gbp_options& options() { return opt_; }

private:
    void push_beta()
    {
        if (!plan_) return;
        if (have_beta_)
            check(gbp_mac_set_beta(plan_.get(), &beta_[0], &beta_[1], &beta_[2], 0.0), "gbp_mac_set_beta");
        else
            check(gbp_mac_set_beta(plan_.get(), nullptr, nullptr, nullptr, const_beta_), "gbp_mac_set_beta");
    }
    gbp_stats run(gbp_array4* phi, double rtol, double atol)
    {
        if (!plan_) throw Error(GBP_BAD_ARG, "MacProjector::project before setDomainBC");
        opt_.rtol = rtol;
        opt_.atol = atol;
        check(gbp_plan_set_options(plan_.get(), &opt_), "gbp_plan_set_options");
        gbp_stats st{};
        check(gbp_mac_project(plan_.get(), &umac_[0], &umac_[1], &umac_[2], phi, phi != nullptr, &st), "gbp_mac_project");
        return st;
    }
    Geometry geom_;
    void* stream_;
    gbp_options opt_{};
    gbp_array4 beta_[3]{}, umac_[3]{};
    double const_beta_ = 0.0;
    bool have_beta_ = false;
    Plan plan_;
};

}  // namespace gb
