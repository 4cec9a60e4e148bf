// C++ mirror of the reference's Integrator interface over the C ABI.
//
// A maintainer of the C++ reference would swap
//   std::make_shared<CentralDifference>(mesh, dt, mtol, ktol, ftol)
// (RP/12-Utilities/Driver.hpp:1818-1820) for svl::gpu::CentralDifference built
// from the same partition arrays.  Method names and meanings follow
// RP/10-Integrators/Integrator.hpp:53-144: ComputeNewStep returns `stop`
// (true = failure), state getters return total-dof vectors.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/svl_gb300.h"

namespace svl {
namespace gpu {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
    int code;
};

inline void check(int st) {
    if (st != SVL_OK) throw Error(st, svl_last_error());
}

// The force entries of a load descriptor (point, body-point and element body
// loads resolved to dofs), kept by the integrators for ComputeProgressiveForce.
class ExternalForce {
public:
    ExternalForce() = default;
    explicit ExternalForce(const svl_load_desc& L) {
        if (L.ndrm > 0) drm_ = true;
        if (L.nseries > 0 && L.series_ptr && L.series_val) {
            ptr_.assign(L.series_ptr, L.series_ptr + L.nseries + 1);
            val_.assign(L.series_val, L.series_val + ptr_.back());
        }
        if (L.nforce > 0) {
            dof_.assign(L.force_dof, L.force_dof + L.nforce);
            ser_.assign(L.force_series, L.force_series + L.nforce);
            coef_.assign(L.force_coef, L.force_coef + L.nforce);
        }
    }
    // Fext(k) on ntotal dofs: sum of coef * series[k], a series read past its
    // end giving 0 (Assembler::ComputeExternalForceVector, Assembler.cpp:291-489).
    std::vector<double> at(unsigned k, int ntotal) const {
        if (drm_) throw Error(SVL_ERR_UNSUPPORTED, "domain-reduction forces are computed on the device only");
        std::vector<double> f((size_t)ntotal, 0.0);
        for (size_t i = 0; i < dof_.size(); ++i) {
            const int s = ser_[i], b = ptr_[s], n = ptr_[s + 1] - b;
            if ((int)k < n) f[dof_[i]] += coef_[i] * val_[b + k];
        }
        return f;
    }

private:
    std::vector<int32_t> ptr_, dof_, ser_;
    std::vector<double> val_, coef_;
    bool drm_ = false;
};

class CentralDifference {
public:
    // CentralDifference(mesh, dt, mtol, ktol, ftol) (CentralDifference.cpp:6-27)
    // A model with PML2DQuad4 / PML3DHexa8 layers goes to the PML-capable
    // handle in its explicit mode (the library's staggered explicit PML scheme:
    // the reference's CentralDifference has no consistent explicit PML, it
    // never applies G, CentralDifference.cpp:114-120).
    CentralDifference(const svl_model_desc& model, const svl_load_desc& loads, double dt,
                      double mtol = 1e-12, double ftol = 1e-12)
        : ntotal_(model.ntotal), fext_(loads) {
        bool pml = false;
        for (int e = 0; model.elem_pml && e < model.nelem; ++e) pml = pml || model.elem_pml[e] != 0;
        if (pml) {
            svl_xnm_opts x{};
            x.dt = dt; x.ftol = ftol; x.mtol = mtol; x.tol = 1e-10; x.maxit = 100000;
            x.algorithm = SVL_ALGO_LINEAR;
            x.integrator = SVL_XNM_CENTRAL_DIFFERENCE;
            check(svl_xnm_create(&model, &loads, &x, &x_));
            return;
        }
        // K = M/dt^2 + C/2dt not diagonal (consistent mass or ak != 0,
        // CentralDifference.cpp:64-70): a PCG solve of K every step
        bool nondiag = !model.lumped;
        for (int e = 0; model.elem_rayleigh && e < model.nelem; ++e) nondiag = nondiag || model.elem_rayleigh[2 * e + 1] != 0.0;
        if (nondiag) {
            svl_nm_opts n{};
            n.dt = dt; n.ftol = ftol; n.mtol = mtol; n.pcg_tol = 1e-12; n.pcg_maxit = 20000;
            n.precond = SVL_PRECOND_JACOBI; n.algorithm = SVL_ALGO_LINEAR;
            n.integrator = SVL_NM_CENTRAL_DIFFERENCE;
            check(svl_nm_create(&model, &loads, &n, &n_));
            return;
        }
        svl_cd_opts o{};
        o.dt = dt;
        o.mtol = mtol;
        o.ftol = ftol;
        o.precision = SVL_PREC_FP64;
        o.check_every = 1;
        check(svl_cd_create(&model, &loads, &o, &h_));
    }
    ~CentralDifference() {
        if (h_) svl_cd_destroy(h_);
        if (x_) svl_xnm_destroy(x_);
        if (n_) svl_nm_destroy(n_);
    }
    CentralDifference(const CentralDifference&) = delete;
    CentralDifference& operator=(const CentralDifference&) = delete;

    // Initialize(mesh): initial conditions from the nodes (CentralDifference.cpp:36-71)
    void Initialize(const double* U0 = nullptr, const double* V0 = nullptr, const double* A0 = nullptr) {
        check(x_ ? svl_xnm_set_initial(x_, U0, V0, A0, nullptr)
                 : n_ ? svl_nm_set_initial(n_, U0, V0, A0) : svl_cd_set_initial(h_, U0, V0, A0));
    }
    // ComputeNewStep(mesh, k) -> stop (CentralDifference.cpp:124-151)
    bool ComputeNewStep(unsigned int k) { return ComputeNewSteps(k, 1); }
    // Many steps in one call, optional displacement history [n][ntotal].
    bool ComputeNewSteps(unsigned int k_first, unsigned int n, double* U_hist = nullptr) {
        const int st = x_ ? svl_xnm_run(x_, (int32_t)k_first, (int32_t)n, U_hist)
                       : n_ ? svl_nm_run(n_, (int32_t)k_first, (int32_t)n, U_hist)
                            : svl_cd_run(h_, (int32_t)k_first, (int32_t)n, U_hist);
        return st != SVL_OK;
    }
    std::vector<double> GetDisplacements() const { return get(0); }
    std::vector<double> GetVelocities() const { return get(1); }
    std::vector<double> GetAccelerations() const { return get(2); }
    // ComputeProgressiveForce(mesh, k) (CentralDifference.cpp:174-186 and the
    // Newmark integrators): Fext(k) + Fbar, Fbar = 0 in a single-stage run
    std::vector<double> ComputeProgressiveForce(unsigned int k) const { return fext_.at(k, ntotal_); }
    // ComputeReactionForce(mesh, k) after step k (CentralDifference.cpp:156-171),
    // as DynamicAnalysis::UpdateDomain stores it at the fixed nodes
    std::vector<double> ComputeReactionForce(unsigned int k) const {
        if (x_) throw Error(SVL_ERR_UNSUPPORTED, "reactions are not covered for PML models");
        std::vector<double> r(ntotal_);
        check(n_ ? svl_nm_reaction(n_, (int32_t)k, r.data()) : svl_cd_reaction(h_, (int32_t)k, r.data()));
        return r;
    }

private:
    std::vector<double> get(int which) const {
        std::vector<double> v(ntotal_);
        check(x_ ? svl_xnm_get(x_, which, v.data()) : n_ ? svl_nm_get(n_, which, v.data()) : svl_cd_get(h_, which, v.data()));
        return v;
    }
    svl_cd* h_ = nullptr;
    svl_xnm* x_ = nullptr;                 // set instead of h_ for models with PML layers
    svl_nm* n_ = nullptr;                  // set instead of h_ when K is not diagonal
    int ntotal_ = 0;
    ExternalForce fext_;
};

// NewtonRaphson(solver, mesh, cnvgtol, nstep, cnvgtest) as the Driver builds it
// (RP/12-Utilities/Driver.hpp:1791-1795); integrators given none use Linear.
struct NewtonRaphson {
    double cnvgtol = 1e-6;
    int nstep = 50;
    int cnvgtest = 4;
};

// NewmarkBeta(mesh, dt, mtol, ktol, ftol) with the Linear algorithm and an
// iterative LinearSystem (RP/10-Integrators/03-Newmark/NewmarkBeta.cpp:6-141,
// RP/11-Solvers/02-Iterative/PetscSolver.cc:16-150): the effective-stiffness
// solve is matrix-free Jacobi-PCG on the GPU to a true relative residual of
// `tol`, optionally with the learned preconditioner (TrainPreconditioner).
class NewmarkBeta {
public:
    NewmarkBeta(const svl_model_desc& model, const svl_load_desc& loads, double dt, double tol = 1e-8,
                double mtol = 1e-12, double ftol = 1e-12, int maxit = 20000, const NewtonRaphson* newton = nullptr)
        : ntotal_(model.ntotal), fext_(loads) {
        bool pml = false;
        for (int e = 0; model.elem_pml && e < model.nelem; ++e) pml = pml || model.elem_pml[e] != 0;
        if (pml) {
            // PML layers: symmetric indefinite Keff, the MINRES handle in NewmarkBeta mode
            svl_xnm_opts x{};
            x.dt = dt; x.ftol = ftol; x.mtol = mtol; x.tol = tol; x.maxit = maxit;
            x.algorithm = newton ? SVL_ALGO_NEWTON : SVL_ALGO_LINEAR;
            if (newton) { x.newton_maxit = newton->nstep; x.cnvgtol = newton->cnvgtol; x.cnvgtest = newton->cnvgtest; }
            x.integrator = SVL_XNM_NEWMARK;
            x.single_inner = 1;
            check(svl_xnm_create(&model, &loads, &x, &x_));
            return;
        }
        svl_nm_opts o{};
        o.dt = dt;
        o.ftol = ftol;
        o.mtol = mtol;
        o.pcg_tol = tol;
        o.pcg_maxit = maxit;
        o.precond = SVL_PRECOND_JACOBI;
        o.single_inner = 1;                // FP32 operator in the inner iterations where the model allows it
        o.algorithm = SVL_ALGO_LINEAR;
        if (newton) {
            o.algorithm = SVL_ALGO_NEWTON;
            o.maxit = newton->nstep;
            o.cnvgtol = newton->cnvgtol;
            o.cnvgtest = newton->cnvgtest;
        }
        check(svl_nm_create(&model, &loads, &o, &h_));
    }
    ~NewmarkBeta() {
        if (h_) svl_nm_destroy(h_);
        if (x_) svl_xnm_destroy(x_);
    }
    NewmarkBeta(const NewmarkBeta&) = delete;
    NewmarkBeta& operator=(const NewmarkBeta&) = delete;

    void Initialize(const double* U0 = nullptr, const double* V0 = nullptr, const double* A0 = nullptr) {
        check(x_ ? svl_xnm_set_initial(x_, U0, V0, A0, nullptr) : svl_nm_set_initial(h_, U0, V0, A0));
    }
    // ComputeNewStep(mesh, k) -> stop (NewmarkBeta.cpp:117-141)
    bool ComputeNewStep(unsigned int k) { return ComputeNewSteps(k, 1); }
    bool ComputeNewSteps(unsigned int k_first, unsigned int n, double* U_hist = nullptr) {
        const int st = x_ ? svl_xnm_run(x_, (int32_t)k_first, (int32_t)n, U_hist)
                          : svl_nm_run(h_, (int32_t)k_first, (int32_t)n, U_hist);
        return st != SVL_OK;
    }
    // Trains the learned preconditioner on synthetic pairs of this model's
    // effective stiffness and switches to it (lattice meshes without PML only).
    float TrainPreconditioner(unsigned int k_next) {
        if (x_) throw Error(SVL_ERR_UNSUPPORTED, "the learned preconditioner does not cover PML models");
        svl_nn_train_opts t{};
        t.n_synthetic = 300;
        t.iters = 1500;
        t.batch = 8;
        t.lr = 2e-3f;
        float loss = 0.f;
        check(svl_nm_train_preconditioner(h_, (int32_t)k_next, &t, &loss));
        return loss;
    }
    std::vector<double> GetDisplacements() const { return get(0); }
    std::vector<double> GetVelocities() const { return get(1); }
    std::vector<double> GetAccelerations() const { return get(2); }
    // ComputeProgressiveForce(mesh, k) (CentralDifference.cpp:174-186 and the
    // Newmark integrators): Fext(k) + Fbar, Fbar = 0 in a single-stage run
    std::vector<double> ComputeProgressiveForce(unsigned int k) const { return fext_.at(k, ntotal_); }
    // NewmarkBeta::ComputeReactionForce after step k
    std::vector<double> ComputeReactionForce(unsigned int k) const {
        std::vector<double> r(ntotal_);
        check(x_ ? svl_xnm_reaction(x_, (int32_t)k, r.data()) : svl_nm_reaction(h_, (int32_t)k, r.data()));
        return r;
    }

private:
    std::vector<double> get(int which) const {
        std::vector<double> v(ntotal_);
        check(x_ ? svl_xnm_get(x_, which, v.data()) : svl_nm_get(h_, which, v.data()));
        return v;
    }
    svl_nm* h_ = nullptr;
    svl_xnm* x_ = nullptr;                 // set instead of h_ for models with PML layers
    int ntotal_ = 0;
    ExternalForce fext_;
};

// ExtendedNewmarkBeta(mesh, dt, mtol, ktol, ftol) with the Linear algorithm or
// NewtonRaphson (RP/10-Integrators/03-Newmark/ExtendedNewmarkBeta.cpp:37-245)
// for meshes with PML2DQuad4 / PML3DHexa8 layers and elastic or J2 solids: the
// effective-stiffness solve is matrix-free MINRES on the GPU to a relative
// residual `tol` (|diag|^-1 norm).
class ExtendedNewmarkBeta {
public:
    ExtendedNewmarkBeta(const svl_model_desc& model, const svl_load_desc& loads, double dt, double tol = 1e-10,
                        double mtol = 1e-12, double ftol = 1e-12, int maxit = 100000,
                        const NewtonRaphson* newton = nullptr)
        : ntotal_(model.ntotal), fext_(loads) {
        svl_xnm_opts o{};
        o.dt = dt;
        o.ftol = ftol;
        o.mtol = mtol;
        o.tol = tol;
        o.maxit = maxit;
        o.algorithm = SVL_ALGO_LINEAR;
        if (newton) {
            o.algorithm = SVL_ALGO_NEWTON;
            o.newton_maxit = newton->nstep;
            o.cnvgtol = newton->cnvgtol;
            o.cnvgtest = newton->cnvgtest;
        }
        o.integrator = SVL_XNM_EXTENDED_NEWMARK;
        o.single_inner = 1;
        check(svl_xnm_create(&model, &loads, &o, &h_));
    }
    ~ExtendedNewmarkBeta() { svl_xnm_destroy(h_); }
    ExtendedNewmarkBeta(const ExtendedNewmarkBeta&) = delete;
    ExtendedNewmarkBeta& operator=(const ExtendedNewmarkBeta&) = delete;

    // Initialize(mesh): U, V, A and the PML history Ubar from the nodes (:37-71)
    void Initialize(const double* U0 = nullptr, const double* V0 = nullptr, const double* A0 = nullptr,
                    const double* Ubar0 = nullptr) {
        check(svl_xnm_set_initial(h_, U0, V0, A0, Ubar0));
    }
    // ComputeNewStep(mesh, k) -> stop (:123-153)
    bool ComputeNewStep(unsigned int k) { return svl_xnm_run(h_, (int32_t)k, 1, nullptr) != SVL_OK; }
    bool ComputeNewSteps(unsigned int k_first, unsigned int n, double* U_hist = nullptr) {
        return svl_xnm_run(h_, (int32_t)k_first, (int32_t)n, U_hist) != SVL_OK;
    }
    std::vector<double> GetDisplacements() const { return get(0); }
    std::vector<double> GetVelocities() const { return get(1); }
    std::vector<double> GetAccelerations() const { return get(2); }
    // ComputeProgressiveForce(mesh, k) (CentralDifference.cpp:174-186 and the
    // Newmark integrators): Fext(k) + Fbar, Fbar = 0 in a single-stage run
    std::vector<double> ComputeProgressiveForce(unsigned int k) const { return fext_.at(k, ntotal_); }
    std::vector<double> GetPMLHistoryVector() const { return get(3); }
    // ComputeReactionForce(mesh, k) after step k (:158-172), as
    // DynamicAnalysis::UpdateDomain stores it at the fixed nodes
    std::vector<double> ComputeReactionForce(unsigned int k) const {
        std::vector<double> r(ntotal_);
        check(svl_xnm_reaction(h_, (int32_t)k, r.data()));
        return r;
    }

private:
    std::vector<double> get(int which) const {
        std::vector<double> v(ntotal_);
        check(svl_xnm_get(h_, which, v.data()));
        return v;
    }
    svl_xnm* h_ = nullptr;
    int ntotal_ = 0;
    ExternalForce fext_;
};

}  // namespace gpu
}  // namespace svl
