// Builds a small Q4 box with the grid generator and steps it through the
// C++ Integrator mirror.  Prints "nodevice" without a GPU, otherwise the
// peak |U| after 100 steps.
#include <cmath>
#include <cstdio>
#include <vector>

#include "svl_gb300/host/svl_integrators.hpp"

int main() {
    svl_grid_spec g{};
    g.ndim = 2; g.ne[0] = 20; g.ne[1] = 10; g.h[0] = g.h[1] = 1.0;
    g.fix_mask[0] = 1; g.fix_mask[1] = 1; g.fix_mask[2] = 3;
    int32_t nn, ne, nt, nf, nc;
    svl::gpu::check(svl_grid_sizes(&g, &nn, &ne, &nt, &nf, &nc));
    std::vector<double> X(nn * 2);
    std::vector<int32_t> td(nn * 2), fd(nn * 2), conn(ne * 4), em(ne, 0), mt(1, SVL_MAT_ELASTIC2DPLANESTRAIN);
    svl::gpu::check(svl_grid_build(&g, X.data(), td.data(), fd.data(), conn.data(), nullptr, nullptr, nullptr, nullptr));
    std::vector<double> mp = {2.0e8, 0.25, 2000.0, 0, 0, 0, 0, 0};
    svl_model_desc md{};
    md.ndim = 2; md.nnode = nn; md.ndof = 2; md.coords = X.data(); md.totaldof = td.data(); md.freedof = fd.data();
    md.ntotal = nt; md.nfree = nf; md.elem_type = SVL_ELEM_LIN2DQUAD4; md.nelem = ne; md.conn = conn.data();
    md.elem_mat = em.data(); md.nmat = 1; md.mat_type = mt.data(); md.mat_param = mp.data(); md.lumped = 1;
    const double dt = 0.5 / std::sqrt(3.0 * 8.0e7 / 2000.0);
    std::vector<double> series(101);
    for (int k = 0; k < 101; ++k) { double t = k * dt - 0.24, b = (M_PI * 5.0 * t) * (M_PI * 5.0 * t); series[k] = 1e6 * (1 - 2 * b) * std::exp(-b); }
    int32_t sp[2] = {0, 101}, fdof[1] = {td[(10 * 21 + 10) * 2 + 1]}, fser[1] = {0};
    double fcoef[1] = {-1.0};
    svl_load_desc ld{};
    ld.nseries = 1; ld.series_ptr = sp; ld.series_val = series.data();
    ld.nforce = 1; ld.force_dof = fdof; ld.force_series = fser; ld.force_coef = fcoef;
    try {
        svl::gpu::CentralDifference cd(md, ld, dt);
        cd.Initialize();
        for (unsigned k = 1; k <= 100; ++k)
            if (cd.ComputeNewStep(k)) { std::printf("stop at %u\n", k); return 2; }
        double mx = 0;
        for (double u : cd.GetDisplacements()) mx = std::fmax(mx, std::fabs(u));
        double rmax = 0;
        for (double r : cd.ComputeReactionForce(100)) rmax = std::fmax(rmax, std::fabs(r));
        svl::gpu::NewmarkBeta nm(md, ld, 4.0 * dt);
        nm.Initialize();
        for (unsigned k = 1; k <= 20; ++k)
            if (nm.ComputeNewStep(k)) { std::printf("newmark stop at %u\n", k); return 3; }
        double mn = 0;
        for (double u : nm.GetDisplacements()) mn = std::fmax(mn, std::fabs(u));
        svl::gpu::ExtendedNewmarkBeta xn(md, ld, 4.0 * dt, 1e-12);
        xn.Initialize();
        if (xn.ComputeNewSteps(1, 20)) { std::printf("extended newmark stop\n"); return 4; }
        double mxn = 0, dmax = 0;
        const std::vector<double> ux = xn.GetDisplacements(), un = nm.GetDisplacements();
        for (size_t i = 0; i < ux.size(); ++i) { mxn = std::fmax(mxn, std::fabs(ux[i])); dmax = std::fmax(dmax, std::fabs(ux[i] - un[i])); }
        // NewtonRaphson (2 iterations, cnvgtol 0) on the elastic box: the second
        // iteration only corrects the first solve's residual
        svl::gpu::NewtonRaphson newton{0.0, 2, 4};
        svl::gpu::NewmarkBeta nw(md, ld, 4.0 * dt, 1e-12, 1e-12, 1e-12, 20000, &newton);
        nw.Initialize();
        if (nw.ComputeNewSteps(1, 20)) { std::printf("newton stop\n"); return 5; }
        double dnw = 0;
        const std::vector<double> uw = nw.GetDisplacements();
        for (size_t i = 0; i < uw.size(); ++i) dnw = std::fmax(dnw, std::fabs(uw[i] - un[i]));
        std::printf("max|U| %.6e newmark %.6e extended %.6e (diff %.3e) newton-diff %.3e reaction %.6e\n", mx, mn,
                    mxn, dmax, dnw, rmax);
    } catch (const svl::gpu::Error& e) {
        if (e.code == SVL_ERR_NODEVICE) { std::printf("nodevice\n"); return 0; }
        std::printf("error %d %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
