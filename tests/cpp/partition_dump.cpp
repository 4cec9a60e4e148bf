// Reads a partition file with the C++ reader (svl_gb300/host/svl_partition.hpp)
// and either prints the model and load descriptors as JSON (`dump`, no GPU
// needed), prints Fext(k) of its loads for every step (`fext`, no GPU), or
// runs the simulation block through the C++ Integrator mirror and prints the
// final displacement vector (`run`).
#include <cstdio>
#include <string>
#include <vector>

#include "svl_gb300/host/svl_partition.hpp"

template <typename T>
static void arr(const char* name, const std::vector<T>& v, bool last = false) {
    std::printf("\"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::printf(i ? ", %.17g" : "%.17g", (double)v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

static int dump(const svl::gpu::Partition& P) {
    std::printf("{\n\"ndim\": %d, \"nnode\": %d, \"stride\": %d, \"ntotal\": %d, \"nfree\": %d, \"elem_type\": %d,\n",
                P.ndim, P.nnode, P.stride, P.ntotal, P.nfree, P.elem_type);
    std::printf("\"lumped\": %d, \"integrator\": \"%s\", \"algorithm\": \"%s\", \"dt\": %.17g, \"nt\": %d,\n", P.lumped ? 1 : 0,
                P.integrator.c_str(), P.algorithm.c_str(), P.dt, P.nt);
    std::printf("\"ndrm\": %d, \"drm_nt\": %d, \"nrecorder\": %d,\n", (int)P.drm_elem.size(), P.drm_nt, (int)P.recorders.size());
    arr("coords", P.coords); arr("totaldof", P.totaldof); arr("freedof", P.freedof); arr("node_ndof", P.node_ndof);
    arr("conn", P.conn); arr("elem_mat", P.elem_mat); arr("mat_type", P.mat_type); arr("mat_param", P.mat_param);
    arr("thickness", P.thickness); arr("node_mass", P.node_mass); arr("rayleigh", P.rayleigh);
    arr("elem_pml", P.elem_pml); arr("pml_param", P.pml_param); arr("dashpot_dof", P.dashpot_dof);
    arr("dashpot_eta", P.dashpot_eta); arr("con_slave", P.con_slave); arr("con_ptr", P.con_ptr);
    arr("con_master", P.con_master); arr("con_factor", P.con_factor);
    arr("series_ptr", P.series_ptr); arr("series_val", P.series_val); arr("force_dof", P.force_dof);
    arr("force_series", P.force_series); arr("force_coef", P.force_coef); arr("sm_dof", P.sm_dof);
    arr("sm_series", P.sm_series); arr("sm_factor", P.sm_factor); arr("drm_elem", P.drm_elem);
    arr("drm_factor", P.drm_factor); arr("drm_node_row", P.drm_node_row); arr("drm_node_ext", P.drm_node_ext);
    arr("drm_motion", P.drm_motion, true);
    std::printf("}\n");
    return 0;
}

// The run-process's dynamic loop over the simulation block's integrator.
static int run(const svl::gpu::Partition& P) {
    using namespace svl::gpu;
    const svl_model_desc md = P.model();
    const svl_load_desc ld = P.loads();
    const NewtonRaphson nr{P.cnvgtol, P.nstep, P.cnvgtest};
    const NewtonRaphson* newton = P.algorithm == "NEWTON" ? &nr : nullptr;
    std::vector<double> U;
    const unsigned nsteps = (unsigned)(P.nt - 1);
    if (P.integrator == "CENTRALDIFFERENCE") {
        CentralDifference cd(md, ld, P.dt, P.mtol, P.ftol);
        cd.Initialize();
        if (cd.ComputeNewSteps(1, nsteps)) { std::printf("stop %s\n", svl_last_error()); return 2; }
        U = cd.GetDisplacements();
    } else if (P.integrator == "NEWMARK") {
        NewmarkBeta nm(md, ld, P.dt, P.solver_tol, P.mtol, P.ftol, 100000, newton);
        nm.Initialize();
        if (nm.ComputeNewSteps(1, nsteps)) { std::printf("stop %s\n", svl_last_error()); return 2; }
        U = nm.GetDisplacements();
    } else if (P.integrator == "EXTENDEDNEWMARK") {
        ExtendedNewmarkBeta x(md, ld, P.dt, P.solver_tol, P.mtol, P.ftol, 100000, newton);
        x.Initialize();
        if (x.ComputeNewSteps(1, nsteps)) { std::printf("stop %s\n", svl_last_error()); return 2; }
        U = x.GetDisplacements();
    } else {
        std::printf("integrator %s\n", P.integrator.c_str());
        return 3;
    }
    std::printf("final");
    for (double u : U) std::printf(" %.17g", u);
    std::printf("\n");
    return 0;
}

// Fext(k) of the partition's loads on the host (the integrators'
// ComputeProgressiveForce without a stage force), for every k in 0..nt.
static int fext(const svl::gpu::Partition& P) {
    const svl::gpu::ExternalForce F(P.loads());
    for (int k = 0; k <= P.nt; ++k) {
        const std::vector<double> f = F.at((unsigned)k, P.ntotal);
        std::printf("%d", k);
        for (double v : f) std::printf(" %.17g", v);
        std::printf("\n");
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s dump|run|fext <partition file>\n", argv[0]);
        return 1;
    }
    try {
        const svl::gpu::Partition P = svl::gpu::load_partition(argv[2]);
        const std::string mode = argv[1];
        return mode == "run" ? run(P) : (mode == "fext" ? fext(P) : dump(P));
    } catch (const svl::gpu::Error& e) {
        std::printf("error %d %s\n", e.code, e.what());
        return 4;
    }
}
