// Explicit central-difference step on the GPU: FP64 plain form for general
// (unstructured) lin2DQuad4 / lin3DHexa8 meshes with elastic or J2
// materials, lumped mass, point/body loads, support motion and EQUAL-type
// constraints.
//
// One step is the reference's CentralDifference::ComputeNewStep with the
// Linear algorithm and the diagonal solve (CentralDifference.cpp:124-151,
// 206-221, Linear.cpp:22-56), reorganised for the GPU:
//
//   k_element   one thread per element: material update from the strain
//               displacement (Algorithm::UpdateStatesIncrements of the
//               previous step, Algorithm.cpp:18-56, fused here) and the
//               element internal force B^T sigma with the assembler's
//               force tolerance applied (Assembler.cpp:262).  Writes the
//               element force block fe[(local dof)][element].
//   k_node      one thread per node: deterministic gather of fe over the
//               node's inverse connectivity in ascending element order
//               (= the reference's std::map summation order, no float
//               atomics), external loads, effective force, diagonal solve
//               and the V/A/Up/U update.  Used when T is the identity on
//               free dofs (no constraints).
//   k_residual / k_free / k_update   the same work split in three when
//               constraints couple total dofs (T^T and T applied as CSR).
//
// The step index k lives in device memory and is advanced by k_element, so
// a captured CUDA graph of G steps replays without parameter updates.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "svl_internal.hpp"

using namespace svl;

namespace {

#define CUDA_TRY(x)                                                                  \
    do {                                                                             \
        cudaError_t err_ = (x);                                                      \
        if (err_ != cudaSuccess) {                                                   \
            set_error("%s failed: %s (%s:%d)", #x, cudaGetErrorString(err_), __FILE__, __LINE__); \
            return SVL_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

constexpr int kMatElastic = 0;
constexpr int kMatJ2 = 1;
constexpr int kJ2State = 13;   // plastic strain (6), back stress (6), alpha

struct DevView {
    int nelem, nnode, ntotal, nfree;
    // elements
    const int32_t* edof;     // [nen*ndof][E]   total dof of each element dof
    const int32_t* egeo;     // [E]             geometry class
    const double* geo;       // [ngeo][ngp][per]
    const int32_t* ekind;    // [E]             kMatElastic / kMatJ2
    const double* ecoef;     // [5][E]          c1,c2,c3 | K,G,H,beta,SY
    double* gstate;          // [13][ngp][E]    J2 state
    double* fe;              // [nen*ndof][E]
    // nodes / dofs
    const int32_t* ntdof;    // [nnode][ndof]
    const int32_t* inv_ptr;  // [nnode+1]
    const int32_t* inv_ent;  // element*8 + local node
    const int32_t* tfree;    // [ntotal] free dof or -1 (identity-T path)
    const double* Md;        // [ntotal]
    const double* kinv;      // [nfree]  1 / (T^T K T)_ff
    const double* Kd;        // [ntotal] 1/dt^2 M
    double *U, *V, *A, *Up, *Us, *R, *du;
    // T and T^T as CSR (constraint path)
    const int32_t *T_ptr, *T_col; const double* T_val;
    const int32_t *TT_ptr, *TT_row; const double* TT_val;
    // loads
    const int32_t* ld_ptr; const int32_t* ld_ser; const double* ld_coef;
    const int32_t* sm_ptr; const int32_t* sm_ser; const double* sm_fac;
    const int32_t* s_ptr; const double* s_val;
    int* step;               // device step index k
    int* flag;               // non-finite flag
    double ftol, inv_dt2, inv_2dt;
};

__device__ __forceinline__ double series_at(const DevView& d, int s, int k) {
    const int b = d.s_ptr[s], n = d.s_ptr[s + 1] - b;
    return (k >= 0 && k < n) ? d.s_val[b + k] : 0.0;
}
__device__ __forceinline__ double support_at(const DevView& d, int s, int k) {
    const int b = d.s_ptr[s], n = d.s_ptr[s + 1] - b;
    if (n <= 0) return 0.0;
    return (k < n) ? d.s_val[b + k] : d.s_val[b];
}
__device__ __forceinline__ double fext_at(const DevView& d, int t, int k) {
    double f = 0.0;
    for (int i = d.ld_ptr[t]; i < d.ld_ptr[t + 1]; ++i) f += d.ld_coef[i] * series_at(d, d.ld_ser[i], k);
    return f;
}
__device__ __forceinline__ double sm_at(const DevView& d, int t, int k) {
    double s = 0.0;
    for (int i = d.sm_ptr[t]; i < d.sm_ptr[t + 1]; ++i) {
        double g = support_at(d, d.sm_ser[i], k);
        if (k > 0) g -= support_at(d, d.sm_ser[i], k - 1);
        s += d.sm_fac[i] * g;
    }
    return s;
}

// J2 radial return on the tensor strain E[6] (shear = gamma/2), in place on
// the Gauss-point state (PlasticPlaneStrainJ2.cpp:227-279, Plastic3DJ2.cpp:206-255).
__device__ __forceinline__ void j2_return(const double E[6], double st[kJ2State], double K, double G,
                                          double H, double beta, double SY, double sig6[6]) {
    const double tr = E[0] + E[1] + E[2];
    double trial[6], rel[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const double dev = E[i] - (i < 3 ? 1.0 / 3.0 * tr : 0.0);
        trial[i] = 2.0 * G * (dev - st[i]);
        rel[i] = trial[i] - st[6 + i];
    }
    const double nrm = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2] +
                            2.0 * (rel[3] * rel[3] + rel[4] * rel[4] + rel[5] * rel[5]));
    const double f = nrm - sqrt(2.0 / 3.0) * (SY + st[12] * beta * H);
    if (f <= 0) {
#pragma unroll
        for (int i = 0; i < 6; ++i) sig6[i] = (i < 3 ? K * tr : 0.0) + trial[i];
    } else {
        const double dg = f / (2.0 * G + 2.0 / 3.0 * H);
        st[12] += sqrt(2.0 / 3.0) * dg;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const double n = rel[i] / nrm;
            st[6 + i] += 2.0 / 3.0 * (1.0 - beta) * H * dg * n;
            st[i] += dg * n;
            sig6[i] = (i < 3 ? K * tr : 0.0) + trial[i] - 2.0 * G * dg * n;
        }
    }
}

template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_element(DevView d, const double* __restrict__ Ustrain, int ngp, int advance_step) {
    constexpr int NC = ND * NEN;
    constexpr int PER = NEN * ND + 1;
    const int E = d.nelem;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (advance_step && blockIdx.x == 0 && threadIdx.x == 0) d.step[0] += 1;
    if (e >= E) return;
    double ue[NC], fe[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) { ue[j] = Ustrain[d.edof[(size_t)j * E + e]]; fe[j] = 0.0; }
    const int kind = d.ekind[e];
    const double* g0 = d.geo + (size_t)d.egeo[e] * ngp * PER;
    const double c1 = d.ecoef[e], c2 = d.ecoef[(size_t)E + e], c3 = d.ecoef[2 * (size_t)E + e];
    for (int q = 0; q < ngp; ++q) {
        const double* g = g0 + q * PER;
        double b[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? __ldg(g + a * ND + j) : 0.0;
        const double w = __ldg(g + PER - 1);
        double sig[6];
        if (ND == 2) {
            double exx = 0, eyy = 0, gxy = 0;
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                exx += b[a][0] * ue[2 * a];
                eyy += b[a][1] * ue[2 * a + 1];
                gxy += b[a][1] * ue[2 * a] + b[a][0] * ue[2 * a + 1];
            }
            if (kind == kMatElastic) {
                sig[0] = c1 * exx + c2 * eyy;
                sig[1] = c2 * exx + c1 * eyy;
                sig[2] = c3 * gxy;
            } else {
                double st[kJ2State];
                double* gs = d.gstate + (size_t)q * E + e;
#pragma unroll
                for (int i = 0; i < kJ2State; ++i) st[i] = gs[(size_t)i * ngp * E];
                const double Ev[6] = {0.0, exx, eyy, 0.0, 0.5 * gxy, 0.0};
                double s6[6];
                j2_return(Ev, st, c1, c2, c3, d.ecoef[3 * (size_t)E + e], d.ecoef[4 * (size_t)E + e], s6);
#pragma unroll
                for (int i = 0; i < kJ2State; ++i) gs[(size_t)i * ngp * E] = st[i];
                sig[0] = s6[1]; sig[1] = s6[2]; sig[2] = s6[4];
            }
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                fe[2 * a] += w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
                fe[2 * a + 1] += w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
            }
        } else {
            double ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const double ux = ue[3 * a], uy = ue[3 * a + 1], uz = ue[3 * a + 2];
                ev[0] += b[a][0] * ux;
                ev[1] += b[a][1] * uy;
                ev[2] += b[a][2] * uz;
                ev[3] += b[a][1] * ux + b[a][0] * uy;
                ev[4] += b[a][2] * uy + b[a][1] * uz;
                ev[5] += b[a][2] * ux + b[a][0] * uz;
            }
            if (kind == kMatElastic) {
                sig[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
                sig[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
                sig[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
                sig[3] = c3 * ev[3]; sig[4] = c3 * ev[4]; sig[5] = c3 * ev[5];
            } else {
                double st[kJ2State];
                double* gs = d.gstate + (size_t)q * E + e;
#pragma unroll
                for (int i = 0; i < kJ2State; ++i) st[i] = gs[(size_t)i * ngp * E];
                const double Ev[6] = {ev[0], ev[1], ev[2], 0.5 * ev[3], 0.5 * ev[4], 0.5 * ev[5]};
                j2_return(Ev, st, c1, c2, c3, d.ecoef[3 * (size_t)E + e], d.ecoef[4 * (size_t)E + e], sig);
#pragma unroll
                for (int i = 0; i < kJ2State; ++i) gs[(size_t)i * ngp * E] = st[i];
            }
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const double bx = b[a][0], by = b[a][1], bz = b[a][2];
                fe[3 * a] += w * (bx * sig[0] + by * sig[3] + bz * sig[5]);
                fe[3 * a + 1] += w * (by * sig[1] + bx * sig[3] + bz * sig[4]);
                fe[3 * a + 2] += w * (bz * sig[2] + by * sig[4] + bx * sig[5]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const double v = fe[j];
        d.fe[(size_t)j * E + e] = (fabs(v) > d.ftol) ? v : 0.0;
    }
}

template <int ND>
__device__ __forceinline__ double gather_fint(const DevView& d, int n, int c) {
    double f = 0.0;
    const int E = d.nelem;
    for (int i = d.inv_ptr[n]; i < d.inv_ptr[n + 1]; ++i) {
        const int ent = d.inv_ent[i];
        const int e = ent >> 3, a = ent & 7;
        f += d.fe[(size_t)(a * ND + c) * E + e];
    }
    return f;
}

// Identity-T path: everything after the element forces, per node.
template <int ND>
__global__ void __launch_bounds__(256) k_node(DevView d) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        const double u = d.U[t], up = d.Up[t];
        const double R = ((fext + 0.0) - fint) + (d.inv_dt2 * d.Md[t]) * (u - up);
        const double sm = sm_at(d, t, k);
        const int f = d.tfree[t];
        double dut = 0.0;
        if (f >= 0) dut = d.kinv[f] * (R - d.Kd[t] * sm);
        const double dU = dut + sm;
        d.Us[t] = u + dut;
        d.V[t] = d.inv_2dt * (u + dU - up);
        d.A[t] = d.inv_dt2 * (dU - u + up);
        d.Up[t] = u;
        const double un = u + dU;
        d.U[t] = un;
        bad |= !isfinite(un);
    }
    if (bad) atomicOr(d.flag, 1);
}

// Constraint path, part 1: total residual R per node.
template <int ND>
__global__ void __launch_bounds__(256) k_residual(DevView d) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        d.R[t] = ((fext + 0.0) - fint) + (d.inv_dt2 * d.Md[t]) * (d.U[t] - d.Up[t]);
    }
}

// Part 2: Feff = T^T R - T^T (K SM), du = (1/Keff) Feff, per free dof.
__global__ void __launch_bounds__(256) k_free(DevView d) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nfree) return;
    const int k = d.step[0];
    double feff = 0.0, lg = 0.0;
    for (int i = d.TT_ptr[f]; i < d.TT_ptr[f + 1]; ++i) {
        const int t = d.TT_row[i];
        feff += d.TT_val[i] * d.R[t];
        lg += d.TT_val[i] * (d.Kd[t] * sm_at(d, t, k));
    }
    d.du[f] = d.kinv[f] * (feff - lg);
}

// Part 3: dU = T du + SM and the state update, per node.
template <int ND>
__global__ void __launch_bounds__(256) k_update(DevView d) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        double dut = 0.0;
        for (int i = d.T_ptr[t]; i < d.T_ptr[t + 1]; ++i) dut += d.T_val[i] * d.du[d.T_col[i]];
        const double sm = sm_at(d, t, k);
        const double u = d.U[t], up = d.Up[t];
        const double dU = dut + sm;
        d.Us[t] = u + dut;
        d.V[t] = d.inv_2dt * (u + dU - up);
        d.A[t] = d.inv_dt2 * (dU - u + up);
        d.Up[t] = u;
        const double un = u + dU;
        d.U[t] = un;
        bad |= !isfinite(un);
    }
    if (bad) atomicOr(d.flag, 1);
}

}  // namespace

// ---------------------------------------------------------------------------

struct svl_cd {
    HostModel m;
    svl_cd_opts opts{};
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    DevView d{};
    int ngeo = 0;
    bool identity_T = true;
    bool has_sm = false;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int64_t launches = 0;
    int64_t launches_last = 0;
    double* hist_dev = nullptr;
    int hist_cap = 0;

    template <typename T>
    int upload(const std::vector<T>& h, const T** out) {
        T* p = nullptr;
        size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
        if (cudaMalloc(&p, bytes) != cudaSuccess) { set_error("cudaMalloc of %zu bytes failed", bytes); return SVL_ERR_NOMEM; }
        allocs.push_back(p);
        if (!h.empty()) CUDA_TRY(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
        *out = p;
        return SVL_OK;
    }
    template <typename T>
    int zeros(size_t n, T** out) {
        T* p = nullptr;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (cudaMalloc(&p, bytes) != cudaSuccess) { set_error("cudaMalloc of %zu bytes failed", bytes); return SVL_ERR_NOMEM; }
        allocs.push_back(p);
        CUDA_TRY(cudaMemsetAsync(p, 0, bytes, stream));
        *out = p;
        return SVL_OK;
    }
    ~svl_cd() {
        if (graph) cudaGraphExecDestroy(graph);
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : allocs) cudaFree(p);
        if (hist_dev) cudaFree(hist_dev);
        if (stream) cudaStreamDestroy(stream);
    }
};

#define TRY(x) do { int st_ = (x); if (st_ != SVL_OK) return st_; } while (0)

static int cd_setup(svl_cd* cd, const svl_load_desc* L) {
    HostModel& m = cd->m;
    const int E = m.nelem, nen = m.nen, nd = m.ndim, nc = nen * nd, per = nen * nd + 1;
    // --- element tables -----------------------------------------------------
    std::vector<int32_t> edof((size_t)nc * E);
    for (int e = 0; e < E; ++e)
        for (int a = 0; a < nen; ++a)
            for (int c = 0; c < nd; ++c)
                edof[(size_t)(a * nd + c) * E + e] = m.tdof[(size_t)m.conn[(size_t)e * nen + a] * nd + c];
    // geometry classes: elements whose Gauss-point data are bitwise equal share one slot
    std::vector<int32_t> egeo(E);
    std::vector<double> geo;
    {
        std::map<std::vector<double>, int> seen;
        std::vector<double> buf((size_t)m.ngp * per);
        for (int e = 0; e < E; ++e) {
            for (int q = 0; q < m.ngp; ++q) {
                double dNx[8][3], N[8];
                const double det = gp_geometry(m, e, q, dNx, N);
                for (int a = 0; a < nen; ++a)
                    for (int j = 0; j < nd; ++j) buf[(size_t)q * per + a * nd + j] = dNx[a][j];
                buf[(size_t)q * per + per - 1] = gp_factor(m, e, det);
            }
            auto it = seen.find(buf);
            if (it == seen.end()) {
                const int id = (int)seen.size();
                if (seen.size() < 4096) seen.emplace(buf, id);
                geo.insert(geo.end(), buf.begin(), buf.end());
                egeo[e] = (int32_t)(geo.size() / buf.size()) - 1;
            } else egeo[e] = it->second;
        }
        cd->ngeo = (int)(geo.size() / buf.size());
    }
    std::vector<int32_t> ekind(E);
    std::vector<double> ecoef((size_t)5 * E, 0.0);
    for (int e = 0; e < E; ++e) {
        const double* p = m.param(e);
        const int t = m.mat_type(e);
        if (t == SVL_MAT_ELASTIC2DPLANESTRAIN || t == SVL_MAT_ELASTIC3DLINEAR) {
            ekind[e] = kMatElastic;
            const double Em = p[0], nu = p[1];
            ecoef[e] = Em * (1.0 - nu) / (1.0 - 2.0 * nu) / (1.0 + nu);
            ecoef[(size_t)E + e] = Em * nu / (1.0 - 2.0 * nu) / (1.0 + nu);
            ecoef[2 * (size_t)E + e] = Em / (2.0 * (1.0 + nu));
        } else {
            ekind[e] = kMatJ2;
            ecoef[e] = p[0]; ecoef[(size_t)E + e] = p[1]; ecoef[2 * (size_t)E + e] = p[3];
            ecoef[3 * (size_t)E + e] = p[4]; ecoef[4 * (size_t)E + e] = p[5];
        }
    }
    // --- inverse connectivity, ascending element order ----------------------
    std::vector<int32_t> inv_ptr(m.nnode + 1, 0), inv_ent;
    for (int e = 0; e < E; ++e)
        for (int a = 0; a < nen; ++a) inv_ptr[m.conn[(size_t)e * nen + a] + 1]++;
    for (int n = 0; n < m.nnode; ++n) inv_ptr[n + 1] += inv_ptr[n];
    inv_ent.resize(inv_ptr.back());
    {
        std::vector<int32_t> fill(inv_ptr.begin(), inv_ptr.end() - 1);
        for (int e = 0; e < E; ++e)
            for (int a = 0; a < nen; ++a) inv_ent[fill[m.conn[(size_t)e * nen + a]]++] = e * 8 + a;
    }
    if ((int64_t)E * 8 > INT32_MAX) { set_error("too many elements for the inverse connectivity encoding"); return SVL_ERR_UNSUPPORTED; }
    // --- mass, T operator ---------------------------------------------------
    std::vector<double> Md;
    lumped_mass_diag(m, cd->opts.mtol, Md);
    const double dt = cd->opts.dt;
    const double inv_dt2 = 1.0 / dt / dt;
    std::vector<double> Kd(m.ntotal);
    for (int t = 0; t < m.ntotal; ++t) Kd[t] = inv_dt2 * Md[t];
    std::vector<int32_t> T_ptr, T_col;
    std::vector<double> T_val;
    build_total_to_free(m, T_ptr, T_col, T_val);
    std::vector<double> kff(m.nfree, 0.0);
    for (int t = 0; t < m.ntotal; ++t)
        for (int i = T_ptr[t]; i < T_ptr[t + 1]; ++i) kff[T_col[i]] += T_val[i] * Kd[t] * T_val[i];
    std::vector<double> kinv(m.nfree);
    for (int f = 0; f < m.nfree; ++f) {
        if (!(kff[f] > 0.0)) { set_error("free dof %d has no mass: the explicit update needs a positive lumped mass", f); return SVL_ERR_INVALID; }
        kinv[f] = 1.0 / kff[f];
    }
    // identity T: each total row has <= 1 entry equal to 1.0 and each free dof one row
    std::vector<int32_t> tfree(m.ntotal, -1);
    cd->identity_T = (m.nconstraint == 0);
    for (int t = 0; t < m.ntotal && cd->identity_T; ++t) {
        const int cnt = T_ptr[t + 1] - T_ptr[t];
        if (cnt > 1 || (cnt == 1 && T_val[T_ptr[t]] != 1.0)) cd->identity_T = false;
        else if (cnt == 1) tfree[t] = T_col[T_ptr[t]];
    }
    std::vector<int32_t> TT_ptr(m.nfree + 1, 0), TT_row;
    std::vector<double> TT_val;
    for (int32_t c : T_col) TT_ptr[c + 1]++;
    for (int f = 0; f < m.nfree; ++f) TT_ptr[f + 1] += TT_ptr[f];
    TT_row.resize(T_col.size()); TT_val.resize(T_col.size());
    {
        std::vector<int32_t> fill(TT_ptr.begin(), TT_ptr.end() - 1);
        for (int t = 0; t < m.ntotal; ++t)
            for (int i = T_ptr[t]; i < T_ptr[t + 1]; ++i) { const int p = fill[T_col[i]]++; TT_row[p] = t; TT_val[p] = T_val[i]; }
    }
    // --- loads ---------------------------------------------------------------
    std::vector<int32_t> s_ptr(1, 0);
    std::vector<double> s_val;
    std::vector<int32_t> ld_ptr(m.ntotal + 1, 0), ld_ser, sm_ptr(m.ntotal + 1, 0), sm_ser;
    std::vector<double> ld_coef, sm_fac;
    if (L) {
        if (L->nseries > 0) {
            if (!L->series_ptr || !L->series_val) { set_error("series arrays are NULL"); return SVL_ERR_INVALID; }
            s_ptr.assign(L->series_ptr, L->series_ptr + L->nseries + 1);
            for (int s = 0; s < L->nseries; ++s)
                if (s_ptr[s + 1] < s_ptr[s]) { set_error("series_ptr is not monotone"); return SVL_ERR_INVALID; }
            s_val.assign(L->series_val, L->series_val + s_ptr.back());
        }
        auto csr = [&](int n, const int32_t* dof, const int32_t* ser, const double* val,
                       std::vector<int32_t>& ptr, std::vector<int32_t>& oser, std::vector<double>& oval) -> int {
            if (n <= 0) return SVL_OK;
            if (!dof || !ser || !val) { set_error("load arrays are NULL"); return SVL_ERR_INVALID; }
            std::vector<int> order(n);
            for (int i = 0; i < n; ++i) {
                if (dof[i] < 0 || dof[i] >= m.ntotal) { set_error("load dof %d out of range", dof[i]); return SVL_ERR_INVALID; }
                if (ser[i] < 0 || ser[i] >= L->nseries) { set_error("load series %d out of range", ser[i]); return SVL_ERR_INVALID; }
                order[i] = i;
                ptr[dof[i] + 1]++;
            }
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dof[a] < dof[b]; });
            for (int t = 0; t < m.ntotal; ++t) ptr[t + 1] += ptr[t];
            for (int i : order) { oser.push_back(ser[i]); oval.push_back(val[i]); }
            return SVL_OK;
        };
        TRY(csr(L->nforce, L->force_dof, L->force_series, L->force_coef, ld_ptr, ld_ser, ld_coef));
        TRY(csr(L->nsupport, L->sm_dof, L->sm_series, L->sm_factor, sm_ptr, sm_ser, sm_fac));
        cd->has_sm = L->nsupport > 0;
    }
    // --- device upload -------------------------------------------------------
    DevView& d = cd->d;
    d.nelem = E; d.nnode = m.nnode; d.ntotal = m.ntotal; d.nfree = m.nfree;
    TRY(cd->upload(edof, &d.edof));
    TRY(cd->upload(egeo, &d.egeo));
    TRY(cd->upload(geo, &d.geo));
    TRY(cd->upload(ekind, &d.ekind));
    TRY(cd->upload(ecoef, &d.ecoef));
    TRY(cd->zeros((size_t)kJ2State * m.ngp * (m.has_j2() ? E : 1), &d.gstate));
    TRY(cd->zeros((size_t)nc * E, &d.fe));
    TRY(cd->upload(m.tdof, &d.ntdof));
    TRY(cd->upload(inv_ptr, &d.inv_ptr));
    TRY(cd->upload(inv_ent, &d.inv_ent));
    TRY(cd->upload(tfree, &d.tfree));
    TRY(cd->upload(Md, &d.Md));
    TRY(cd->upload(kinv, &d.kinv));
    TRY(cd->upload(Kd, &d.Kd));
    TRY(cd->zeros(m.ntotal, &d.U)); TRY(cd->zeros(m.ntotal, &d.V)); TRY(cd->zeros(m.ntotal, &d.A));
    TRY(cd->zeros(m.ntotal, &d.Up)); TRY(cd->zeros(m.ntotal, &d.Us)); TRY(cd->zeros(m.ntotal, &d.R));
    TRY(cd->zeros(m.nfree, &d.du));
    TRY(cd->upload(T_ptr, &d.T_ptr)); TRY(cd->upload(T_col, &d.T_col)); TRY(cd->upload(T_val, &d.T_val));
    TRY(cd->upload(TT_ptr, &d.TT_ptr)); TRY(cd->upload(TT_row, &d.TT_row)); TRY(cd->upload(TT_val, &d.TT_val));
    TRY(cd->upload(ld_ptr, &d.ld_ptr)); TRY(cd->upload(ld_ser, &d.ld_ser)); TRY(cd->upload(ld_coef, &d.ld_coef));
    TRY(cd->upload(sm_ptr, &d.sm_ptr)); TRY(cd->upload(sm_ser, &d.sm_ser)); TRY(cd->upload(sm_fac, &d.sm_fac));
    TRY(cd->upload(s_ptr, &d.s_ptr)); TRY(cd->upload(s_val, &d.s_val));
    TRY(cd->zeros(2, &d.step));
    TRY(cd->zeros(1, &d.flag));
    d.ftol = cd->opts.ftol;
    d.inv_dt2 = inv_dt2;
    d.inv_2dt = 1.0 / 2.0 / dt;
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

// Launches kernel `kind` of one step (0 element, 1 node, 2 residual,
// 3 free, 4 update); returns SVL_OK, or 1 when the kind is not used.
static int cd_launch_kind(svl_cd* cd, int kind) {
    const HostModel& m = cd->m;
    const DevView& d = cd->d;
    const int eb = 128, nb = 256;
    const int eg = (m.nelem + eb - 1) / eb, ng = (m.nnode + nb - 1) / nb, fg = (m.nfree + nb - 1) / nb;
    switch (kind) {
    case 0:
        // The strain displacement of the previous step (U + T du, without the
        // support-motion increment) feeds the material update.
        if (m.ndim == 2) k_element<2, 4><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
        else k_element<3, 8><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
        break;
    case 1:
        if (!cd->identity_T) return 1;
        if (m.ndim == 2) k_node<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_node<3><<<ng, nb, 0, cd->stream>>>(d);
        break;
    case 2:
        if (cd->identity_T) return 1;
        if (m.ndim == 2) k_residual<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_residual<3><<<ng, nb, 0, cd->stream>>>(d);
        break;
    case 3:
        if (cd->identity_T || m.nfree == 0) return 1;
        k_free<<<fg, nb, 0, cd->stream>>>(d);
        break;
    case 4:
        if (cd->identity_T) return 1;
        if (m.ndim == 2) k_update<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_update<3><<<ng, nb, 0, cd->stream>>>(d);
        break;
    default:
        return 1;
    }
    ++cd->launches;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

static int cd_launch_step(svl_cd* cd) {
    for (int kind = 0; kind < 5; ++kind) {
        const int st = cd_launch_kind(cd, kind);
        if (st != SVL_OK && st != 1) return st;
    }
    return SVL_OK;
}

static int launches_per_step(const svl_cd* cd) { return cd->identity_T ? 2 : (cd->m.nfree > 0 ? 4 : 3); }

extern "C" {

int svl_device_info(int* device_count, int* sm_count, int* cc_major, int* cc_minor) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        if (device_count) *device_count = 0;
        set_error("no CUDA device: %s", cudaGetErrorString(e));
        return SVL_ERR_NODEVICE;
    }
    cudaDeviceProp p;
    CUDA_TRY(cudaGetDeviceProperties(&p, 0));
    if (device_count) *device_count = n;
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return SVL_OK;
}

int svl_set_device(int device) {
    CUDA_TRY(cudaSetDevice(device));
    return SVL_OK;
}

int svl_cd_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_cd_opts* opts, svl_cd** out) {
    if (!out || !opts) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *out = nullptr;
    if (!(opts->dt > 0.0)) { set_error("dt must be positive"); return SVL_ERR_INVALID; }
    if (opts->precision != SVL_PREC_FP64) {
        set_error("svl_cd_create: precision %d is served by svl_cdx_create (structured grids)", opts->precision);
        return SVL_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device available"); return SVL_ERR_NODEVICE; }
    svl_cd* cd = new svl_cd();
    cd->opts = *opts;
    if (!model_from_desc(model, cd->m)) { delete cd; return SVL_ERR_INVALID; }
    if (!cd->m.lumped) { delete cd; set_error("the explicit path needs a lumped mass (massform LUMPED)"); return SVL_ERR_UNSUPPORTED; }
    if (cudaStreamCreateWithFlags(&cd->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete cd; set_error("cudaStreamCreate failed"); return SVL_ERR_CUDA;
    }
    int st = cd_setup(cd, loads);
    if (st != SVL_OK) { delete cd; return st; }
    *out = cd;
    return SVL_OK;
}

int svl_cd_set_initial(svl_cd* cd, const double* U0, const double* V0, const double* A0) {
    if (!cd) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    const int nt = cd->m.ntotal;
    const double dt = cd->opts.dt;
    std::vector<double> U(nt, 0.0), V(nt, 0.0), A(nt, 0.0), Up(nt);
    if (U0) std::memcpy(U.data(), U0, sizeof(double) * nt);
    if (V0) std::memcpy(V.data(), V0, sizeof(double) * nt);
    if (A0) std::memcpy(A.data(), A0, sizeof(double) * nt);
    for (int t = 0; t < nt; ++t) Up[t] = U[t] - dt * V[t] + dt * dt / 2.0 * A[t];
    CUDA_TRY(cudaMemcpyAsync(cd->d.U, U.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, cd->stream));
    CUDA_TRY(cudaMemcpyAsync(cd->d.V, V.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, cd->stream));
    CUDA_TRY(cudaMemcpyAsync(cd->d.A, A.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, cd->stream));
    CUDA_TRY(cudaMemcpyAsync(cd->d.Up, Up.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, cd->stream));
    // fresh analysis: strain displacement, element forces and material state
    // return to the virgin state (Element::InitialState)
    CUDA_TRY(cudaMemsetAsync(cd->d.Us, 0, sizeof(double) * nt, cd->stream));
    CUDA_TRY(cudaMemsetAsync(cd->d.gstate, 0, sizeof(double) * (size_t)kJ2State * cd->m.ngp * (cd->m.has_j2() ? cd->m.nelem : 1), cd->stream));
    CUDA_TRY(cudaMemsetAsync(cd->d.flag, 0, sizeof(int), cd->stream));
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

int svl_cd_run(svl_cd* cd, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!cd) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (nsteps < 0) { set_error("nsteps must be >= 0"); return SVL_ERR_INVALID; }
    const int nt = cd->m.ntotal;
    const int64_t l0 = cd->launches;
    int kstart = k_first - 1;
    CUDA_TRY(cudaMemcpyAsync(cd->d.step, &kstart, sizeof(int), cudaMemcpyHostToDevice, cd->stream));
    if (U_hist) {
        // chunked device history, copied out as each chunk completes
        const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(nsteps, (int64_t)(256ll << 20) / ((int64_t)nt * 8)));
        if (cd->hist_cap < chunk) {
            CUDA_TRY(cudaStreamSynchronize(cd->stream));
            if (cd->hist_dev) cudaFree(cd->hist_dev);
            cd->hist_dev = nullptr;
            cd->hist_cap = 0;
            if (cudaMalloc(&cd->hist_dev, (size_t)chunk * nt * sizeof(double)) != cudaSuccess) {
                set_error("history buffer allocation failed"); return SVL_ERR_NOMEM;
            }
            cd->hist_cap = chunk;
        }
        for (int s0 = 0; s0 < nsteps; s0 += chunk) {
            const int n = std::min(chunk, nsteps - s0);
            for (int i = 0; i < n; ++i) {
                TRY(cd_launch_step(cd));
                CUDA_TRY(cudaMemcpyAsync(cd->hist_dev + (size_t)i * nt, cd->d.U, sizeof(double) * nt, cudaMemcpyDeviceToDevice, cd->stream));
            }
            CUDA_TRY(cudaMemcpyAsync(U_hist + (size_t)s0 * nt, cd->hist_dev, sizeof(double) * nt * n, cudaMemcpyDeviceToHost, cd->stream));
            CUDA_TRY(cudaStreamSynchronize(cd->stream));
        }
    } else {
        // G steps per CUDA graph replay
        const int G = 16;
        if (!cd->graph && nsteps >= G) {
            cudaGraph_t g;
            const int64_t lsave = cd->launches;
            CUDA_TRY(cudaStreamBeginCapture(cd->stream, cudaStreamCaptureModeThreadLocal));
            for (int i = 0; i < G; ++i) {
                int st = cd_launch_step(cd);
                if (st != SVL_OK) { cudaStreamEndCapture(cd->stream, &g); return st; }
            }
            CUDA_TRY(cudaStreamEndCapture(cd->stream, &g));
            CUDA_TRY(cudaGraphInstantiate(&cd->graph, g, 0));
            cudaGraphDestroy(g);
            cd->graph_steps = G;
            cd->launches = lsave;
        }
        int done = 0;
        if (cd->graph) {
            for (; done + cd->graph_steps <= nsteps; done += cd->graph_steps) {
                CUDA_TRY(cudaGraphLaunch(cd->graph, cd->stream));
                cd->launches += (int64_t)cd->graph_steps * launches_per_step(cd);
            }
        }
        for (; done < nsteps; ++done) TRY(cd_launch_step(cd));
    }
    cd->launches_last = cd->launches - l0;
    if (cd->opts.check_every > 0) {
        int flag = 0;
        CUDA_TRY(cudaMemcpyAsync(&flag, cd->d.flag, sizeof(int), cudaMemcpyDeviceToHost, cd->stream));
        CUDA_TRY(cudaStreamSynchronize(cd->stream));
        if (flag) { set_error("non-finite displacement detected"); return SVL_ERR_NONFINITE; }
    }
    return SVL_OK;
}

int svl_cd_run_timed(svl_cd* cd, int32_t k_first, int32_t nsteps, float* ms) {
    if (!cd || !ms) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    CUDA_TRY(cudaEventRecord(a, cd->stream));
    int st = svl_cd_run(cd, k_first, nsteps, nullptr);
    CUDA_TRY(cudaEventRecord(b, cd->stream));
    CUDA_TRY(cudaEventSynchronize(b));
    CUDA_TRY(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return st;
}

int svl_cd_profile(svl_cd* cd, int32_t k_first, int32_t nsteps, double* ms_kernel) {
    if (!cd || !ms_kernel) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    for (int i = 0; i < 5; ++i) ms_kernel[i] = 0.0;
    int kstart = k_first - 1;
    CUDA_TRY(cudaMemcpyAsync(cd->d.step, &kstart, sizeof(int), cudaMemcpyHostToDevice, cd->stream));
    cudaEvent_t ev[6];
    for (int i = 0; i < 6; ++i) CUDA_TRY(cudaEventCreate(&ev[i]));
    for (int s = 0; s < nsteps; ++s) {
        int used[5];
        CUDA_TRY(cudaEventRecord(ev[0], cd->stream));
        for (int kind = 0; kind < 5; ++kind) {
            const int st = cd_launch_kind(cd, kind);
            if (st != SVL_OK && st != 1) return st;
            used[kind] = (st == SVL_OK);
            CUDA_TRY(cudaEventRecord(ev[kind + 1], cd->stream));
        }
        CUDA_TRY(cudaEventSynchronize(ev[5]));
        for (int kind = 0; kind < 5; ++kind) {
            if (!used[kind]) continue;
            float t = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&t, ev[kind], ev[kind + 1]));
            ms_kernel[kind] += t;
        }
    }
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    return SVL_OK;
}

int svl_cd_get(svl_cd* cd, int32_t which, double* out) {
    if (!cd || !out) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    const double* src = which == 0 ? cd->d.U : which == 1 ? cd->d.V : which == 2 ? cd->d.A : nullptr;
    if (!src) { set_error("which must be 0, 1 or 2"); return SVL_ERR_INVALID; }
    CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * cd->m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

int svl_cd_device_ptr(svl_cd* cd, int32_t which, const double** dptr) {
    if (!cd || !dptr) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *dptr = which == 0 ? cd->d.U : which == 1 ? cd->d.V : which == 2 ? cd->d.A : nullptr;
    if (!*dptr) { set_error("which must be 0, 1 or 2"); return SVL_ERR_INVALID; }
    return SVL_OK;
}

int svl_cd_launch_count(svl_cd* cd, int64_t* launches) {
    if (!cd || !launches) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *launches = cd->launches_last;
    return SVL_OK;
}

int svl_cd_sync(svl_cd* cd) {
    if (!cd) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

void svl_cd_destroy(svl_cd* cd) { delete cd; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Stepping without device allocation (svl_cd_run_noalloc).
//
// For callers that must not let the library allocate device memory while
// their time loop runs (they own all device memory through their own pool,
// and cudaMalloc/cudaFree would synchronise the device and may fail or
// fragment that pool).  The element force block, the only per-step scratch
// of the CD kernels, lives in this file-scope static array instead of the
// handle's buffer; every GPU that loads the library holds it until exit.

static __device__ __align__(256) double g_noalloc_scratch[SVL_NOALLOC_SCRATCH_BYTES / sizeof(double)];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_addr[kNoallocMaxDevices] = {};

// Once per device, with that device current: the device address of the
// static array (the host-side symbol is only a stand-in, never a device
// pointer).
int noalloc_scratch(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (dev < 0 || dev >= kNoallocMaxDevices) { set_error("device %d out of range for the no-alloc scratch", dev); return SVL_ERR_INVALID; }
    if (!g_noalloc_addr[dev]) {
        int prev = 0;
        CUDA_TRY(cudaGetDevice(&prev));
        if (prev != dev) CUDA_TRY(cudaSetDevice(dev));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (prev != dev) cudaSetDevice(prev);
        if (e != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress of the no-alloc scratch failed on device %d: %s", dev, cudaGetErrorString(e));
            return SVL_ERR_CUDA;
        }
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[dev];
    return SVL_OK;
}

__global__ void k_set_step(int* step, int value) { step[0] = value; }

// The launches of one step, as in svl_cd_run, on a view whose element force
// block points at the static scratch.
int noalloc_launch_step(svl_cd* cd, const DevView& d) {
    const HostModel& m = cd->m;
    const int eb = 128, nb = 256;
    const int eg = (m.nelem + eb - 1) / eb, ng = (m.nnode + nb - 1) / nb, fg = (m.nfree + nb - 1) / nb;
    if (m.ndim == 2) k_element<2, 4><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
    else k_element<3, 8><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
    if (cd->identity_T) {
        if (m.ndim == 2) k_node<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_node<3><<<ng, nb, 0, cd->stream>>>(d);
    } else {
        if (m.ndim == 2) k_residual<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_residual<3><<<ng, nb, 0, cd->stream>>>(d);
        if (m.nfree > 0) k_free<<<fg, nb, 0, cd->stream>>>(d);
        if (m.ndim == 2) k_update<2><<<ng, nb, 0, cd->stream>>>(d);
        else k_update<3><<<ng, nb, 0, cd->stream>>>(d);
    }
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

}  // namespace

extern "C" int svl_cd_run_noalloc(svl_cd* cd, int32_t k_first, int32_t nsteps, double* d_U_out) {
    if (!cd) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (nsteps < 0) { set_error("nsteps must be >= 0"); return SVL_ERR_INVALID; }
    const HostModel& m = cd->m;
    const size_t need = (size_t)m.nelem * m.nen * m.ndof * sizeof(double);
    if (need > (size_t)SVL_NOALLOC_SCRATCH_BYTES) {
        set_error("svl_cd_run_noalloc: the element force block needs %zu bytes but the no-alloc scratch holds "
                  "at most %u bytes (%d elements of %d dofs); use svl_cd_run for this model",
                  need, (unsigned)SVL_NOALLOC_SCRATCH_BYTES, m.nelem, m.nen * m.ndof);
        return SVL_ERR_UNSUPPORTED;
    }
    cudaPointerAttributes attr{};
    CUDA_TRY(cudaPointerGetAttributes(&attr, cd->d.U));
    double* scratch = nullptr;
    TRY(noalloc_scratch(attr.device, &scratch));
    DevView d = cd->d;
    d.fe = scratch;
    k_set_step<<<1, 1, 0, cd->stream>>>(d.step, k_first - 1);
    CUDA_TRY(cudaGetLastError());
    for (int s = 0; s < nsteps; ++s) TRY(noalloc_launch_step(cd, d));
    if (d_U_out)
        CUDA_TRY(cudaMemcpyAsync(d_U_out, d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToDevice, cd->stream));
    return SVL_OK;
}
