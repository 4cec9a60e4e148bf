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
#include "svl_j2.cuh"
#include "svl_nnpc.hpp"

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

struct DevView {
    int nelem, nnode, ntotal, nfree;
    // elements
    const int32_t* edof;     // [nen*ndof][E]   total dof of each element dof
    const int32_t* egeo;     // [E]             geometry class
    const double* geo;       // [ngeo][ngp][per]
    const int32_t* ekind;    // [E]             kMatElastic / kMatJ2
    const double* ecoef;     // [5][E]          c1,c2,c3 | K,G,H,beta,SY
    double* gstate;          // [13][ngp][E]    J2 state
    double* ctan;            // [nt][ngp][E]    J2 consistent tangent of the last update, or null
                             //                 (nt = 9: rows/cols 1,2,4 in 2D; 36 in 3D)
    double* fe;              // [nen*ndof][E]
    // nodes / dofs
    const int32_t* ntdof;    // [nnode][ndof]
    const int32_t* inv_ptr;  // [nnode+1]
    const int32_t* inv_ent;  // element*8 + local node
    const int32_t* tfree;    // [ntotal] free dof or -1 (identity-T path)
    const double* Md;        // [ntotal] lumped mass (consistent-mass models: the nodal masses only)
    const double* erho;      // [E] density per element for the consistent mass action, or null (lumped)
    const double* fem;       // [nen*ndof][E] consistent mass action of the effective force, or null
    const double* kinv;      // [nfree]  1 / (T^T K T)_ff
    const double* Kd;        // [ntotal] 1/dt^2 M
    // Rayleigh damping C = sum_e (am_e M_e + ak_e K0_e) (lin2DQuad4.cpp:355-366)
    const double* Cd;        // [ntotal] sum_e am_e M_e (lumped), or null
    const double* dk0;       // [3][E]   ak_e * (c1, c2, c3) of the initial elastic tangent, or null
    // Lysmer dashpots on the implicit path: y_t += c sum eta (x_t - x_partner)
    const int32_t* dp_ptr; const int32_t* dp_col; const double* dp_eta;
    // domain-reduction entries: element, factor, ak of its Rayleigh damping;
    // node rows into the free-field motion, exterior flags; element force
    // blocks and their per-dof gather (entry order)
    int ndrm, drm_nt;
    const int32_t* drm_elem; const double* drm_factor; const double* drm_ak;
    const int32_t* drm_node_of;              // [ndrm][nen] node positions of each entry's element
    const int32_t* drm_row; const int32_t* drm_ext; const double* drm_motion;
    double* drm_fe;
    const int32_t* drm_ptr; const int32_t* drm_idx;
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
    return (k >= 0 && k < n) ? d.s_val[b + k] : d.s_val[b];
}
__device__ __forceinline__ double fext_at(const DevView& d, int t, int k) {
    double f = 0.0;
    for (int i = d.ld_ptr[t]; i < d.ld_ptr[t + 1]; ++i) f += d.ld_coef[i] * series_at(d, d.ld_ser[i], k);
    if (d.drm_ptr)
        for (int i = d.drm_ptr[t]; i < d.drm_ptr[t + 1]; ++i) f += d.drm_fe[d.drm_idx[i]];
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
                j2_return<2>(Ev, st, c1, c2, c3, d.ecoef[3 * (size_t)E + e], d.ecoef[4 * (size_t)E + e], s6,
                             d.ctan ? d.ctan + (size_t)q * E + e : nullptr, (size_t)ngp * E);
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
                j2_return<3>(Ev, st, c1, c2, c3, d.ecoef[3 * (size_t)E + e], d.ecoef[4 * (size_t)E + e], sig,
                             d.ctan ? d.ctan + (size_t)q * E + e : nullptr, (size_t)ngp * E);
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

// Tangent stiffness action q_e = sum_q w B^T C_t B p_e (element stiffness of
// lin2DQuad4.cpp:289-318 / lin3DHexa8.cpp:289-318 with Material::GetTangentStiffness):
// elastic elements from c1, c2, c3; J2 elements from the tangent stored at
// their last update (2D: rows/cols 1,2,4 of the 6x6 tensor-strain tangent
// applied to the engineering strain, as the reference assembles it).  Writes
// the unfiltered element vectors into d.fe (an operator scratch block).
// With damping tables, adds cc * ak_e K0_e p_e (the stiffness-proportional
// part of C); with_tan = 0 leaves the tangent out (damping action only).
template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_element_tan(DevView d, const double* __restrict__ P, int ngp, int with_tan,
                                                     double cc) {
    constexpr int NC = ND * NEN;
    constexpr int PER = NEN * ND + 1;
    constexpr int NS = ND == 2 ? 3 : 6;
    const int E = d.nelem;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    double ue[NC], fe[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) { ue[j] = P[d.edof[(size_t)j * E + e]]; fe[j] = 0.0; }
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
        double ev[NS], sig[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) ev[i] = 0.0;
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            if (ND == 2) {
                ev[0] += b[a][0] * ue[2 * a];
                ev[1] += b[a][1] * ue[2 * a + 1];
                ev[2] += b[a][1] * ue[2 * a] + b[a][0] * ue[2 * a + 1];
            } else {
                const double ux = ue[3 * a], uy = ue[3 * a + 1], uz = ue[3 * a + 2];
                ev[0] += b[a][0] * ux;
                ev[1] += b[a][1] * uy;
                ev[2] += b[a][2] * uz;
                ev[3 % NS] += b[a][1] * ux + b[a][0] * uy;
                ev[4 % NS] += b[a][2] * uy + b[a][1] * uz;
                ev[5 % NS] += b[a][2] * ux + b[a][0] * uz;
            }
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) sig[i] = 0.0;
        if (with_tan && kind == kMatElastic) {
            if (ND == 2) {
                sig[0] = c1 * ev[0] + c2 * ev[1];
                sig[1] = c2 * ev[0] + c1 * ev[1];
                sig[2] = c3 * ev[2];
            } else {
                sig[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
                sig[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
                sig[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
                sig[3 % NS] = c3 * ev[3 % NS]; sig[4 % NS] = c3 * ev[4 % NS]; sig[5 % NS] = c3 * ev[5 % NS];
            }
        } else if (with_tan) {
            const double* ct = d.ctan + (size_t)q * E + e;
            const size_t st = (size_t)ngp * E;
#pragma unroll
            for (int a = 0; a < NS; ++a) {
                double v = 0.0;
#pragma unroll
                for (int bb = 0; bb < NS; ++bb) v += ct[(size_t)(a * NS + bb) * st] * ev[bb];
                sig[a] = v;
            }
        }
        if (d.dk0) {
            const double k1 = cc * d.dk0[e], k2 = cc * d.dk0[(size_t)E + e], k3 = cc * d.dk0[2 * (size_t)E + e];
            if (ND == 2) {
                sig[0] += k1 * ev[0] + k2 * ev[1];
                sig[1] += k2 * ev[0] + k1 * ev[1];
                sig[2] += k3 * ev[2];
            } else {
                sig[0] += k1 * ev[0] + k2 * ev[1] + k2 * ev[2];
                sig[1] += k2 * ev[0] + k1 * ev[1] + k2 * ev[2];
                sig[2] += k2 * ev[0] + k2 * ev[1] + k1 * ev[2];
                sig[3 % NS] += k3 * ev[3 % NS]; sig[4 % NS] += k3 * ev[4 % NS]; sig[5 % NS] += k3 * ev[5 % NS];
            }
        }
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            if (ND == 2) {
                fe[2 * a] += w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
                fe[2 * a + 1] += w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
            } else {
                const double bx = b[a][0], by = b[a][1], bz = b[a][2];
                fe[3 * a] += w * (bx * sig[0] + by * sig[3 % NS] + bz * sig[5 % NS]);
                fe[3 * a + 1] += w * (by * sig[1] + bx * sig[3 % NS] + bz * sig[4 % NS]);
                fe[3 * a + 2] += w * (bz * sig[2] + by * sig[4 % NS] + bx * sig[5 % NS]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NC; ++j) d.fe[(size_t)j * E + e] = fe[j];
}

// Reaction forces (DynamicAnalysis::UpdateDomain, DynamicAnalysis.cpp:128-150;
// CentralDifference.cpp:156-171): one thread per element with a fixed node,
// Fint_e + C_e V_e + M_e A_e unfiltered (lin2DQuad4.cpp:416-434) from the
// strain displacement of the last update.  map_state = 1: J2 elements take the
// return mapping of that strain on a copy of their state (the explicit path
// updates the states at the start of the next step); 0: their stress follows
// from the updated state, K tr(eps) 1 + 2G (dev eps - eps_p) (the Newmark path
// updated them in place).  C_e = am_e M_e + ak_e K0_e with a lumped M_e.
// Gauss point q of element e with element displacement ue: shape
// derivatives b and weight w, engineering strain ev (element order: 2D xx yy
// xy, 3D xx yy zz xy yz zx), the J2 material strain Ev ([0 exx eyy 0 gxy/2 0]
// in 2D, PlasticPlaneStrainJ2.cpp:236; half shears in 3D, Plastic3DJ2.cpp:215)
// and the stress sig in the element order (J2 2D: material indices 1 2 4).
// J2 stress: map_state = 1 maps the strain on a copy of the committed state
// (explicit path: the states are updated at the start of the next step),
// 0 reads the state of the last update.
template <int ND, int NEN>
__device__ __forceinline__ void gp_state(const DevView& d, int e, int q, int ngp, const double* ue, int map_state,
                                         double (&b)[NEN][3], double& w, double ev[6], double Ev[6], double sig[6]) {
    constexpr int PER = NEN * ND + 1;
    const int E = d.nelem;
    const double* g = d.geo + ((size_t)d.egeo[e] * ngp + q) * PER;
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? g[a * ND + j] : 0.0;
    w = g[PER - 1];
#pragma unroll
    for (int i = 0; i < 6; ++i) { ev[i] = 0.0; sig[i] = 0.0; }
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        if (ND == 2) {
            ev[0] += b[a][0] * ue[2 * a]; ev[1] += b[a][1] * ue[2 * a + 1];
            ev[2] += b[a][1] * ue[2 * a] + b[a][0] * ue[2 * a + 1];
        } else {
            const double* u = ue + 3 * a;
            ev[0] += b[a][0] * u[0]; ev[1] += b[a][1] * u[1]; ev[2] += b[a][2] * u[2];
            ev[3] += b[a][1] * u[0] + b[a][0] * u[1]; ev[4] += b[a][2] * u[1] + b[a][1] * u[2];
            ev[5] += b[a][2] * u[0] + b[a][0] * u[2];
        }
    }
    if (ND == 2) { Ev[0] = 0.0; Ev[1] = ev[0]; Ev[2] = ev[1]; Ev[3] = 0.0; Ev[4] = 0.5 * ev[2]; Ev[5] = 0.0; }
    else { Ev[0] = ev[0]; Ev[1] = ev[1]; Ev[2] = ev[2]; Ev[3] = 0.5 * ev[3]; Ev[4] = 0.5 * ev[4]; Ev[5] = 0.5 * ev[5]; }
    const double c1 = d.ecoef[e], c2 = d.ecoef[(size_t)E + e], c3 = d.ecoef[2 * (size_t)E + e];
    if (d.ekind[e] == kMatElastic) {
        if (ND == 2) { sig[0] = c1 * ev[0] + c2 * ev[1]; sig[1] = c2 * ev[0] + c1 * ev[1]; sig[2] = c3 * ev[2]; }
        else {
            sig[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
            sig[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
            sig[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
            sig[3] = c3 * ev[3]; sig[4] = c3 * ev[4]; sig[5] = c3 * ev[5];
        }
        return;
    }
    double st[kJ2State];
    const double* gs = d.gstate + (size_t)q * E + e;
#pragma unroll
    for (int k2 = 0; k2 < kJ2State; ++k2) st[k2] = gs[(size_t)k2 * ngp * E];
    const double K = c1, G = c2;
    double s6[6];
    if (map_state) {
        j2_return<ND>(Ev, st, K, G, c3, d.ecoef[3 * (size_t)E + e], d.ecoef[4 * (size_t)E + e], s6);
    } else {
        const double tr = Ev[0] + Ev[1] + Ev[2];
#pragma unroll
        for (int k2 = 0; k2 < 6; ++k2)
            s6[k2] = (k2 < 3 ? K * tr : 0.0) + 2.0 * G * (Ev[k2] - (k2 < 3 ? 1.0 / 3.0 * tr : 0.0) - st[k2]);
    }
    if (ND == 2) { sig[0] = s6[1]; sig[1] = s6[2]; sig[2] = s6[4]; }
    else for (int k2 = 0; k2 < 6; ++k2) sig[k2] = s6[k2];
}

template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_react_elem(DevView d, const int32_t* __restrict__ list, int nlist,
                                                    const double* __restrict__ rm, const double* __restrict__ ram,
                                                    int ngp, int map_state, double* __restrict__ out) {
    constexpr int NC = ND * NEN;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlist) return;
    const int E = d.nelem, e = list[i];
    double ue[NC], ve[NC], fi[NC], cv[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int t = d.edof[(size_t)j * E + e];
        ue[j] = d.Us[t]; ve[j] = d.V[t]; fi[j] = 0.0; cv[j] = 0.0;
    }
    for (int q = 0; q < ngp; ++q) {
        double b[NEN][3], w, ev[6], Ev[6], sig[6];
        gp_state<ND, NEN>(d, e, q, ngp, ue, map_state, b, w, ev, Ev, sig);
        // engineering strain rate of V (the stiffness-proportional damping)
        double vv[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            if (ND == 2) {
                vv[0] += b[a][0] * ve[2 * a]; vv[1] += b[a][1] * ve[2 * a + 1];
                vv[2] += b[a][1] * ve[2 * a] + b[a][0] * ve[2 * a + 1];
            } else {
                const double* v = ve + 3 * a;
                vv[0] += b[a][0] * v[0]; vv[1] += b[a][1] * v[1]; vv[2] += b[a][2] * v[2];
                vv[3] += b[a][1] * v[0] + b[a][0] * v[1]; vv[4] += b[a][2] * v[1] + b[a][1] * v[2];
                vv[5] += b[a][2] * v[0] + b[a][0] * v[2];
            }
        }
        double sk[6] = {0, 0, 0, 0, 0, 0};
        if (d.dk0) {
            const double k1 = d.dk0[e], k2c = d.dk0[(size_t)E + e], k3 = d.dk0[2 * (size_t)E + e];
            if (ND == 2) { sk[0] = k1 * vv[0] + k2c * vv[1]; sk[1] = k2c * vv[0] + k1 * vv[1]; sk[2] = k3 * vv[2]; }
            else {
                sk[0] = k1 * vv[0] + k2c * vv[1] + k2c * vv[2];
                sk[1] = k2c * vv[0] + k1 * vv[1] + k2c * vv[2];
                sk[2] = k2c * vv[0] + k2c * vv[1] + k1 * vv[2];
                sk[3] = k3 * vv[3]; sk[4] = k3 * vv[4]; sk[5] = k3 * vv[5];
            }
        }
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            if (ND == 2) {
                fi[2 * a] += w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
                fi[2 * a + 1] += w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
                cv[2 * a] += w * (b[a][0] * sk[0] + b[a][1] * sk[2]);
                cv[2 * a + 1] += w * (b[a][1] * sk[1] + b[a][0] * sk[2]);
            } else {
                const double bx = b[a][0], by = b[a][1], bz = b[a][2];
                fi[3 * a] += w * (bx * sig[0] + by * sig[3] + bz * sig[5]);
                fi[3 * a + 1] += w * (by * sig[1] + bx * sig[3] + bz * sig[4]);
                fi[3 * a + 2] += w * (bz * sig[2] + by * sig[4] + bx * sig[5]);
                cv[3 * a] += w * (bx * sk[0] + by * sk[3] + bz * sk[5]);
                cv[3 * a + 1] += w * (by * sk[1] + bx * sk[3] + bz * sk[4]);
                cv[3 * a + 2] += w * (bz * sk[2] + by * sk[4] + bx * sk[5]);
            }
        }
    }
    double* o = out + (size_t)i * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int a = j / ND;
        const int t = d.edof[(size_t)j * E + e];
        const double c = ram[(size_t)i * NEN + a] * ve[j] + cv[j];
        o[j] = (fi[j] + c) + rm[(size_t)i * NEN + a] * d.A[t];
    }
}

// Element responses of the listed elements for the ELEMENT recorders
// (Recorder.cpp:272-323): 0 = material strain per Gauss point (elastic: the
// engineering strain, Elastic2DPlaneStrain / Elastic3DLinear::GetStrain; J2:
// the material's strain, tensor shears, PlasticPlaneStrainJ2.cpp:114-119),
// 1 = material total stress per Gauss point (GetTotalStress), 2 = internal
// force w t |J| B^T sig (lin2DQuad4.cpp:383-412, unfiltered), 3 = strain rate
// (zero for these materials, Elastic2DPlaneStrain.cpp:103-109).  out: [nlist]
// [ngp * ncomp] (0, 1, 3) or [nlist][NC] (2).
template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_elem_response(DevView d, const int32_t* __restrict__ list, int nlist,
                                                       int ngp, int map_state, int response, double* __restrict__ out) {
    constexpr int NC = ND * NEN, NS = ND == 2 ? 3 : 6;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlist) return;
    const int E = d.nelem, e = list[i];
    double ue[NC], fi[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) { ue[j] = d.Us[d.edof[(size_t)j * E + e]]; fi[j] = 0.0; }
    const bool j2 = d.ekind[e] != kMatElastic;
    for (int q = 0; q < ngp; ++q) {
        double b[NEN][3], w, ev[6], Ev[6], sig[6];
        gp_state<ND, NEN>(d, e, q, ngp, ue, map_state, b, w, ev, Ev, sig);
        double* o = out + ((size_t)i * ngp + q) * NS;
        if (response == 0) {
            if (!j2) for (int c = 0; c < NS; ++c) o[c] = ev[c];
            else if (ND == 2) { o[0] = Ev[1]; o[1] = Ev[2]; o[2] = Ev[4]; }
            else for (int c = 0; c < 6; ++c) o[c] = Ev[c];
        } else if (response == 1) {
            for (int c = 0; c < NS; ++c) o[c] = sig[c];
        } else if (response == 3) {
            for (int c = 0; c < NS; ++c) o[c] = 0.0;
        } else {
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                if (ND == 2) {
                    fi[2 * a] += w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
                    fi[2 * a + 1] += w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
                } else {
                    const double bx = b[a][0], by = b[a][1], bz = b[a][2];
                    fi[3 * a] += w * (bx * sig[0] + by * sig[3] + bz * sig[5]);
                    fi[3 * a + 1] += w * (by * sig[1] + bx * sig[3] + bz * sig[4]);
                    fi[3 * a + 2] += w * (bz * sig[2] + by * sig[4] + bx * sig[5]);
                }
            }
        }
    }
    if (response == 2)
        for (int j = 0; j < NC; ++j) out[(size_t)i * NC + j] = fi[j];
}

// R_t = (m_t A_t + sum of the listed elements' entries of t in element order
// + dashpots with a fixed node eta (V_t - V_partner)) - Fext_t(k), for the
// dofs of fixed nodes
__global__ void k_react_dof(DevView d, int k, int nr, const int32_t* __restrict__ rdof,
                            const int32_t* __restrict__ rptr, const int32_t* __restrict__ ridx,
                            const double* __restrict__ elem_out, const double* __restrict__ rnm,
                            const int32_t* __restrict__ dptr, const int32_t* __restrict__ dcol,
                            const double* __restrict__ deta, double* __restrict__ R) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    const int t = rdof[i];
    double v = rnm ? rnm[i] * d.A[t] : 0.0;
    for (int p = rptr[i]; p < rptr[i + 1]; ++p) v += elem_out[ridx[p]];
    for (int p = dptr[i]; p < dptr[i + 1]; ++p) v += deta[p] * (d.V[t] - d.V[dcol[p]]);
    R[t] = (v - fext_at(d, t, k)) - 0.0;
}

// Domain-reduction forces of step d.step[0] (lin2DQuad4.cpp:564-614,
// lin3DHexa8.cpp:661-718) for elastic elements with a lumped mass: the
// lumped mass is diagonal, so M~ (equal-condition blocks zeroed) vanishes and
// C~ = ak K~; each entry computes factor * K~ (U_o + ak V_o) as
// K (w on exterior nodes) on the boundary rows and K (w on boundary nodes) on
// the exterior rows.  Rows past the end of the signals read as zero.
template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_drm(DevView d, int ngp) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.ndrm) return;
    const int E = d.nelem, e = d.drm_elem[i], k = d.step[0];
    const double ak = d.drm_ak[i];
    double wb[NC], we[NC], yb[NC], ye[NC];
    int ext[NEN];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int a = j / ND, c = j % ND;
        const int node = d.drm_node_of[(size_t)i * NEN + a];
        const int r = d.drm_row[node];
        const bool x = d.drm_ext[node] != 0;
        ext[a] = x;
        double u = 0.0, v = 0.0;
        if (k >= 0 && k < d.drm_nt) {
            const double* row = d.drm_motion + ((size_t)r * d.drm_nt + k) * (3 * ND);
            u = row[c];
            v = row[ND + c];
        }
        const double w = (x ? -1.0 : 1.0) * (u + ak * v);
        wb[j] = x ? 0.0 : w;
        we[j] = x ? w : 0.0;
        yb[j] = 0.0; ye[j] = 0.0;
    }
    const double c1 = d.ecoef[e], c2 = d.ecoef[(size_t)E + e], c3 = d.ecoef[2 * (size_t)E + e];
    const double* g0 = d.geo + (size_t)d.egeo[e] * ngp * PER;
    for (int q = 0; q < ngp; ++q) {
        const double* g = g0 + q * PER;
        double b[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? __ldg(g + a * ND + j) : 0.0;
        const double w = __ldg(g + PER - 1);
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
            const double* uu = pass == 0 ? wb : we;
            double* yy = pass == 0 ? yb : ye;
            if (ND == 2) {
                double exx = 0, eyy = 0, gxy = 0;
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    exx += b[a][0] * uu[2 * a];
                    eyy += b[a][1] * uu[2 * a + 1];
                    gxy += b[a][1] * uu[2 * a] + b[a][0] * uu[2 * a + 1];
                }
                const double s0 = c1 * exx + c2 * eyy, s1 = c2 * exx + c1 * eyy, s2 = c3 * gxy;
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    yy[2 * a] += w * (b[a][0] * s0 + b[a][1] * s2);
                    yy[2 * a + 1] += w * (b[a][1] * s1 + b[a][0] * s2);
                }
            } else {
                double ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double ux = uu[3 * a], uy = uu[3 * a + 1], uz = uu[3 * a + 2];
                    ev[0] += b[a][0] * ux;
                    ev[1] += b[a][1] * uy;
                    ev[2] += b[a][2] * uz;
                    ev[3] += b[a][1] * ux + b[a][0] * uy;
                    ev[4] += b[a][2] * uy + b[a][1] * uz;
                    ev[5] += b[a][2] * ux + b[a][0] * uz;
                }
                double sg[6];
                sg[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
                sg[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
                sg[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
                sg[3] = c3 * ev[3]; sg[4] = c3 * ev[4]; sg[5] = c3 * ev[5];
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double bx = b[a][0], by = b[a][1], bz = b[a][2];
                    yy[3 * a] += w * (bx * sg[0] + by * sg[3] + bz * sg[5]);
                    yy[3 * a + 1] += w * (by * sg[1] + bx * sg[3] + bz * sg[4]);
                    yy[3 * a + 2] += w * (bz * sg[2] + by * sg[4] + bx * sg[5]);
                }
            }
        }
    }
    const double fac = d.drm_factor[i];
    double* out = d.drm_fe + (size_t)i * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) out[j] = fac * (ext[j / ND] ? yb[j] : ye[j]);
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

// Sum of an element-vector block (layout of fe) at node n, component c, in
// element order.
template <int ND>
__device__ __forceinline__ double gather_block(const DevView& d, const double* __restrict__ blk, int n, int c) {
    double f = 0.0;
    const int E = d.nelem;
    for (int i = d.inv_ptr[n]; i < d.inv_ptr[n + 1]; ++i) {
        const int ent = d.inv_ent[i];
        f += blk[(size_t)((ent & 7) * ND + c) * E + (ent >> 3)];
    }
    return f;
}

// Consistent mass action of every element, M_e = rho sum_q w t |J| N_a N_b on
// each displacement component (lin2DQuad4.cpp:243-285 and lin3DHexa8.cpp:
// 243-285 without the lumping branch): fe = s_e M_e x_e, or fe += when
// accumulate, with s_e = scale (+ cam * eam[e] when eam is given: the
// mass-proportional Rayleigh part of a central-difference operator).  Gauss
// points and shape functions as the element's.
template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_mass_elem(DevView d, const double* __restrict__ x, double* __restrict__ fe,
                                                    double scale, int accumulate,
                                                    const double* __restrict__ eam = nullptr, double cam = 0.0) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int E = d.nelem;
    if (e >= E) return;
    double xe[NC], y[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) { xe[j] = x[d.edof[(size_t)j * E + e]]; y[j] = 0.0; }
    const double rho = d.erho[e];
    const double* g0 = d.geo + (size_t)d.egeo[e] * NEN * PER;
    const double g = kGaussAbscissa;
    for (int q = 0; q < NEN; ++q) {
        const double r = (q & 1) ? g : -g, s2 = (q & 2) ? g : -g, t = (q & 4) ? g : -g;
        double N[NEN];
        if (ND == 2) {
            const double sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) N[a] = 0.25 * (1.0 + sr[a % 4] * r) * (1.0 + ss[a % 4] * s2);
        } else {
            const double sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                         st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) N[a] = 0.125 * (1.0 + sr[a] * r) * (1.0 + ss[a] * s2) * (1.0 + st[a] * t);
        }
        const double c = rho * g0[q * PER + PER - 1];
        double xg[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) {
            double v = 0.0;
#pragma unroll
            for (int a = 0; a < NEN; ++a) v += N[a] * xe[a * ND + k];
            xg[k] = v;
        }
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int k = 0; k < ND; ++k) y[a * ND + k] += c * N[a] * xg[k];
    }
    const double se = eam ? scale + cam * eam[e] : scale;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        double* o = fe + (size_t)j * E + e;
        *o = accumulate ? *o + se * y[j] : se * y[j];
    }
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
        // Fext - Fint + (1/dt^2 M - 1/2/dt C)(U - Up)   (CentralDifference.cpp:217)
        const double mc = d.Cd ? d.inv_dt2 * d.Md[t] - d.inv_2dt * d.Cd[t] : d.inv_dt2 * d.Md[t];
        const double R = ((fext + 0.0) - fint) + mc * (u - up);
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
        const double mc = d.Cd ? d.inv_dt2 * d.Md[t] - d.inv_2dt * d.Cd[t] : d.inv_dt2 * d.Md[t];
        d.R[t] = ((fext + 0.0) - fint) + mc * (d.U[t] - d.Up[t]);
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
    bool implicit = false;                 // tables for the Newmark path (dashpot couplings)
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    int64_t launches = 0;
    int64_t launches_last = 0;
    double* hist2[2] = {nullptr, nullptr};  // history chunks (run with a host history)
    int hist_cap = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t filled[2] = {nullptr, nullptr}, drained[2] = {nullptr, nullptr};
    // reaction tables (built on the first svl_cd_reaction call)
    bool react_ready = false;
    int r_nlist = 0, r_ndof = 0;
    const int32_t *r_list = nullptr, *r_dof = nullptr, *r_ptr = nullptr, *r_idx = nullptr;
    const int32_t *r_dptr = nullptr, *r_dcol = nullptr;
    const double *r_m = nullptr, *r_am = nullptr, *r_nm = nullptr, *r_deta = nullptr;
    double *r_out = nullptr, *r_R = nullptr;
    // element-response scratch (ELEMENT recorders), grown on demand
    int32_t* er_list = nullptr;
    double* er_out = nullptr;
    int er_cap = 0;

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
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (int i = 0; i < 2; ++i) {
            if (hist2[i]) cudaFree(hist2[i]);
            if (filled[i]) cudaEventDestroy(filled[i]);
            if (drained[i]) cudaEventDestroy(drained[i]);
        }
        if (copy_stream) cudaStreamDestroy(copy_stream);
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
    // Rayleigh damping: the mass-proportional diagonal sum_e am_e M_e and the
    // per-element ak_e-scaled initial elastic coefficients
    std::vector<double> Cdm, dk0;
    if (!m.ray.empty()) {
        rayleigh_mass_diag(m, Cdm);
        bool any_ak = false;
        for (int e = 0; e < E; ++e) any_ak |= m.ray[2 * (size_t)e + 1] != 0.0;
        if (any_ak) {
            dk0.assign((size_t)3 * E, 0.0);
            for (int e = 0; e < E; ++e) {
                const double ak = m.ray[2 * (size_t)e + 1];
                double c1 = ecoef[e], c2 = ecoef[(size_t)E + e], c3 = ecoef[2 * (size_t)E + e];
                if (ekind[e] == kMatJ2) {
                    // K 1(x)1 + 2G (I - 1/3 1(x)1), shear entries 1/2 (PlasticPlaneStrainJ2.cpp:163-180)
                    const double K = ecoef[e], G = ecoef[(size_t)E + e];
                    c1 = K * 1.0 + 2.0 * G * (1.0 - 1.0 / 3.0);
                    c2 = K * 1.0 + 2.0 * G * (0.0 - 1.0 / 3.0);
                    c3 = 2.0 * G * 0.5;
                }
                dk0[e] = ak * c1; dk0[(size_t)E + e] = ak * c2; dk0[2 * (size_t)E + e] = ak * c3;
            }
        }
    }
    // Lysmer dashpots (ZeroLength1D, C_e = eta [1 -1; -1 1]).  Explicit path:
    // the solve stays diagonal when each dashpot ties a free dof to a restrained
    // one that carries no support motion (its off-diagonal term then always
    // multiplies zero); their diagonal joins C.  Implicit path: couplings per dof.
    std::vector<int32_t> dp_ptr, dp_col;
    std::vector<double> dp_eta;
    if (!m.dp_eta.empty()) {
        if (cd->implicit) {
            dashpot_tables(m, dp_ptr, dp_col, dp_eta);
        } else {
            std::vector<signed char> kind(m.ntotal, 0), smd(m.ntotal, 0);     // 0 restrained, 1 free, 2 constrained
            for (int n = 0; n < m.nnode; ++n)
                for (int j = 0; j < m.nndof[n]; ++j)
                    if (m.fdof_all[(size_t)n * m.dstride + j] >= 0) kind[m.tdof_all[(size_t)n * m.dstride + j]] = 1;
            for (int c = 0; c < m.nconstraint; ++c) kind[m.cslave[c]] = 2;
            if (L) for (int i = 0; i < L->nsupport; ++i)
                if (L->sm_dof && L->sm_dof[i] >= 0 && L->sm_dof[i] < m.ntotal) smd[L->sm_dof[i]] = 1;
            if (Cdm.empty()) Cdm.assign(m.ntotal, 0.0);
            for (size_t i = 0; i < m.dp_eta.size(); ++i) {
                const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
                if (kind[a] == 2 || kind[b] == 2 || (kind[a] == 1 && kind[b] == 1) ||
                    (kind[a] == 0 && smd[a]) || (kind[b] == 0 && smd[b])) {
                    set_error("dashpot %zu: the explicit path needs each dashpot between a free dof and a restrained "
                              "dof without support motion (otherwise M/dt^2 + C/2dt is not diagonal)", i);
                    return SVL_ERR_UNSUPPORTED;
                }
                Cdm[a] += m.dp_eta[i];
                Cdm[b] += m.dp_eta[i];
            }
        }
    }
    // K = 1/dt/dt M + 1/2/dt C (CentralDifference.cpp:70); C diagonal here
    std::vector<double> Kd(m.ntotal);
    for (int t = 0; t < m.ntotal; ++t) Kd[t] = Cdm.empty() ? inv_dt2 * Md[t] : inv_dt2 * Md[t] + 1.0 / 2.0 / dt * Cdm[t];
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
    LoadTables lt;
    TRY(build_load_tables(m, L, lt));
    cd->has_sm = lt.has_sm;
    const std::vector<int32_t>& s_ptr = lt.s_ptr; const std::vector<double>& s_val = lt.s_val;
    const std::vector<int32_t>& ld_ptr = lt.ld_ptr; const std::vector<int32_t>& ld_ser = lt.ld_ser;
    const std::vector<double>& ld_coef = lt.ld_coef;
    const std::vector<int32_t>& sm_ptr = lt.sm_ptr; const std::vector<int32_t>& sm_ser = lt.sm_ser;
    const std::vector<double>& sm_fac = lt.sm_fac;
    // --- domain-reduction entries ----------------------------------------------
    std::vector<int32_t> drm_elem, drm_node_of, drm_row, drm_ext, drm_ptr, drm_idx;
    std::vector<double> drm_factor, drm_ak, drm_motion;
    int drm_nt = 0;
    if (L && L->ndrm > 0) {
        if (!L->drm_elem || !L->drm_factor || !L->drm_node_row || !L->drm_node_ext || !L->drm_motion || L->drm_nt <= 0) {
            set_error("domain-reduction arrays are NULL or drm_nt <= 0"); return SVL_ERR_INVALID;
        }
        drm_nt = L->drm_nt;
        drm_row.assign(L->drm_node_row, L->drm_node_row + m.nnode);
        drm_ext.assign(L->drm_node_ext, L->drm_node_ext + m.nnode);
        int nblk = 0;
        for (int r : drm_row) nblk = std::max(nblk, r + 1);
        drm_motion.assign(L->drm_motion, L->drm_motion + (size_t)nblk * drm_nt * 3 * nd);
        drm_ptr.assign(m.ntotal + 1, 0);
        for (int i = 0; i < L->ndrm; ++i) {
            const int e = L->drm_elem[i];
            if (e < 0 || e >= E) { set_error("DRM entry %d: element %d out of range", i, e); return SVL_ERR_INVALID; }
            if (ekind[e] != kMatElastic) { set_error("DRM element %d: elastic materials only", e); return SVL_ERR_UNSUPPORTED; }
            drm_elem.push_back(e);
            drm_factor.push_back(L->drm_factor[i]);
            drm_ak.push_back(m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1]);
            for (int a = 0; a < nen; ++a) {
                const int n = m.conn[(size_t)e * nen + a];
                if (drm_row[n] < 0) { set_error("DRM element %d: node %d has no free-field motion", e, n); return SVL_ERR_INVALID; }
                drm_node_of.push_back(n);
                for (int c = 0; c < nd; ++c) drm_ptr[m.tdof[(size_t)n * nd + c] + 1]++;
            }
        }
        for (int t = 0; t < m.ntotal; ++t) drm_ptr[t + 1] += drm_ptr[t];
        drm_idx.resize(drm_ptr.back());
        std::vector<int32_t> fill(drm_ptr.begin(), drm_ptr.end() - 1);
        for (int i = 0; i < L->ndrm; ++i) {
            const int e = drm_elem[i];
            for (int a = 0; a < nen; ++a)
                for (int c = 0; c < nd; ++c)
                    drm_idx[fill[m.tdof[(size_t)m.conn[(size_t)e * nen + a] * nd + c]]++] = i * nc + a * nd + c;
        }
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
    if (!m.lumped) {
        // consistent mass (implicit path): the element masses act through
        // k_mass_elem; the diagonal keeps the nodal (point) masses only
        for (int t = 0; t < m.ntotal; ++t)
            Md[t] = (!m.nodemass.empty() && std::fabs(m.nodemass[t]) > cd->opts.mtol) ? m.nodemass[t] : 0.0;
        std::vector<double> erho(m.nelem);
        for (int e = 0; e < m.nelem; ++e) erho[e] = m.param(e)[2];
        TRY(cd->upload(erho, &d.erho));
    }
    TRY(cd->upload(Md, &d.Md));
    TRY(cd->upload(kinv, &d.kinv));
    TRY(cd->upload(Kd, &d.Kd));
    if (!Cdm.empty()) TRY(cd->upload(Cdm, &d.Cd));
    if (!dp_eta.empty()) {
        TRY(cd->upload(dp_ptr, &d.dp_ptr)); TRY(cd->upload(dp_col, &d.dp_col)); TRY(cd->upload(dp_eta, &d.dp_eta));
    }
    if (!drm_elem.empty()) {
        d.ndrm = (int)drm_elem.size();
        d.drm_nt = drm_nt;
        TRY(cd->upload(drm_elem, &d.drm_elem)); TRY(cd->upload(drm_factor, &d.drm_factor));
        TRY(cd->upload(drm_ak, &d.drm_ak)); TRY(cd->upload(drm_node_of, &d.drm_node_of));
        TRY(cd->upload(drm_row, &d.drm_row)); TRY(cd->upload(drm_ext, &d.drm_ext));
        TRY(cd->upload(drm_motion, &d.drm_motion));
        TRY(cd->upload(drm_ptr, &d.drm_ptr)); TRY(cd->upload(drm_idx, &d.drm_idx));
        TRY(cd->zeros((size_t)d.ndrm * nc, &d.drm_fe));
    }
    if (!dk0.empty()) TRY(cd->upload(dk0, &d.dk0));
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
// 3 free, 4 update) on the buffers of view `d` (the handle's own view, or
// the no-alloc copy whose element force block is the static scratch);
// returns SVL_OK, or 1 when the kind is not used.
static int cd_launch_kind(svl_cd* cd, const DevView& d, int kind) {
    const HostModel& m = cd->m;
    const int eb = 128, nb = 256;
    const int eg = (m.nelem + eb - 1) / eb, ng = (m.nnode + nb - 1) / nb, fg = (m.nfree + nb - 1) / nb;
    switch (kind) {
    case 0:
        // The strain displacement of the previous step (U + T du, without the
        // support-motion increment) feeds the material update.
        if (m.ndim == 2) k_element<2, 4><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
        else k_element<3, 8><<<eg, eb, 0, cd->stream>>>(d, d.Us, m.ngp, 1);
        if (d.ndrm > 0) {                   // domain-reduction forces of this step
            const int gd = (d.ndrm + 127) / 128;
            if (m.ndim == 2) k_drm<2, 4><<<gd, 128, 0, cd->stream>>>(d, m.ngp);
            else k_drm<3, 8><<<gd, 128, 0, cd->stream>>>(d, m.ngp);
            ++cd->launches;
        }
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

static int cd_launch_step_view(svl_cd* cd, const DevView& d) {
    for (int kind = 0; kind < 5; ++kind) {
        const int st = cd_launch_kind(cd, d, kind);
        if (st != SVL_OK && st != 1) return st;
    }
    return SVL_OK;
}

static int cd_launch_step(svl_cd* cd) { return cd_launch_step_view(cd, cd->d); }

// kernels per step: element forces (+ domain-reduction forces), then the
// node kernel, or residual / free-dof solve / update with constraints
static int launches_per_step(const svl_cd* cd) {
    return (cd->identity_T ? 2 : (cd->m.nfree > 0 ? 4 : 3)) + (cd->d.ndrm > 0 ? 1 : 0);
}

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

static int cd_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_cd_opts* opts, svl_cd** out,
                     bool implicit);

int svl_cd_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_cd_opts* opts, svl_cd** out) {
    return cd_create(model, loads, opts, out, false);
}

}  // extern "C"

// implicit: the model serves the Newmark path, whose solve takes any damping
static int cd_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_cd_opts* opts, svl_cd** out,
                     bool implicit) {
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
    if (!cd->m.lumped && !implicit) {
        delete cd;
        set_error("the diagonal explicit path needs a lumped mass (massform LUMPED); a consistent mass is served by "
                  "svl_nm_create with integrator SVL_NM_CENTRAL_DIFFERENCE");
        return SVL_ERR_UNSUPPORTED;
    }
    if (cd->m.has_pml()) {
        delete cd;
        set_error("PML elements are served by svl_xnm_create (ExtendedNewmarkBeta)");
        return SVL_ERR_UNSUPPORTED;
    }
    if (!implicit)
        for (size_t e = 0; e < cd->m.ray.size() / 2; ++e)
            if (cd->m.ray[2 * e + 1] != 0.0) {
                delete cd;
                set_error("element %zu: stiffness-proportional Rayleigh damping (ak) makes the central-difference "
                          "effective stiffness non-diagonal; served by svl_nm_create with integrator "
                          "SVL_NM_CENTRAL_DIFFERENCE", e);
                return SVL_ERR_UNSUPPORTED;
            }
    if (cudaStreamCreateWithFlags(&cd->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete cd; set_error("cudaStreamCreate failed"); return SVL_ERR_CUDA;
    }
    cd->implicit = implicit;
    int st = cd_setup(cd, loads);
    if (st != SVL_OK) { delete cd; return st; }
    *out = cd;
    return SVL_OK;
}

extern "C" {

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
    if (U_hist && nsteps > 0) {
        // two device history chunks: the copy of chunk c (copy stream)
        // overlaps the stepping of chunk c + 1
        const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(nsteps, (int64_t)(256ll << 20) / ((int64_t)nt * 8)));
        if (cd->hist_cap < chunk) {
            CUDA_TRY(cudaStreamSynchronize(cd->stream));
            if (cd->copy_stream) CUDA_TRY(cudaStreamSynchronize(cd->copy_stream));
            for (int i = 0; i < 2; ++i) {
                if (cd->hist2[i]) cudaFree(cd->hist2[i]);
                cd->hist2[i] = nullptr;
            }
            cd->hist_cap = 0;
            for (int i = 0; i < 2; ++i)
                if (cudaMalloc(&cd->hist2[i], (size_t)chunk * nt * sizeof(double)) != cudaSuccess) {
                    set_error("history buffer allocation failed"); return SVL_ERR_NOMEM;
                }
            if (!cd->copy_stream) {
                CUDA_TRY(cudaStreamCreateWithFlags(&cd->copy_stream, cudaStreamNonBlocking));
                for (int i = 0; i < 2; ++i) {
                    CUDA_TRY(cudaEventCreateWithFlags(&cd->filled[i], cudaEventDisableTiming));
                    CUDA_TRY(cudaEventCreateWithFlags(&cd->drained[i], cudaEventDisableTiming));
                    CUDA_TRY(cudaEventRecord(cd->drained[i], cd->copy_stream));
                }
            }
            cd->hist_cap = chunk;
        }
        auto fill = [&](int s0, int slot) -> int {
            const int n = std::min(chunk, nsteps - s0);
            CUDA_TRY(cudaStreamWaitEvent(cd->stream, cd->drained[slot], 0));
            for (int i = 0; i < n; ++i) {
                TRY(cd_launch_step(cd));
                CUDA_TRY(cudaMemcpyAsync(cd->hist2[slot] + (size_t)i * nt, cd->d.U, sizeof(double) * nt, cudaMemcpyDeviceToDevice, cd->stream));
            }
            CUDA_TRY(cudaEventRecord(cd->filled[slot], cd->stream));
            return SVL_OK;
        };
        const int nch = (nsteps + chunk - 1) / chunk;
        TRY(fill(0, 0));
        for (int c = 0; c < nch; ++c) {
            const int s0 = c * chunk, n = std::min(chunk, nsteps - s0), slot = c & 1;
            if (c + 1 < nch) TRY(fill(s0 + chunk, slot ^ 1));
            CUDA_TRY(cudaStreamWaitEvent(cd->copy_stream, cd->filled[slot], 0));
            CUDA_TRY(cudaMemcpyAsync(U_hist + (size_t)s0 * nt, cd->hist2[slot], sizeof(double) * nt * n, cudaMemcpyDeviceToHost, cd->copy_stream));
            CUDA_TRY(cudaEventRecord(cd->drained[slot], cd->copy_stream));
        }
        CUDA_TRY(cudaStreamSynchronize(cd->copy_stream));
    } else if (!U_hist) {
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
            const int st = cd_launch_kind(cd, cd->d, kind);
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

}  // extern "C"

// Reaction forces after step k (see k_react_elem); map_state as there.
static int cd_reaction(svl_cd* cd, int k, int map_state, double* R) {
    const HostModel& m = cd->m;
    const int nen = m.nen, nd = m.ndim, E = m.nelem, NC = nen * nd;
    if (!cd->react_ready) {
        std::vector<char> fixed(m.nnode, 0);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j)
                if (m.fdof_all[(size_t)n * m.dstride + j] == -1) fixed[n] = 1;
        std::vector<int32_t> list, pos_of(E, -1);
        for (int e = 0; e < E; ++e) {
            bool hf = false;
            for (int a = 0; a < nen; ++a) hf = hf || fixed[m.conn[(size_t)e * nen + a]];
            if (hf) { pos_of[e] = (int32_t)list.size(); list.push_back(e); }
        }
        std::vector<double> diag;
        element_lumped_masses(m, diag);
        std::vector<double> rm((size_t)list.size() * nen), ram(rm.size());
        for (size_t i = 0; i < list.size(); ++i) {
            const int e = list[i];
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e];
            for (int a = 0; a < nen; ++a) {
                rm[i * nen + a] = diag[((size_t)e * nen + a) * nd];
                ram[i * nen + a] = am * rm[i * nen + a];
            }
        }
        // dofs of fixed nodes, their element entries (element order) and dashpots
        std::vector<int32_t> rdof, dof_pos(m.ntotal, -1), node_of(m.ntotal, -1);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j) node_of[m.tdof_all[(size_t)n * m.dstride + j]] = n;
        for (int n = 0; n < m.nnode; ++n)
            if (fixed[n])
                for (int j = 0; j < m.nndof[n]; ++j) {
                    const int t = m.tdof_all[(size_t)n * m.dstride + j];
                    dof_pos[t] = (int32_t)rdof.size();
                    rdof.push_back(t);
                }
        const int nr = (int)rdof.size();
        std::vector<std::vector<int32_t>> ent(nr);
        for (size_t i = 0; i < list.size(); ++i) {
            const int e = list[i];
            for (int a = 0; a < nen; ++a)
                for (int c = 0; c < nd; ++c) {
                    const int t = m.tdof[(size_t)m.conn[(size_t)e * nen + a] * nd + c];
                    if (dof_pos[t] >= 0) ent[dof_pos[t]].push_back((int32_t)(i * NC + a * nd + c));
                }
        }
        std::vector<int32_t> rptr(nr + 1, 0), ridx;
        for (int i = 0; i < nr; ++i) { ridx.insert(ridx.end(), ent[i].begin(), ent[i].end()); rptr[i + 1] = (int32_t)ridx.size(); }
        std::vector<std::vector<std::pair<int32_t, double>>> dps(nr);
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
            if (!fixed[node_of[a]] && !fixed[node_of[b]]) continue;
            if (dof_pos[a] >= 0) dps[dof_pos[a]].push_back({b, m.dp_eta[i]});
            if (dof_pos[b] >= 0) dps[dof_pos[b]].push_back({a, m.dp_eta[i]});
        }
        std::vector<int32_t> dptr(nr + 1, 0), dcol;
        std::vector<double> deta, rnm;
        for (int i = 0; i < nr; ++i) {
            for (auto& pr : dps[i]) { dcol.push_back(pr.first); deta.push_back(pr.second); }
            dptr[i + 1] = (int32_t)dcol.size();
        }
        if (!m.nodemass.empty()) { rnm.resize(nr); for (int i = 0; i < nr; ++i) rnm[i] = m.nodemass[rdof[i]]; }
        TRY(cd->upload(list, &cd->r_list)); TRY(cd->upload(rm, &cd->r_m)); TRY(cd->upload(ram, &cd->r_am));
        TRY(cd->upload(rdof, &cd->r_dof)); TRY(cd->upload(rptr, &cd->r_ptr)); TRY(cd->upload(ridx, &cd->r_idx));
        TRY(cd->upload(dptr, &cd->r_dptr)); TRY(cd->upload(dcol, &cd->r_dcol)); TRY(cd->upload(deta, &cd->r_deta));
        if (!rnm.empty()) TRY(cd->upload(rnm, &cd->r_nm));
        TRY(cd->zeros((size_t)list.size() * NC, &cd->r_out));
        TRY(cd->zeros((size_t)m.ntotal, &cd->r_R));
        cd->r_nlist = (int)list.size();
        cd->r_ndof = nr;
        cd->react_ready = true;
    }
    if (cd->r_nlist > 0) {
        const int g = (cd->r_nlist + 127) / 128;
        if (nd == 2) k_react_elem<2, 4><<<g, 128, 0, cd->stream>>>(cd->d, cd->r_list, cd->r_nlist, cd->r_m, cd->r_am, m.ngp, map_state, cd->r_out);
        else k_react_elem<3, 8><<<g, 128, 0, cd->stream>>>(cd->d, cd->r_list, cd->r_nlist, cd->r_m, cd->r_am, m.ngp, map_state, cd->r_out);
    }
    if (cd->r_ndof > 0)
        k_react_dof<<<(cd->r_ndof + 255) / 256, 256, 0, cd->stream>>>(cd->d, k, cd->r_ndof, cd->r_dof, cd->r_ptr, cd->r_idx,
                                                                     cd->r_out, cd->r_nm, cd->r_dptr, cd->r_dcol,
                                                                     cd->r_deta, cd->r_R);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(R, cd->r_R, sizeof(double) * m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

extern "C" {

int svl_cd_reaction(svl_cd* cd, int32_t k, double* R) {
    if (!cd || !R) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    return cd_reaction(cd, k, 1, R);
}

// Element responses after the last step (see k_elem_response); map_state as
// in cd_reaction.
static int cd_element_response(svl_cd* cd, int map_state, int32_t response, int32_t nlist, const int32_t* elems,
                               double* out) {
    const HostModel& m = cd->m;
    if (response < 0 || response > 3 || nlist < 0 || (nlist > 0 && (!elems || !out))) {
        set_error("bad argument"); return SVL_ERR_INVALID;
    }
    for (int i = 0; i < nlist; ++i)
        if (elems[i] < 0 || elems[i] >= m.nelem) { set_error("element %d out of range", elems[i]); return SVL_ERR_INVALID; }
    if (nlist == 0) return SVL_OK;
    const int nd = m.ndim, nen = m.nen, per = response == 2 ? nen * nd : m.ngp * (nd == 2 ? 3 : 6);
    if (cd->er_cap < nlist) {
        TRY(cd->zeros((size_t)nlist, &cd->er_list));
        TRY(cd->zeros((size_t)nlist * 48, &cd->er_out));
        cd->er_cap = nlist;
    }
    CUDA_TRY(cudaMemcpyAsync(cd->er_list, elems, sizeof(int32_t) * nlist, cudaMemcpyHostToDevice, cd->stream));
    const int g = (nlist + 127) / 128;
    if (nd == 2) k_elem_response<2, 4><<<g, 128, 0, cd->stream>>>(cd->d, cd->er_list, nlist, m.ngp, map_state, response, cd->er_out);
    else k_elem_response<3, 8><<<g, 128, 0, cd->stream>>>(cd->d, cd->er_list, nlist, m.ngp, map_state, response, cd->er_out);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, cd->er_out, sizeof(double) * (size_t)nlist * per, cudaMemcpyDeviceToHost, cd->stream));
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    return SVL_OK;
}

int svl_cd_element_response(svl_cd* cd, int32_t response, int32_t nlist, const int32_t* elems, double* out) {
    if (!cd) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    return cd_element_response(cd, 1, response, nlist, elems, out);
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
    const int64_t l0 = cd->launches;
    k_set_step<<<1, 1, 0, cd->stream>>>(d.step, k_first - 1);
    CUDA_TRY(cudaGetLastError());
    ++cd->launches;
    // the launch sequence of svl_cd_run, kernel for kernel, on the swapped view
    for (int s = 0; s < nsteps; ++s) TRY(cd_launch_step_view(cd, d));
    cd->launches_last = cd->launches - l0;
    if (d_U_out)
        CUDA_TRY(cudaMemcpyAsync(d_U_out, d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToDevice, cd->stream));
    return SVL_OK;
}

// ===========================================================================
// Implicit Newmark (average acceleration, beta = 1/4, gamma = 1/2) with the
// Linear algorithm and a matrix-free Jacobi-preconditioned conjugate-gradient
// solve of the effective stiffness (FP64).
//
// Per step (RP/10-Integrators/03-Newmark/NewmarkBeta.cpp:117-141, 198-235;
// ExtendedNewmarkBeta with G = 0):
//   Feff = T^T [Fext - Fint + M (4/dt V + A)]
//   Keff = T^T (K + 4/dt^2 M) T          (applied matrix-free: element
//                                          stiffness action + lumped mass)
//   solve Keff du = Feff                    (EigenSolver / PetscSolver.cc:53-150 KSPCG)
//   dU = T du;  U += dU;  A = 4/dt^2 dU - 4/dt V - A;  V = 2/dt dU - V
// The solve stops on the true relative residual |Feff - Keff du| / |Feff|.
// Dot products are reduced in a fixed order (block partials, then one block),
// so runs are bitwise reproducible.

namespace {

constexpr int kDotBlocks = 304;         // 2 x 152 SMs, fixed so the reduction order is fixed
constexpr int kDotThreads = 256;

// partial[blockIdx] = sum over a fixed strided subset of a[i]*b[i]
__global__ void __launch_bounds__(kDotThreads) k_dot_partial(const double* __restrict__ a, const double* __restrict__ b,
                                                             int n, double* __restrict__ partial) {
    __shared__ double sh[kDotThreads / 32];
    double s = 0.0;
    for (int i = blockIdx.x * kDotThreads + threadIdx.x; i < n; i += kDotBlocks * kDotThreads) s += a[i] * b[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < kDotThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

// out[slot] = sum of the kDotBlocks partials (one block, fixed order)
__global__ void k_dot_final(const double* __restrict__ partial, double* out, int slot) {
    __shared__ double sh[kDotThreads / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < kDotBlocks; i += kDotThreads) s += partial[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < kDotThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) out[slot] = t;
    }
}

// Scalars of the PCG, in device memory: 0 rz, 1 pq, 2 rr, 3 bb, 4 rz_new
enum { S_RZ = 0, S_PQ = 1, S_RR = 2, S_BB = 3, S_RZN = 4, S_NSCAL = 8 };

// Effective force per node (identity T): b_f = (Fext - Fint) + M (4/dt V + A)
template <int ND>
__global__ void __launch_bounds__(256) k_nm_rhs(DevView d, double* __restrict__ b, double c_v,
                                                const double* __restrict__ dUf, double c_m) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        if (f < 0) continue;
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        // Fext - Fint + M (4/dt V + A - 4/dt^2 dU)   (NewmarkBeta.cpp:215, C = 0)
        const double w = dUf ? (c_v * d.V[t] + d.A[t]) - c_m * dUf[f] : c_v * d.V[t] + d.A[t];
        b[f] = ((fext + 0.0) - fint) + d.Md[t] * w;
        if (d.fem) b[f] += gather_block<ND>(d, d.fem, n, c);    // consistent mass: sum_e M_e w_e
    }
}

// w = 4/dt V + A (- 4/dt^2 dU on free dofs): the vector the effective force's
// mass term multiplies (NewmarkBeta.cpp:215)
__global__ void k_nm_wvec(DevView d, const double* __restrict__ dUf, double c_v, double c_m, double* __restrict__ w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    const int f = d.tfree[t];
    w[t] = (dUf && f >= 0) ? (c_v * d.V[t] + d.A[t]) - c_m * dUf[f] : c_v * d.V[t] + d.A[t];
}

// Us = U + dU on total dofs (identity T) for the state update of a Newton iteration
__global__ void k_nm_us(DevView d, const double* __restrict__ dUf) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    const int f = d.tfree[t];
    d.Us[t] = d.U[t] + (f >= 0 ? dUf[f] : 0.0);
}

// --- implicit path with a general T (constraints) and support motion -----
// pt = T pf (rows of T over total dofs)
__global__ void k_nmg_expand(DevView d, const double* __restrict__ pf, double* __restrict__ pt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    double v = 0.0;
    for (int i = d.T_ptr[t]; i < d.T_ptr[t + 1]; ++i) v += d.T_val[i] * pf[d.T_col[i]];
    pt[t] = v;
}

// sum over the dashpots at dof t of eta (x_t - x_partner)
__device__ __forceinline__ double dashpot_sum(const DevView& d, int t, const double* __restrict__ x) {
    double v = 0.0;
    const double xt = x[t];
    for (int i = d.dp_ptr[t]; i < d.dp_ptr[t + 1]; ++i) v += d.dp_eta[i] * (xt - x[d.dp_col[i]]);
    return v;
}

// ft = sum_e K_e p_e + c_m M p (+ c_c C p) on total dofs (ordered gather of d.fe)
template <int ND>
__global__ void __launch_bounds__(256) k_nmg_total(DevView d, const double* __restrict__ pt, double* __restrict__ ft,
                                                   double c_m, double c_c) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        double v = gather_fint<ND>(d, n, c) + c_m * d.Md[t] * pt[t];
        if (d.Cd) v += c_c * d.Cd[t] * pt[t];
        if (d.dp_ptr) v += c_c * dashpot_sum(d, t, pt);
        ft[t] = v;
    }
}

// w = V - 2/dt dU_t: the vector the damping acts on in the effective force
__global__ void k_nmg_wdamp(DevView d, const double* __restrict__ dUt, double c_u, double* __restrict__ w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < d.ntotal) w[t] = d.V[t] - c_u * dUt[t];
}

// w = 4/dt V + A - 4/dt^2 dU_t: the vector the mass acts on in the effective
// force (NewmarkBeta.cpp:215), for a consistent mass on the general path
__global__ void k_nmg_wmass(DevView d, const double* __restrict__ dUt, double c_v, double c_m, double* __restrict__ w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < d.ntotal) w[t] = (c_v * d.V[t] + d.A[t]) - c_m * dUt[t];
}

// ft += sum_e blk_e per total dof (element order)
template <int ND>
__global__ void __launch_bounds__(256) k_nmg_addblk(DevView d, const double* __restrict__ blk, double* __restrict__ ft) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) ft[d.ntdof[n * ND + c]] += gather_block<ND>(d, blk, n, c);
}

// ft += C w: the element damping vectors in d.fe (gather_fe) plus the
// mass-proportional diagonal
template <int ND>
__global__ void __launch_bounds__(256) k_nmg_damp(DevView d, const double* __restrict__ w, double* __restrict__ ft,
                                                  int gather_fe) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        double v = gather_fe ? gather_fint<ND>(d, n, c) : 0.0;
        if (d.Cd) v += d.Cd[t] * w[t];
        if (d.dp_ptr) v += dashpot_sum(d, t, w);
        ft[t] += v;
    }
}

// q = T^T ft (optionally minus T^T lg)
__global__ void k_nmg_reduce(DevView d, const double* __restrict__ ft, const double* __restrict__ lg,
                             double* __restrict__ q) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= d.nfree) return;
    double v = 0.0, w = 0.0;
    for (int i = d.TT_ptr[f]; i < d.TT_ptr[f + 1]; ++i) {
        v += d.TT_val[i] * ft[d.TT_row[i]];
        if (lg) w += d.TT_val[i] * lg[d.TT_row[i]];
    }
    q[f] = lg ? v - w : v;
}

// total-dof effective force Fext - Fint + M (4/dt V + A - 4/dt^2 dU_t)
template <int ND>
__global__ void __launch_bounds__(256) k_nmg_rhs(DevView d, double* __restrict__ ft, const double* __restrict__ dUt,
                                                 double c_v, double c_m) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        const double w = (c_v * d.V[t] + d.A[t]) - c_m * dUt[t];
        ft[t] = ((fext + 0.0) - fint) + d.Md[t] * w;
    }
}

// support-motion increment of step k - 1 (NewmarkBeta.cpp:186) on total dofs
__global__ void k_nmg_sm(DevView d, double* __restrict__ sm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    sm[t] = sm_at(d, t, d.step[0] - 1);
}

// Us = U + dU_t;  at the end of the step U += dU_t + SM, A and V from dU_t
template <int ND>
__global__ void __launch_bounds__(256) k_nmg_update(DevView d, const double* __restrict__ dUt,
                                                    const double* __restrict__ sm, double c_a, double c_av,
                                                    double c_vv, int* flag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double dU = dUt[t];
        const double u0 = d.U[t];
        const double u = u0 + (dU + sm[t]);
        d.U[t] = u;
        d.Us[t] = u0 + dU;          // states follow U + T du, without the support motion
        d.A[t] = c_a * dU - c_av * d.V[t] - d.A[t];
        d.V[t] = c_vv * dU - d.V[t];
        bad |= !isfinite(u);
    }
    if (bad) atomicOr(flag, 1);
}

__global__ void k_nmg_us(DevView d, const double* __restrict__ dUt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < d.ntotal) d.Us[t] = d.U[t] + dUt[t];
}

__global__ void k_axpy1(double* __restrict__ y, const double* __restrict__ x, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += x[i];
}

// q = Keff p: scatter p to total dofs (free part), element stiffness action done by
// k_element on that vector, then q_f = sum_e (K_e p_e) + 4/dt^2 M p (identity T).
__global__ void k_nm_expand(DevView d, const double* __restrict__ pf, double* __restrict__ pt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    const int f = d.tfree[t];
    pt[t] = f >= 0 ? pf[f] : 0.0;
}

template <int ND>
__global__ void __launch_bounds__(256) k_nm_apply(DevView d, const double* __restrict__ pt, double* __restrict__ q, double c_m) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        if (f < 0) continue;
        q[f] = gather_fint<ND>(d, n, c) + c_m * d.Md[t] * pt[t];
    }
}

// ---- single-precision operator of the inner solve iterations ----------------
// q = (K + 4/dt^2 M) v for elastic models without damping or constraints:
// the element action in FP32, one thread per (element, Gauss point) on float
// geometry tables, node values shared by warp shuffles, the element vector
// summed by a butterfly over the element's lanes; the per-node gather sums
// the float element entries in element order and adds the lumped-mass term
// in FP64.  The solves confirm every answer with the FP64 operator (true
// residual) and restart from it, so the result keeps the FP64 tolerance.
__global__ void k_nm_expand_f(DevView d, const double* __restrict__ pf, double* __restrict__ pt,
                              float* __restrict__ pt_f) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    const int f = d.tfree[t];
    const double v = f >= 0 ? pf[f] : 0.0;
    pt[t] = v;
    pt_f[t] = (float)v;
}

template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_nm_op_f(DevView d, const float* __restrict__ geo_f,
                                                  const float* __restrict__ coef_f, const float* __restrict__ pt,
                                                  float* __restrict__ fe_f) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int E = d.nelem;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int e = gtid / NEN, q = gtid % NEN;
    const bool valid = e < E;
    const int ec = valid ? e : E - 1;
    const int lane = threadIdx.x & 31, base = lane - q;
    float pq[ND];
#pragma unroll
    for (int c = 0; c < ND; ++c) pq[c] = pt[d.edof[(size_t)(q * ND + c) * E + ec]];
    const float c1 = coef_f[ec], c2 = coef_f[(size_t)E + ec], c3 = coef_f[2 * (size_t)E + ec];
    const float* g = geo_f + ((size_t)d.egeo[ec] * NEN + q) * PER;
    float b[NEN][3];
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? g[a * ND + j] : 0.0f;
    const float w = g[PER - 1];
    float ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        float ua[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < ND; ++c) ua[c] = __shfl_sync(0xffffffffu, pq[c], base + a);
        if (ND == 2) {
            ev[0] += b[a][0] * ua[0];
            ev[1] += b[a][1] * ua[1];
            ev[2] += b[a][1] * ua[0] + b[a][0] * ua[1];
        } else {
            ev[0] += b[a][0] * ua[0];
            ev[1] += b[a][1] * ua[1];
            ev[2] += b[a][2] * ua[2];
            ev[3] += b[a][1] * ua[0] + b[a][0] * ua[1];
            ev[4] += b[a][2] * ua[1] + b[a][1] * ua[2];
            ev[5] += b[a][2] * ua[0] + b[a][0] * ua[2];
        }
    }
    float sig[6];
    if (ND == 2) {
        sig[0] = c1 * ev[0] + c2 * ev[1]; sig[1] = c2 * ev[0] + c1 * ev[1]; sig[2] = c3 * ev[2];
    } else {
        sig[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
        sig[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
        sig[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
        sig[3] = c3 * ev[3]; sig[4] = c3 * ev[4]; sig[5] = c3 * ev[5];
    }
    float y[NC];
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        if (ND == 2) {
            y[2 * a] = w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
            y[2 * a + 1] = w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
        } else {
            const float bx = b[a][0], by = b[a][1], bz = b[a][2];
            y[3 * a] = w * (bx * sig[0] + by * sig[3] + bz * sig[5]);
            y[3 * a + 1] = w * (by * sig[1] + bx * sig[3] + bz * sig[4]);
            y[3 * a + 2] = w * (bz * sig[2] + by * sig[4] + bx * sig[5]);
        }
    }
#pragma unroll
    for (int off = 1; off < NEN; off <<= 1)
#pragma unroll
        for (int j = 0; j < NC; ++j) y[j] += __shfl_xor_sync(0xffffffffu, y[j], off);
    if (!valid) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        float mine = 0.f;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
            if (a == q) mine = y[a * ND + c];
        fe_f[(size_t)(q * ND + c) * E + e] = mine;
    }
}

template <int ND>
__global__ void __launch_bounds__(256) k_nm_apply_f(DevView d, const float* __restrict__ fe_f,
                                                     const double* __restrict__ pt, double* __restrict__ q, double c_m) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int E = d.nelem;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        if (f < 0) continue;
        float s = 0.f;
        for (int i = d.inv_ptr[n]; i < d.inv_ptr[n + 1]; ++i) {
            const int ent = d.inv_ent[i];
            s += fe_f[(size_t)((ent & 7) * ND + c) * E + (ent >> 3)];
        }
        q[f] = (double)s + c_m * d.Md[t] * pt[t];
    }
}

// x += alpha p; r -= alpha q; z = Dinv r   (alpha = rz / pq)
__global__ void k_pcg_xr(const double* __restrict__ sc, const double* __restrict__ p, const double* __restrict__ q,
                         const double* __restrict__ dinv, double* x, double* r, double* z, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double alpha = sc[S_RZ] / sc[S_PQ];
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    z[i] = dinv[i] * ri;
}

// p = z + beta p (beta = rz_new / rz), then rz = rz_new
__global__ void k_pcg_p(double* sc, const double* __restrict__ z, double* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = sc[S_RZN] / sc[S_RZ];
    if (i < n) p[i] = z[i] + beta * p[i];
}
__global__ void k_pcg_roll(double* sc) { sc[S_RZ] = sc[S_RZN]; }

// r = b - q; z = Dinv r; p = z   (start / residual replacement)
__global__ void k_pcg_reset(const double* __restrict__ b, const double* __restrict__ q, const double* __restrict__ dinv,
                            double* r, double* z, double* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ri = b[i] - q[i];
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    p[i] = zi;
}

// ---- central difference with a non-diagonal effective stiffness ------------
// K = M/dt^2 + C/2dt with a consistent mass and/or C containing ak_e K0_e
// (CentralDifference.cpp:64-151), identity T, no support motion.  The element
// parts of K p (or of (M/dt^2 - C/2dt) w) arrive in an element block `blk`
// (k_mass_elem with the per-element Rayleigh scale, k_element_tan with the
// ak-scaled initial elastic coefficients); the diagonal parts are the nodal
// or lumped masses Md and, with a lumped mass, the mass-proportional diagonal
// Cd.
__global__ void k_ncd_w(DevView d, double* __restrict__ w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < d.ntotal) w[t] = d.U[t] - d.Up[t];
}

// q_f = sum_e blk_e + (c_m Md + c_c Cd) p on free dofs
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_apply(DevView d, const double* __restrict__ blk, const double* __restrict__ pt,
                                                   double* __restrict__ q, double c_m, double c_c,
                                                   const double* __restrict__ Cd) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        if (f < 0) continue;
        const double dg = Cd ? c_m * d.Md[t] + c_c * Cd[t] : c_m * d.Md[t];
        double v = (blk ? gather_block<ND>(d, blk, n, c) : 0.0) + dg * pt[t];
        if (d.dp_ptr) v += c_c * dashpot_sum(d, t, pt);
        q[f] = v;
    }
}

// b_f = Fext - Fint + (M/dt^2 - C/2dt)(U - Up)   (CentralDifference.cpp:217):
// Fint gathered from d.fe, the element part of the last term from blk
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_rhs(DevView d, const double* __restrict__ blk, const double* __restrict__ w,
                                                 double* __restrict__ b, double c_m, double c_c,
                                                 const double* __restrict__ Cd) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        if (f < 0) continue;
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        const double dg = Cd ? c_m * d.Md[t] - c_c * Cd[t] : c_m * d.Md[t];
        double v = ((fext + 0.0) - fint) + dg * w[t];
        if (blk) v += gather_block<ND>(d, blk, n, c);
        if (d.dp_ptr) v -= c_c * dashpot_sum(d, t, w);
        b[f] = v;
    }
}

// General T (constraints) and support motion: the same terms on every total
// dof, reduced to the free dofs by T^T afterwards (k_nmg_reduce).
// ft = K p = blk + (c_m Md + c_c Cd) p + c_c (dashpots) p
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_total(DevView d, const double* __restrict__ blk, const double* __restrict__ pt,
                                                   double* __restrict__ ft, double c_m, double c_c,
                                                   const double* __restrict__ Cd) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double dg = Cd ? c_m * d.Md[t] + c_c * Cd[t] : c_m * d.Md[t];
        double v = (blk ? gather_block<ND>(d, blk, n, c) : 0.0) + dg * pt[t];
        if (d.dp_ptr) v += c_c * dashpot_sum(d, t, pt);
        ft[t] = v;
    }
}

// ft = Fext - Fint + (M/dt^2 - C/2dt) w on every total dof
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_rtotal(DevView d, const double* __restrict__ blk, const double* __restrict__ w,
                                                    double* __restrict__ ft, double c_m, double c_c,
                                                    const double* __restrict__ Cd) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    const int k = d.step[0];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double fint = gather_fint<ND>(d, n, c);
        const double fext = fext_at(d, t, k);
        const double dg = Cd ? c_m * d.Md[t] - c_c * Cd[t] : c_m * d.Md[t];
        double v = ((fext + 0.0) - fint) + dg * w[t];
        if (blk) v += gather_block<ND>(d, blk, n, c);
        if (d.dp_ptr) v -= c_c * dashpot_sum(d, t, w);
        ft[t] = v;
    }
}

// support-motion increment of step k (CentralDifference.cpp:195)
__global__ void k_ncd_sm(DevView d, double* __restrict__ sm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.ntotal) return;
    sm[t] = sm_at(d, t, d.step[0]);
}

// dU = T du + SM (CentralDifference.cpp:138), Us = U + T du (the strain
// displacement of the next step's element update), then the update of
// CentralDifference.cpp:141-148
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_gupdate(DevView d, const double* __restrict__ dUt, const double* __restrict__ sm,
                                                     double c_m, double c_c, int* flag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const double dut = dUt[t], dU = sm ? dut + sm[t] : dut;
        const double u = d.U[t], up = d.Up[t];
        d.Us[t] = u + dut;
        d.V[t] = c_c * (u + dU - up);
        d.A[t] = c_m * (dU - u + up);
        d.Up[t] = u;
        const double un = u + dU;
        d.U[t] = un;
        bad |= !isfinite(un);
    }
    if (bad) atomicOr(flag, 1);
}

// V = (U + dU - Up)/2dt, A = (dU - U + Up)/dt^2, Up = U, U += dU
// (CentralDifference.cpp:138-148)
template <int ND>
__global__ void __launch_bounds__(256) k_ncd_update(DevView d, const double* __restrict__ du, double c_m, double c_c,
                                                    int* flag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        const double dU = f >= 0 ? du[f] : 0.0;
        const double u = d.U[t], up = d.Up[t];
        d.V[t] = c_c * (u + dU - up);
        d.A[t] = c_m * (dU - u + up);
        d.Up[t] = u;
        const double un = u + dU;
        d.U[t] = un;
        d.Us[t] = un;
        bad |= !isfinite(un);
    }
    if (bad) atomicOr(flag, 1);
}

// state update after the solve (NewmarkBeta.cpp:130-139), identity T, no support motion
template <int ND>
__global__ void __launch_bounds__(256) k_nm_update(DevView d, const double* __restrict__ du, double c_a, double c_av,
                                                   double c_vv, int* flag) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= d.nnode) return;
    bool bad = false;
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        const int t = d.ntdof[n * ND + c];
        const int f = d.tfree[t];
        const double dU = f >= 0 ? du[f] : 0.0;
        const double u = d.U[t] + dU;
        d.U[t] = u;
        d.Us[t] = u;
        d.A[t] = c_a * dU - c_av * d.V[t] - d.A[t];
        d.V[t] = c_vv * dU - d.V[t];
        bad |= !isfinite(u);
    }
    if (bad) atomicOr(flag, 1);
}

__global__ void k_step_inc(int* step) { step[0] += 1; }

// two dot products in one pass: partial[0..B) = a1.b1, partial[B..2B) = a2.b2
__global__ void __launch_bounds__(kDotThreads) k_dot2_partial(const double* __restrict__ a1, const double* __restrict__ b1,
                                                              const double* __restrict__ a2, const double* __restrict__ b2,
                                                              int n, double* __restrict__ partial) {
    __shared__ double sh[2][kDotThreads / 32];
    double s1 = 0.0, s2 = 0.0;
    for (int i = blockIdx.x * kDotThreads + threadIdx.x; i < n; i += kDotBlocks * kDotThreads) {
        s1 += a1[i] * b1[i];
        s2 += a2[i] * b2[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = s1; sh[1][threadIdx.x >> 5] = s2; }
    __syncthreads();
    if (threadIdx.x < 32) {
        double t1 = threadIdx.x < kDotThreads / 32 ? sh[0][threadIdx.x] : 0.0;
        double t2 = threadIdx.x < kDotThreads / 32 ? sh[1][threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            t1 += __shfl_xor_sync(0xffffffffu, t1, o);
            t2 += __shfl_xor_sync(0xffffffffu, t2, o);
        }
        if (threadIdx.x == 0) { partial[blockIdx.x] = t1; partial[kDotBlocks + blockIdx.x] = t2; }
    }
}

// flexible CG scalars (slots of the same array as the PCG ones)
enum { S_RP = 5, S_ZQ = 6 };

// x += alpha p; r -= alpha q   (alpha = r.p / p.q)
__global__ void k_fcg_xr(const double* __restrict__ sc, const double* __restrict__ p, const double* __restrict__ q,
                         double* x, double* r, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double alpha = sc[S_RP] / sc[S_PQ];
    x[i] += alpha * p[i];
    r[i] -= alpha * q[i];
}

// p = z - (z.q / p.q) p   (A-orthogonal to the previous direction)
__global__ void k_fcg_p(const double* __restrict__ sc, const double* __restrict__ z, double* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double beta = -sc[S_ZQ] / sc[S_PQ];
    p[i] = z[i] + beta * p[i];
}

__global__ void k_vmul(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] * b[i];
}

// e -= w * sdinv .* q   (one Richardson sweep with the scaled operator)
__global__ void k_smooth(double* e, const double* __restrict__ q, const double* __restrict__ sdinv, double w, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) e[i] -= w * sdinv[i] * q[i];
}

// e_hat = D^1/2 (x* - x_k)
__global__ void k_ehat(const double* __restrict__ xs, const double* __restrict__ xk, const double* __restrict__ sdinv,
                       double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (xs[i] - xk[i]) / sdinv[i];
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// standard normal samples (counter-based hash + Box-Muller)
__global__ void k_randn(double* e, int n, uint64_t seed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t h1 = mix64(seed + 2ull * (uint64_t)i + 0x9E3779B97F4A7C15ull);
    const uint64_t h2 = mix64(h1 ^ 0xD6E8FEB86659FD93ull);
    const double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
    e[i] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

}  // namespace

constexpr int kRecMax = 12;        // recorded CG iterates per solve

struct svl_nm {
    svl_cd* cd = nullptr;          // model tables, state vectors, stream (shared layout)
    svl_nm_opts opts{};
    int nf = 0;
    double *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *pt = nullptr;
    double *dinv = nullptr, *partial = nullptr, *sc = nullptr;
    int64_t iters_total = 0, iters_last = 0;
    double res_last = 0.0;
    // node-lattice models: learned preconditioner
    bool lattice = false;
    int lnx = 0, lny = 0, lnz = 0;
    std::vector<int32_t> gmap;
    std::vector<double> sdinv_h, rho_h;
    double* sdinv = nullptr;
    double *e1 = nullptr, *e2 = nullptr;
    svl::NnPrecond* nn = nullptr;
    int precond = SVL_PRECOND_JACOBI;
    int64_t jac_ref = 0, fallbacks = 0, learned_solves = 0;
    int64_t train_trial_iters = 0;          // trial-solve iterations of the kept weights
    // Newton: operator scratch block, accumulated increment, iteration counts
    double* fe_op = nullptr;                // [nc][E] element vectors of the operator action
    bool general = false;                   // constraints (T not identity), support motion or damping
    bool damped = false;                    // Rayleigh damping present
    double *ft = nullptr, *dUt = nullptr, *smv = nullptr, *lg = nullptr, *pt2 = nullptr;   // total-dof scratch
    double* dUf = nullptr;                  // [nfree] displacement increment of the step
    bool newton = false, tangent = false;   // tangent: J2 elements present (stored tangents)
    int64_t newton_iters_total = 0, newton_iters_last = 0;
    double newton_res_last = 0.0;
    // consistent mass: the mass term of the effective force through element actions
    bool consistent = false;
    double* wvec = nullptr;                 // [ntotal] 4/dt V + A - 4/dt^2 dU
    // single-precision operator of the inner iterations (eligible models only)
    bool fast_op = false;
    float *geo_f = nullptr, *coef_f = nullptr, *pt_f = nullptr, *fe_f = nullptr;
    // central difference with a non-diagonal K = M/dt^2 + C/2dt (integrator
    // SVL_NM_CENTRAL_DIFFERENCE): element block of (M/dt^2 - C/2dt)(U - Up)
    // and the per-element mass-proportional Rayleigh factors (consistent mass)
    bool cdmode = false, cd_general = false; // cd_general: constraints (T not identity) or support motion
    double* blk_cd = nullptr;               // [nc][E], or null (lumped mass, ak = 0 everywhere)
    double* eam = nullptr;                  // [E] am_e, or null
    // CG iterates recorded for training pairs
    int rec_every = 0, rec_n = 0;
    std::vector<double*> rec_x, rec_r;
    ~svl_nm() {
        if (nn) svl::nn_destroy(nn);
        delete cd;
    }
};

static int nm_dot(svl_nm* nm, const double* a, const double* b, int slot) {
    k_dot_partial<<<kDotBlocks, kDotThreads, 0, nm->cd->stream>>>(a, b, nm->nf, nm->partial);
    k_dot_final<<<1, kDotThreads, 0, nm->cd->stream>>>(nm->partial, nm->sc, slot);
    nm->cd->launches += 2;
    return SVL_OK;
}

static int nm_dot2(svl_nm* nm, const double* a1, const double* b1, int slot1, const double* a2, const double* b2, int slot2) {
    k_dot2_partial<<<kDotBlocks, kDotThreads, 0, nm->cd->stream>>>(a1, b1, a2, b2, nm->nf, nm->partial);
    k_dot_final<<<1, kDotThreads, 0, nm->cd->stream>>>(nm->partial, nm->sc, slot1);
    k_dot_final<<<1, kDotThreads, 0, nm->cd->stream>>>(nm->partial + kDotBlocks, nm->sc, slot2);
    nm->cd->launches += 3;
    return SVL_OK;
}

static int nm_scalars(svl_nm* nm, double* hs) {
    CUDA_TRY(cudaMemcpyAsync(hs, nm->sc, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, nm->cd->stream));
    CUDA_TRY(cudaStreamSynchronize(nm->cd->stream));
    return SVL_OK;
}

// out = (K + 4/dt^2 M) pt on total dofs (K: element stiffness or tangent action)
static int nm_op_total(svl_nm* nm, const double* pt, double* out) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    DevView d = cd->d;
    d.ftol = -1.0;
    d.fe = nm->fe_op;
    const int tb = 256, eg = (m.nelem + 127) / 128, ng = (m.nnode + tb - 1) / tb;
    const double c_c = 2.0 / nm->opts.dt;     // K + 4/dt^2 M + 2/dt C (NewmarkBeta.cpp:231)
    if (nm->tangent || d.dk0) {
        if (m.ndim == 2) k_element_tan<2, 4><<<eg, 128, 0, cd->stream>>>(d, pt, m.ngp, 1, c_c);
        else k_element_tan<3, 8><<<eg, 128, 0, cd->stream>>>(d, pt, m.ngp, 1, c_c);
    } else {
        if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(d, pt, m.ngp, 0);
        else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(d, pt, m.ngp, 0);
    }
    const double c_m = 4.0 / nm->opts.dt / nm->opts.dt;
    if (nm->consistent) {
        // + sum_e (4/dt^2 + 2/dt am_e) M_e p_e; the diagonal keeps the nodal
        // masses only and no lumped mass-proportional part
        if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, pt, nm->fe_op, c_m, 1, nm->eam, c_c);
        else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, pt, nm->fe_op, c_m, 1, nm->eam, c_c);
        d.Cd = nullptr;
        cd->launches += 1;
    }
    if (m.ndim == 2) k_nmg_total<2><<<ng, tb, 0, cd->stream>>>(d, pt, out, c_m, c_c);
    else k_nmg_total<3><<<ng, tb, 0, cd->stream>>>(d, pt, out, c_m, c_c);
    cd->launches += 2;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

// Element parts of (c_m M + c_cs C) x, C's element part being sum_e (am_e M_e
// with a consistent mass) + ak_e K0_e, into blkbuf; returns blkbuf, or null
// when the model has no element part (lumped mass and ak = 0: diagonal only).
static const double* ncd_elem(svl_nm* nm, const double* x, double* blkbuf, double c_m, double c_cs) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    DevView d = cd->d;
    d.ftol = -1.0;
    d.fe = blkbuf;
    const int eg = (m.nelem + 127) / 128;
    const double* blk = nullptr;
    if (d.dk0) {                            // sum_e c_cs ak_e K0_e x_e
        if (m.ndim == 2) k_element_tan<2, 4><<<eg, 128, 0, cd->stream>>>(d, x, m.ngp, 0, c_cs);
        else k_element_tan<3, 8><<<eg, 128, 0, cd->stream>>>(d, x, m.ngp, 0, c_cs);
        blk = blkbuf;
        cd->launches += 1;
    }
    if (nm->consistent) {                   // + sum_e (c_m + c_cs am_e) M_e x_e
        if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, x, blkbuf, c_m, blk ? 1 : 0, nm->eam, c_cs);
        else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, x, blkbuf, c_m, blk ? 1 : 0, nm->eam, c_cs);
        blk = blkbuf;
        cd->launches += 1;
    }
    return blk;
}

// q = Keff v (free dofs); inner: an inner solve iteration, which takes the
// single-precision operator when the handle has one
static int nm_apply(svl_nm* nm, const double* v, double* q, bool inner = false) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const int tb = 256;
    if (nm->cdmode) {                       // q = (M/dt^2 + C/2dt) v (CentralDifference.cpp:70)
        const DevView& d = cd->d;
        const double c_m = 1.0 / nm->opts.dt / nm->opts.dt, c_c = 1.0 / 2.0 / nm->opts.dt;
        if (nm->cd_general) k_nmg_expand<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, v, nm->pt);
        else k_nm_expand<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, v, nm->pt);
        const double* blk = ncd_elem(nm, nm->pt, nm->fe_op, c_m, c_c);
        const double* Cd = nm->consistent ? nullptr : d.Cd;
        if (nm->cd_general) {               // q = T^T K T v
            if (m.ndim == 2) k_ncd_total<2><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, blk, nm->pt, nm->ft, c_m, c_c, Cd);
            else k_ncd_total<3><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, blk, nm->pt, nm->ft, c_m, c_c, Cd);
            k_nmg_reduce<<<(nm->nf + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, nm->ft, nullptr, q);
            cd->launches += 3;
            CUDA_TRY(cudaGetLastError());
            return SVL_OK;
        }
        if (m.ndim == 2) k_ncd_apply<2><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, blk, nm->pt, q, c_m, c_c, Cd);
        else k_ncd_apply<3><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, blk, nm->pt, q, c_m, c_c, Cd);
        cd->launches += 2;
        CUDA_TRY(cudaGetLastError());
        return SVL_OK;
    }
    if (inner && nm->fast_op) {
        DevView d = cd->d;
        k_nm_expand_f<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, v, nm->pt, nm->pt_f);
        const int gg = (int)(((int64_t)m.nelem * m.nen + 127) / 128);
        if (m.ndim == 2) k_nm_op_f<2, 4><<<gg, 128, 0, cd->stream>>>(d, nm->geo_f, nm->coef_f, nm->pt_f, nm->fe_f);
        else k_nm_op_f<3, 8><<<gg, 128, 0, cd->stream>>>(d, nm->geo_f, nm->coef_f, nm->pt_f, nm->fe_f);
        const double c_m = 4.0 / nm->opts.dt / nm->opts.dt;
        if (m.ndim == 2) k_nm_apply_f<2><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->fe_f, nm->pt, q, c_m);
        else k_nm_apply_f<3><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->fe_f, nm->pt, q, c_m);
        cd->launches += 3;
        CUDA_TRY(cudaGetLastError());
        return SVL_OK;
    }
    if (nm->general) {                      // q = T^T (K + c_m M) T v
        k_nmg_expand<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, v, nm->pt);
        TRY(nm_op_total(nm, nm->pt, nm->ft));
        k_nmg_reduce<<<(nm->nf + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, nm->ft, nullptr, q);
        cd->launches += 2;
        CUDA_TRY(cudaGetLastError());
        return SVL_OK;
    }
    DevView d = cd->d;
    d.ftol = -1.0;                  // the operator action is not filtered
    d.fe = nm->fe_op;               // and keeps the state's element forces intact
    k_nm_expand<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, v, nm->pt);
    const int eg = (m.nelem + 127) / 128;
    if (nm->tangent) {
        if (m.ndim == 2) k_element_tan<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->pt, m.ngp, 1, 0.0);
        else k_element_tan<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->pt, m.ngp, 1, 0.0);
    } else {
        if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->pt, m.ngp, 0);
        else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->pt, m.ngp, 0);
    }
    const double c_m = 4.0 / nm->opts.dt / nm->opts.dt;
    if (nm->consistent) {                   // + 4/dt^2 M_e p_e in the same element vectors
        if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->pt, d.fe, c_m, 1);
        else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->pt, d.fe, c_m, 1);
        cd->launches += 1;
    }
    if (m.ndim == 2) k_nm_apply<2><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->pt, q, c_m);
    else k_nm_apply<3><<<(m.nnode + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->pt, q, c_m);
    cd->launches += 3;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

static int nm_record(svl_nm* nm, int it) {
    if (nm->rec_every <= 0 || it % nm->rec_every != 0 || nm->rec_n >= (int)nm->rec_x.size()) return SVL_OK;
    const size_t bytes = sizeof(double) * nm->nf;
    CUDA_TRY(cudaMemcpyAsync(nm->rec_x[nm->rec_n], nm->x, bytes, cudaMemcpyDeviceToDevice, nm->cd->stream));
    CUDA_TRY(cudaMemcpyAsync(nm->rec_r[nm->rec_n], nm->r, bytes, cudaMemcpyDeviceToDevice, nm->cd->stream));
    nm->rec_n++;
    return SVL_OK;
}

// Jacobi-PCG from x = 0 (warm = false) or from the current x.
static int nm_solve_jacobi(svl_nm* nm, bool warm, int64_t maxit) {
    svl_cd* cd = nm->cd;
    const int n = nm->nf, tb = 256, g = (n + tb - 1) / tb;
    double hs[S_NSCAL];
    if (warm) {
        TRY(nm_apply(nm, nm->x, nm->q));
    } else {
        CUDA_TRY(cudaMemsetAsync(nm->x, 0, sizeof(double) * n, cd->stream));
        CUDA_TRY(cudaMemsetAsync(nm->q, 0, sizeof(double) * n, cd->stream));
    }
    nm_dot(nm, nm->b, nm->b, S_BB);
    k_pcg_reset<<<g, tb, 0, cd->stream>>>(nm->b, nm->q, nm->dinv, nm->r, nm->z, nm->p, n);
    nm_dot(nm, nm->r, nm->z, S_RZ);
    nm_dot(nm, nm->r, nm->r, S_RR);
    TRY(nm_scalars(nm, hs));
    const double bb = hs[S_BB];
    if (bb == 0.0) { nm->res_last = 0.0; return SVL_OK; }
    const double tol2 = nm->opts.pcg_tol * nm->opts.pcg_tol * bb;
    if (warm && hs[S_RR] <= tol2) { nm->res_last = std::sqrt(hs[S_RR] / bb); return SVL_OK; }
    const int check = 4;
    for (int64_t it = 1; it <= maxit; ++it) {
        TRY(nm_apply(nm, nm->p, nm->q, true));
        nm_dot(nm, nm->p, nm->q, S_PQ);
        k_pcg_xr<<<g, tb, 0, cd->stream>>>(nm->sc, nm->p, nm->q, nm->dinv, nm->x, nm->r, nm->z, n);
        nm_dot2(nm, nm->r, nm->z, S_RZN, nm->r, nm->r, S_RR);
        k_pcg_p<<<g, tb, 0, cd->stream>>>(nm->sc, nm->z, nm->p, n);
        k_pcg_roll<<<1, 1, 0, cd->stream>>>(nm->sc);
        cd->launches += 3;
        nm->iters_last++;
        nm->iters_total++;
        TRY(nm_record(nm, (int)it));
        if (it % check == 0 || it == maxit) {
            TRY(nm_scalars(nm, hs));
            if (!(hs[S_PQ] > 0.0)) { set_error("PCG breakdown: p.Kp = %g at iteration %lld", hs[S_PQ], (long long)it); return SVL_ERR_BREAKDOWN; }
            if (!std::isfinite(hs[S_RR])) { set_error("PCG residual is not finite"); return SVL_ERR_NONFINITE; }
            if (hs[S_RR] <= tol2) {
                // confirm with the true residual; restart from it if the recursive one drifted
                TRY(nm_apply(nm, nm->x, nm->q));
                k_pcg_reset<<<g, tb, 0, cd->stream>>>(nm->b, nm->q, nm->dinv, nm->r, nm->z, nm->p, n);
                nm_dot2(nm, nm->r, nm->r, S_RR, nm->r, nm->z, S_RZ);
                cd->launches += 1;
                TRY(nm_scalars(nm, hs));
                nm->res_last = std::sqrt(hs[S_RR] / bb);
                if (hs[S_RR] <= tol2) {
                    if (!warm) nm->jac_ref = it;
                    return SVL_OK;
                }
            }
        }
    }
    TRY(nm_scalars(nm, hs));
    nm->res_last = std::sqrt(hs[S_RR] / bb);
    set_error("PCG did not reach %g in %lld iterations (relative residual %g)", nm->opts.pcg_tol, (long long)maxit, nm->res_last);
    return SVL_ERR_MAXITER;
}

// Flexible CG with the learned preconditioner; falls back to Jacobi-PCG
// (continuing from the current iterate) once it has used as many iterations
// as the last plain Jacobi solve needed.
static int nm_solve_learned(svl_nm* nm, bool allow_fallback = true) {
    svl_cd* cd = nm->cd;
    const int n = nm->nf, tb = 256, g = (n + tb - 1) / tb;
    double hs[S_NSCAL];
    const size_t bytes = sizeof(double) * n;
    CUDA_TRY(cudaMemsetAsync(nm->x, 0, bytes, cd->stream));
    CUDA_TRY(cudaMemcpyAsync(nm->r, nm->b, bytes, cudaMemcpyDeviceToDevice, cd->stream));
    nm_dot(nm, nm->b, nm->b, S_BB);
    TRY(svl::nn_apply(nm->nn, nm->r, nm->z));
    CUDA_TRY(cudaMemcpyAsync(nm->p, nm->z, bytes, cudaMemcpyDeviceToDevice, cd->stream));
    cd->launches += 7;
    TRY(nm_scalars(nm, hs));
    const double bb = hs[S_BB];
    nm->learned_solves++;
    if (bb == 0.0) { nm->res_last = 0.0; return SVL_OK; }
    const double tol2 = nm->opts.pcg_tol * nm->opts.pcg_tol * bb;
    const int64_t budget = std::min<int64_t>(nm->opts.pcg_maxit, nm->jac_ref > 0 ? nm->jac_ref : nm->opts.pcg_maxit);
    const int check = 4;
    bool cold = false;
    for (int64_t it = 1; it <= budget; ++it) {
        TRY(nm_apply(nm, nm->p, nm->q, true));
        nm_dot2(nm, nm->p, nm->q, S_PQ, nm->r, nm->p, S_RP);
        k_fcg_xr<<<g, tb, 0, cd->stream>>>(nm->sc, nm->p, nm->q, nm->x, nm->r, n);
        TRY(svl::nn_apply(nm->nn, nm->r, nm->z));
        nm_dot2(nm, nm->z, nm->q, S_ZQ, nm->r, nm->r, S_RR);
        k_fcg_p<<<g, tb, 0, cd->stream>>>(nm->sc, nm->z, nm->p, n);
        cd->launches += 2 + 7;
        nm->iters_last++;
        nm->iters_total++;
        if (it % check == 0 || it == budget) {
            TRY(nm_scalars(nm, hs));
            if (!(hs[S_PQ] > 0.0) || !std::isfinite(hs[S_RR]) || !std::isfinite(hs[S_PQ])) {
                cold = !std::isfinite(hs[S_RR]) || !std::isfinite(hs[S_PQ]);    // the iterate may be spoiled
                break;
            }
            if (hs[S_RR] <= tol2) {
                TRY(nm_apply(nm, nm->x, nm->q));
                k_pcg_reset<<<g, tb, 0, cd->stream>>>(nm->b, nm->q, nm->dinv, nm->r, nm->z, nm->p, n);
                nm_dot(nm, nm->r, nm->r, S_RR);
                cd->launches += 1;
                TRY(nm_scalars(nm, hs));
                nm->res_last = std::sqrt(hs[S_RR] / bb);
                if (hs[S_RR] <= tol2) return svl::nn_status(nm->nn);
                // drifted: restart the flexible iteration from the true residual
                TRY(svl::nn_apply(nm->nn, nm->r, nm->z));
                CUDA_TRY(cudaMemcpyAsync(nm->p, nm->z, bytes, cudaMemcpyDeviceToDevice, cd->stream));
            }
        }
    }
    if (!allow_fallback) { set_error("learned preconditioner did not converge within the Jacobi budget"); return SVL_ERR_MAXITER; }
    nm->fallbacks++;
    return nm_solve_jacobi(nm, !cold, std::max<int64_t>(1, nm->opts.pcg_maxit - nm->iters_last));
}

static int nm_solve(svl_nm* nm) {
    nm->iters_last = 0;
    nm->res_last = 0.0;
    if (nm->precond == SVL_PRECOND_LEARNED && nm->nn && nm->rec_every == 0) return nm_solve_learned(nm);
    return nm_solve_jacobi(nm, false, nm->opts.pcg_maxit);
}

// training pairs from the CG iterates recorded during the last solve: e_hat =
// D^1/2 (x* - x_k), r_hat = D^-1/2 r_k, normalised by |e_hat|
static int nm_pairs_from_iterates(svl_nm* nm) {
    svl_cd* cd = nm->cd;
    const int n = nm->nf, tb = 256, g = (n + tb - 1) / tb;
    double hs[S_NSCAL];
    for (int j = 0; j < nm->rec_n; ++j) {
        k_ehat<<<g, tb, 0, cd->stream>>>(nm->x, nm->rec_x[j], nm->sdinv, nm->e1, n);
        k_vmul<<<g, tb, 0, cd->stream>>>(nm->rec_r[j], nm->sdinv, nm->e2, n);
        nm_dot(nm, nm->e1, nm->e1, S_RP);
        TRY(nm_scalars(nm, hs));
        if (hs[S_RP] > 0.0 && std::isfinite(hs[S_RP])) TRY(svl::nn_record_pair(nm->nn, nm->e2, nm->e1, 1.0 / std::sqrt(hs[S_RP])));
    }
    nm->rec_n = 0;
    return SVL_OK;
}

// Node lattice of a 3D hexahedral model: distinct x, y, z coordinate values
// whose product is the node count, each node on its own lattice point.
static bool detect_lattice(const HostModel& m, int dims[3], std::vector<int32_t>& cell) {
    if (m.ndim != 3 || m.nen != 8 || m.nnode == 0) return false;
    int nd[3];
    std::vector<std::vector<double>> vals(3);
    for (int a = 0; a < 3; ++a) {
        std::vector<double> v(m.nnode);
        double lo = 1e300, hi = -1e300;
        for (int n = 0; n < m.nnode; ++n) { v[n] = m.X[(size_t)n * 3 + a]; lo = std::min(lo, v[n]); hi = std::max(hi, v[n]); }
        std::sort(v.begin(), v.end());
        const double tol = 1e-9 * std::max(1.0, hi - lo);
        std::vector<double> u;
        for (double x : v) if (u.empty() || x - u.back() > tol) u.push_back(x);
        vals[a] = u;
        nd[a] = (int)u.size();
    }
    if ((int64_t)nd[0] * nd[1] * nd[2] != m.nnode) return false;
    cell.assign(m.nnode, -1);
    std::vector<char> used((size_t)m.nnode, 0);
    for (int n = 0; n < m.nnode; ++n) {
        int ijk[3];
        for (int a = 0; a < 3; ++a) {
            const auto& u = vals[a];
            const double x = m.X[(size_t)n * 3 + a];
            size_t k = std::lower_bound(u.begin(), u.end(), x) - u.begin();
            if (k == u.size() || (k > 0 && std::fabs(u[k - 1] - x) < std::fabs(u[k] - x))) k = k == 0 ? 0 : k - 1;
            ijk[a] = (int)k;
        }
        const int c = ijk[0] + nd[0] * (ijk[1] + nd[1] * ijk[2]);
        if (used[c]) return false;
        used[c] = 1;
        cell[n] = c;
    }
    dims[0] = nd[0]; dims[1] = nd[1]; dims[2] = nd[2];
    return true;
}

// Diagonal of the initial elastic element stiffness K0_e (per element dof,
// node-major): sum_q w B_a^T D B_a with the elastic moduli (J2: K, G).
static void elem_k0_diag(const HostModel& m, int e, double* kd) {
    const double* pr = m.param(e);
    const int mt = m.mat_type(e);
    double c1, c3;
    if (mt == SVL_MAT_ELASTIC2DPLANESTRAIN || mt == SVL_MAT_ELASTIC3DLINEAR) {
        const double E = pr[0], nu = pr[1];
        c1 = E * (1.0 - nu) / (1.0 - 2.0 * nu) / (1.0 + nu);
        c3 = E / (2.0 * (1.0 + nu));
    } else {                    // J2: the elastic moduli K, G
        c1 = pr[0] + 4.0 / 3.0 * pr[1];
        c3 = pr[1];
    }
    for (int j = 0; j < m.nen * m.ndof; ++j) kd[j] = 0.0;
    for (int q = 0; q < m.ngp; ++q) {
        double dNx[8][3], N[8];
        const double w = gp_factor(m, e, gp_geometry(m, e, q, dNx, N));
        for (int a = 0; a < m.nen; ++a) {
            const double bx = dNx[a][0], by = dNx[a][1], bz = dNx[a][2];
            if (m.ndim == 2) {
                kd[2 * a] += w * (c1 * bx * bx + c3 * by * by);
                kd[2 * a + 1] += w * (c1 * by * by + c3 * bx * bx);
            } else {
                kd[3 * a] += w * (c1 * bx * bx + c3 * (by * by + bz * bz));
                kd[3 * a + 1] += w * (c1 * by * by + c3 * (bx * bx + bz * bz));
                kd[3 * a + 2] += w * (c1 * bz * bz + c3 * (bx * bx + by * by));
            }
        }
    }
}

// Diagonal of the consistent element mass per node: rho sum_q w t |J| N_a^2.
static void elem_cmass_diag(const HostModel& m, int e, double* md) {
    const double rho = m.param(e)[2];
    for (int a = 0; a < m.nen; ++a) md[a] = 0.0;
    for (int q = 0; q < m.ngp; ++q) {
        double dNx[8][3], N[8];
        const double w = gp_factor(m, e, gp_geometry(m, e, q, dNx, N));
        for (int a = 0; a < m.nen; ++a) md[a] += rho * w * N[a] * N[a];
    }
}

// Handle set-up of the central-difference mode (SVL_NM_CENTRAL_DIFFERENCE):
// checks, the Jacobi diagonal of K = M/dt^2 + C/2dt, work vectors.
static int ncd_setup(svl_nm* nm) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const svl_nm_opts& o = nm->opts;
    if (o.algorithm != SVL_ALGO_LINEAR || o.precond != SVL_PRECOND_JACOBI) {
        set_error("central difference: the Linear algorithm with the Jacobi preconditioner");
        return SVL_ERR_UNSUPPORTED;
    }
    if (cd->d.ndrm > 0) {
        set_error("central difference with a non-diagonal effective stiffness is covered without domain-reduction loads");
        return SVL_ERR_UNSUPPORTED;
    }
    nm->cdmode = true;
    nm->cd_general = !cd->identity_T || cd->has_sm;
    nm->consistent = !m.lumped;
    nm->general = nm->damped = nm->newton = nm->tangent = false;
    nm->nf = m.nfree;
    const double c_m = 1.0 / o.dt / o.dt, c_c = 1.0 / 2.0 / o.dt;
    const int nc = m.nen * m.ndof;
    // diagonal of K: element parts, then the nodal / lumped diagonal
    std::vector<double> Kd(m.ntotal, 0.0), eam;
    bool any_am = false;
    for (int e = 0; e < m.nelem; ++e) {
        const double am = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e], ak = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1];
        any_am = any_am || am != 0.0;
        double kd[24], md[8];
        if (ak != 0.0) elem_k0_diag(m, e, kd);
        if (nm->consistent) elem_cmass_diag(m, e, md);
        for (int a = 0; a < m.nen; ++a)
            for (int c = 0; c < m.ndof; ++c) {
                double v = 0.0;
                if (ak != 0.0) v += c_c * ak * kd[a * m.ndof + c];
                if (nm->consistent) v += (c_m + c_c * am) * md[a];
                Kd[m.tdof[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndof + c]] += v;
            }
    }
    std::vector<double> Md;
    if (nm->consistent) {
        Md.assign(m.ntotal, 0.0);
        if (!m.nodemass.empty())
            for (int t = 0; t < m.ntotal; ++t) if (std::fabs(m.nodemass[t]) > o.mtol) Md[t] = m.nodemass[t];
    } else {
        lumped_mass_diag(m, o.mtol, Md);
        std::vector<double> Cm;
        rayleigh_mass_diag(m, Cm);
        for (int t = 0; t < m.ntotal; ++t) Kd[t] += c_c * Cm[t];
    }
    for (int t = 0; t < m.ntotal; ++t) Kd[t] += c_m * Md[t];
    for (size_t i = 0; i < m.dp_eta.size(); ++i) {   // ZeroLength1D dashpots: eta on both dofs
        Kd[m.dp_dof[2 * i]] += c_c * m.dp_eta[i];
        Kd[m.dp_dof[2 * i + 1]] += c_c * m.dp_eta[i];
    }
    // Jacobi scale: the diagonal of T^T diag(K) T
    std::vector<int32_t> Tp, Tc;
    std::vector<double> Tv, dg(std::max(m.nfree, 1), 0.0);
    build_total_to_free(m, Tp, Tc, Tv);
    for (int t = 0; t < m.ntotal; ++t)
        for (int i = Tp[t]; i < Tp[t + 1]; ++i) dg[Tc[i]] += Tv[i] * Tv[i] * Kd[t];
    std::vector<double> dinv(std::max(m.nfree, 1), 1.0);
    for (int f = 0; f < m.nfree; ++f) {
        if (!(dg[f] > 0.0)) { set_error("free dof %d has no mass", f); return SVL_ERR_INVALID; }
        dinv[f] = 1.0 / dg[f];
    }
    int st;
    double** vecs[] = {&nm->b, &nm->x, &nm->r, &nm->z, &nm->p, &nm->q};
    for (double** pv : vecs) if ((st = cd->zeros((size_t)std::max(m.nfree, 1), pv))) return st;
    if ((st = cd->zeros((size_t)m.ntotal, &nm->pt)) || (st = cd->zeros(2 * kDotBlocks, &nm->partial)) ||
        (st = cd->zeros(S_NSCAL, &nm->sc)) || (st = cd->zeros((size_t)m.ntotal, &nm->wvec)))
        return st;
    const double* dd = nullptr;
    if ((st = cd->upload(dinv, &dd))) return st;
    nm->dinv = const_cast<double*>(dd);
    if (nm->consistent || cd->d.dk0) {
        if ((st = cd->zeros((size_t)nc * m.nelem, &nm->fe_op)) || (st = cd->zeros((size_t)nc * m.nelem, &nm->blk_cd))) return st;
    }
    if (nm->cd_general) {
        double** tv[] = {&nm->ft, &nm->dUt, &nm->smv, &nm->lg};
        for (double** pv : tv) if ((st = cd->zeros((size_t)m.ntotal, pv))) return st;
    }
    if (nm->consistent && any_am) {
        for (int e = 0; e < m.nelem; ++e) eam.push_back(m.ray[2 * (size_t)e]);
        const double* ea = nullptr;
        if ((st = cd->upload(eam, &ea))) return st;
        nm->eam = const_cast<double*>(ea);
    }
    return SVL_OK;
}

static int nm_step(svl_nm* nm, double* U_hist_row);

extern "C" {

int svl_nm_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_nm_opts* opts, svl_nm** out) {
    if (!out || !opts) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *out = nullptr;
    if (!(opts->dt > 0.0) || !(opts->pcg_tol > 0.0) || opts->pcg_maxit <= 0) { set_error("bad Newmark options"); return SVL_ERR_INVALID; }
    if (opts->precond != SVL_PRECOND_JACOBI && opts->precond != SVL_PRECOND_LEARNED) { set_error("unknown preconditioner %d", opts->precond); return SVL_ERR_INVALID; }
    if (opts->integrator != SVL_NM_NEWMARK && opts->integrator != SVL_NM_CENTRAL_DIFFERENCE) {
        set_error("unknown integrator %d", opts->integrator);
        return SVL_ERR_INVALID;
    }
    svl_cd_opts co{};
    co.dt = opts->dt; co.ftol = opts->ftol; co.mtol = opts->mtol; co.precision = SVL_PREC_FP64; co.check_every = 0;
    svl_cd* cd = nullptr;
    int st = cd_create(model, loads, &co, &cd, true);
    if (st) return st;
    svl_nm* nm = new svl_nm();
    nm->cd = cd;
    nm->opts = *opts;
    auto fail = [&](int s2) { delete nm; return s2; };
    const HostModel& m = cd->m;
    if (opts->integrator == SVL_NM_CENTRAL_DIFFERENCE) {
        if ((st = ncd_setup(nm))) return fail(st);
        if (cudaStreamSynchronize(cd->stream) != cudaSuccess) { set_error("upload failed"); return fail(SVL_ERR_CUDA); }
        *out = nm;
        return SVL_OK;
    }
    nm->damped = !m.ray.empty() || !m.dp_eta.empty();
    nm->general = !cd->identity_T || cd->has_sm || nm->damped;
    if (opts->algorithm != SVL_ALGO_LINEAR && opts->algorithm != SVL_ALGO_NEWTON) { set_error("unknown algorithm %d", opts->algorithm); return fail(SVL_ERR_INVALID); }
    nm->newton = opts->algorithm == SVL_ALGO_NEWTON;
    if (nm->newton && (opts->maxit <= 0 || !(opts->cnvgtol >= 0.0) || opts->cnvgtest < 1 || opts->cnvgtest > 8)) {
        set_error("Newton needs maxit > 0, cnvgtol >= 0 (0: always maxit iterations) and cnvgtest 1..8");
        return fail(SVL_ERR_INVALID);
    }
    if (m.has_j2() && !nm->newton) {
        // Linear with a nonlinear material (Linear.cpp:22-56): effective force from
        // the committed states, one solve with the tangent stiffness, one state
        // update from U + dU -- exactly one Newton iteration
        nm->newton = true;
        nm->opts.maxit = 1;
        nm->opts.cnvgtol = 0.0;
        nm->opts.cnvgtest = 4;
    }
    nm->tangent = nm->newton && m.has_j2();
    nm->nf = m.nfree;
    const double c_m = 4.0 / opts->dt / opts->dt, c_c = 2.0 / opts->dt;
    // Jacobi diagonal: diag(K + 2/dt C) + 4/dt^2 M on free dofs (identity T)
    std::vector<double> Kd(m.ntotal, 0.0);
    const int nc = m.nen * m.ndof;
    for (int e = 0; e < m.nelem; ++e) {
        double kd[24];
        elem_k0_diag(m, e, kd);
        const double ak = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1];
        for (int a = 0; a < m.nen; ++a)
            for (int c = 0; c < m.ndof; ++c) Kd[m.tdof[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndof + c]] += (1.0 + c_c * ak) * kd[a * m.ndof + c];
    }
    std::vector<double> M;
    lumped_mass_diag(m, opts->mtol, M);
    nm->consistent = !m.lumped;
    if (nm->consistent) {
        // diagonal of the consistent mass: rho sum_q w t |J| N_a^2, plus the nodal masses
        std::fill(M.begin(), M.end(), 0.0);
        for (int e = 0; e < m.nelem; ++e) {
            double md[8];
            elem_cmass_diag(m, e, md);
            for (int a = 0; a < m.nen; ++a)
                for (int c = 0; c < m.ndof; ++c) M[m.tdof[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndof + c]] += md[a];
        }
        if (!m.nodemass.empty())
            for (int t = 0; t < m.ntotal; ++t) if (std::fabs(m.nodemass[t]) > opts->mtol) M[t] += m.nodemass[t];
    }
    if (nm->damped) {                       // + 2/dt (sum_e am_e M_e + dashpot diagonal)
        std::vector<double> Cm;
        if (nm->consistent) {               // am_e times the consistent element mass's diagonal
            Cm.assign(m.ntotal, 0.0);
            for (int e = 0; e < m.nelem && !m.ray.empty(); ++e) {
                const double am = m.ray[2 * (size_t)e];
                if (am == 0.0) continue;
                double md[8];
                elem_cmass_diag(m, e, md);
                for (int a = 0; a < m.nen; ++a)
                    for (int c = 0; c < m.ndof; ++c) Cm[m.tdof[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndof + c]] += am * md[a];
            }
        } else {
            rayleigh_mass_diag(m, Cm);
        }
        for (int t = 0; t < m.ntotal; ++t) Kd[t] += c_c * Cm[t];
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            Kd[m.dp_dof[2 * i]] += c_c * m.dp_eta[i];
            Kd[m.dp_dof[2 * i + 1]] += c_c * m.dp_eta[i];
        }
    }
    std::vector<double> dinv(std::max(m.nfree, 1), 1.0);
    if (!cd->identity_T) {
        // diagonal of T^T diag(K + c_m M) T (the Jacobi preconditioner only)
        std::vector<int32_t> Tp, Tc;
        std::vector<double> Tv, dg(std::max(m.nfree, 1), 0.0);
        build_total_to_free(m, Tp, Tc, Tv);
        for (int t = 0; t < m.ntotal; ++t)
            for (int i = Tp[t]; i < Tp[t + 1]; ++i) dg[Tc[i]] += Tv[i] * Tv[i] * (Kd[t] + c_m * M[t]);
        for (int f = 0; f < m.nfree; ++f) dinv[f] = dg[f] > 0.0 ? 1.0 / dg[f] : 1.0;
    } else {
        for (int n = 0; n < m.nnode; ++n)
            for (int c = 0; c < m.ndof; ++c) {
                const int t = m.tdof[(size_t)n * m.ndof + c], f = m.fdof[(size_t)n * m.ndof + c];
                if (f >= 0) dinv[f] = 1.0 / (Kd[t] + c_m * M[t]);
            }
    }
    double** vecs[] = {&nm->b, &nm->x, &nm->r, &nm->z, &nm->p, &nm->q};
    for (double** pv : vecs) if ((st = cd->zeros((size_t)std::max(m.nfree, 1), pv))) return fail(st);
    if ((st = cd->zeros((size_t)m.ntotal, &nm->pt)) || (st = cd->zeros(2 * kDotBlocks, &nm->partial)) ||
        (st = cd->zeros(S_NSCAL, &nm->sc)))
        return fail(st);
    const double* dd = nullptr;
    if ((st = cd->upload(dinv, &dd))) return fail(st);
    nm->dinv = const_cast<double*>(dd);
    if ((st = cd->zeros((size_t)nc * m.nelem, &nm->fe_op)) || (st = cd->zeros((size_t)std::max(m.nfree, 1), &nm->dUf)))
        return fail(st);
    if (nm->consistent) {
        double* fm = nullptr;
        if ((st = cd->zeros((size_t)nc * m.nelem, &fm)) || (st = cd->zeros((size_t)m.ntotal, &nm->wvec))) return fail(st);
        cd->d.fem = fm;
        bool any_am = false;
        for (size_t e = 0; e < m.ray.size() / 2; ++e) any_am = any_am || m.ray[2 * e] != 0.0;
        if (any_am) {                       // am_e of the consistent element masses in C
            std::vector<double> eam(m.nelem);
            for (int e = 0; e < m.nelem; ++e) eam[e] = m.ray[2 * (size_t)e];
            const double* ea = nullptr;
            if ((st = cd->upload(eam, &ea))) return fail(st);
            nm->eam = const_cast<double*>(ea);
        }
    }
    if (nm->general) {
        double** tv[] = {&nm->ft, &nm->dUt, &nm->smv, &nm->lg, &nm->pt2};
        for (double** pv : tv) if ((st = cd->zeros((size_t)m.ntotal, pv))) return fail(st);
    }
    if (nm->tangent) {
        double* ct = nullptr;
        if ((st = cd->zeros((size_t)(m.ndim == 2 ? 9 : 36) * m.ngp * m.nelem, &ct))) return fail(st);
        cd->d.ctan = ct;
    }
    // single-precision operator of the inner iterations: elastic models without
    // damping or constraints (the FP64 operator confirms every answer)
    if (opts->single_inner && !nm->general && !nm->tangent && !m.has_j2() && !cd->d.dk0 && !nm->consistent &&
        m.nelem > 0 && m.nfree > 0) {
        const int per = m.nen * m.ndim + 1;
        std::vector<double> gh((size_t)cd->ngeo * m.ngp * per), ch((size_t)3 * m.nelem);
        if (cudaMemcpy(gh.data(), cd->d.geo, gh.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(ch.data(), cd->d.ecoef, ch.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
            set_error("reading the operator tables failed"); return fail(SVL_ERR_CUDA);
        }
        std::vector<float> gf(gh.begin(), gh.end()), cf(ch.begin(), ch.end());
        const float *g2 = nullptr, *c2 = nullptr;
        float *p2 = nullptr, *f2 = nullptr;
        if ((st = cd->upload(gf, &g2)) || (st = cd->upload(cf, &c2)) || (st = cd->zeros((size_t)m.ntotal, &p2)) ||
            (st = cd->zeros((size_t)nc * m.nelem, &f2)))
            return fail(st);
        nm->geo_f = const_cast<float*>(g2); nm->coef_f = const_cast<float*>(c2); nm->pt_f = p2; nm->fe_f = f2;
        nm->fast_op = true;
    }
    // lattice models: the maps and scalings of the learned preconditioner
    int dims[3];
    std::vector<int32_t> cell;
    if (m.nfree > 0 && cd->identity_T && detect_lattice(m, dims, cell)) {
        nm->lattice = true;
        nm->lnx = dims[0]; nm->lny = dims[1]; nm->lnz = dims[2];
        const int64_t V = (int64_t)dims[0] * dims[1] * dims[2];
        nm->gmap.assign(m.nfree, 0);
        nm->sdinv_h.assign(m.nfree, 0.0);
        nm->rho_h.assign(m.nfree, 0.0);
        for (int n = 0; n < m.nnode; ++n)
            for (int c = 0; c < 3; ++c) {
                const int t = m.tdof[(size_t)n * 3 + c], f = m.fdof[(size_t)n * 3 + c];
                if (f < 0) continue;
                nm->gmap[f] = (int32_t)(c * V + cell[n]);
                nm->sdinv_h[f] = std::sqrt(dinv[f]);
                nm->rho_h[f] = c_m * M[t] * dinv[f];
            }
        const double* sd = nullptr;
        if ((st = cd->upload(nm->sdinv_h, &sd)) || (st = cd->zeros((size_t)m.nfree, &nm->e1)) ||
            (st = cd->zeros((size_t)m.nfree, &nm->e2)))
            return fail(st);
        nm->sdinv = const_cast<double*>(sd);
        if (opts->precond == SVL_PRECOND_LEARNED) {
            if ((st = svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, cd->stream, &nm->nn))) return fail(st);
            nm->precond = SVL_PRECOND_LEARNED;
        }
    } else if (opts->precond == SVL_PRECOND_LEARNED) {
        set_error("the learned preconditioner needs a hexahedral model without constraints whose nodes form a lattice");
        return fail(SVL_ERR_UNSUPPORTED);
    }
    if (cudaStreamSynchronize(cd->stream) != cudaSuccess) { set_error("upload failed"); return fail(SVL_ERR_CUDA); }
    *out = nm;
    return SVL_OK;
}

int svl_nm_set_initial(svl_nm* nm, const double* U0, const double* V0, const double* A0) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    TRY(svl_cd_set_initial(nm->cd, U0, V0, A0));
    // strain displacement = U0 for an elastic start from given displacements;
    // the central-difference mode keeps the virgin element state, as
    // CentralDifference::Initialize leaves the elements (first Fint = 0)
    if (U0 && !nm->cdmode) CUDA_TRY(cudaMemcpyAsync(nm->cd->d.Us, nm->cd->d.U, sizeof(double) * nm->cd->m.ntotal, cudaMemcpyDeviceToDevice, nm->cd->stream));
    if (nm->newton) {
        // element states, forces and tangents of the initial displacement
        svl_cd* cd = nm->cd;
        const HostModel& m = cd->m;
        const int eg = (m.nelem + 127) / 128;
        if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
        else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
        CUDA_TRY(cudaGetLastError());
    }
    CUDA_TRY(cudaStreamSynchronize(nm->cd->stream));
    return SVL_OK;
}

}  // extern "C"

// domain-reduction forces of the step just begun (d.step already advanced)
static int nm_drm(svl_nm* nm) {
    svl_cd* cd = nm->cd;
    if (cd->d.ndrm <= 0) return SVL_OK;
    const int gd = (cd->d.ndrm + 127) / 128;
    if (cd->m.ndim == 2) k_drm<2, 4><<<gd, 128, 0, cd->stream>>>(cd->d, cd->m.ngp);
    else k_drm<3, 8><<<gd, 128, 0, cd->stream>>>(cd->d, cd->m.ngp);
    cd->launches += 1;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

static int nmg_rhs(svl_nm* nm);

// Effective force of step k into nm->b (state untouched).
// Consistent mass: the element actions M_e w_e of the effective force's mass
// term into d.fem (k_nm_rhs gathers them); nothing with a lumped mass.
static int nm_mass_rhs(svl_nm* nm, const double* dUf, double c_m) {
    if (!nm->consistent) return SVL_OK;
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const int tb = 256, eg = (m.nelem + 127) / 128;
    k_nm_wvec<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, dUf, 4.0 / nm->opts.dt, c_m, nm->wvec);
    DevView d = cd->d;
    if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->wvec, const_cast<double*>(d.fem), 1.0, 0);
    else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->wvec, const_cast<double*>(d.fem), 1.0, 0);
    cd->launches += 2;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

static int nm_rhs(svl_nm* nm, int k) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double dt = nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb, eg = (m.nelem + 127) / 128;
    const int km1 = k - 1;
    CUDA_TRY(cudaMemcpyAsync(cd->d.step, &km1, sizeof(int), cudaMemcpyHostToDevice, cd->stream));
    k_step_inc<<<1, 1, 0, cd->stream>>>(cd->d.step);
    TRY(nm_drm(nm));
    if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    if (nm->general) {
        k_nmg_sm<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, nm->smv);
        CUDA_TRY(cudaMemsetAsync(nm->dUt, 0, sizeof(double) * m.ntotal, cd->stream));
        return nmg_rhs(nm);
    }
    TRY(nm_mass_rhs(nm, nullptr, 0.0));
    if (m.ndim == 2) k_nm_rhs<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nullptr, 0.0);
    else k_nm_rhs<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nullptr, 0.0);
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

// Right-hand side for scoring the network: the effective force of step k, or
// K_eff applied to a smooth random field when that force is zero.
static int nm_trial_rhs(svl_nm* nm, int k) {
    TRY(nm_rhs(nm, k));
    double hs[S_NSCAL];
    nm_dot(nm, nm->b, nm->b, S_RP);
    TRY(nm_scalars(nm, hs));
    if (hs[S_RP] > 0.0) return SVL_OK;
    svl_cd* cd = nm->cd;
    const int n = nm->nf, tb = 256, g = (n + tb - 1) / tb;
    k_randn<<<g, tb, 0, cd->stream>>>(nm->e1, n, 0x5EEDull + (uint64_t)k);
    for (int sweep = 0; sweep < 3; ++sweep) {
        k_vmul<<<g, tb, 0, cd->stream>>>(nm->e1, nm->sdinv, nm->e2, n);
        TRY(nm_apply(nm, nm->e2, nm->q));
        k_smooth<<<g, tb, 0, cd->stream>>>(nm->e1, nm->q, nm->sdinv, 0.5, n);
    }
    k_vmul<<<g, tb, 0, cd->stream>>>(nm->e1, nm->sdinv, nm->e2, n);
    return nm_apply(nm, nm->e2, nm->b);
}

// Flexible-CG iterations the current network needs on the effective force of
// step k (a large number if it does not converge within the Jacobi budget);
// counters and state are left as they were.
static int64_t nm_trial(svl_nm* nm, int k) {
    const int64_t it_tot = nm->iters_total, it_last = nm->iters_last, ls = nm->learned_solves, fb = nm->fallbacks;
    const double res = nm->res_last;
    int64_t score = INT64_MAX / 4;
    if (nm_trial_rhs(nm, k) == SVL_OK) {
        nm->iters_last = 0;
        if (nm_solve_learned(nm, false) == SVL_OK) score = nm->iters_last;
    }
    nm->iters_total = it_tot; nm->iters_last = it_last; nm->learned_solves = ls; nm->fallbacks = fb; nm->res_last = res;
    return score;
}

// b = T^T (Fext - Fint + M(4/dt V + A - 4/dt^2 T dU)) - T^T (Keff SM), general T;
// dUt (total) must hold T dUf, smv the step's support-motion increment.
static int nmg_rhs(svl_nm* nm) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double dt = nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb;
    if (m.ndim == 2) k_nmg_rhs<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->ft, nm->dUt, 4.0 / dt, 4.0 / dt / dt);
    else k_nmg_rhs<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->ft, nm->dUt, 4.0 / dt, 4.0 / dt / dt);
    cd->launches += 1;
    const int eg = (m.nelem + 127) / 128;
    if (nm->consistent) {
        // + sum_e M_e (4/dt V + A - 4/dt^2 dU)_e (the diagonal above holds the nodal masses)
        DevView d = cd->d;
        double* blk = const_cast<double*>(cd->d.fem);
        k_nmg_wmass<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->dUt, 4.0 / dt, 4.0 / dt / dt, nm->wvec);
        if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->wvec, blk, 1.0, 0);
        else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->wvec, blk, 1.0, 0);
        if (m.ndim == 2) k_nmg_addblk<2><<<ng, tb, 0, cd->stream>>>(d, blk, nm->ft);
        else k_nmg_addblk<3><<<ng, tb, 0, cd->stream>>>(d, blk, nm->ft);
        cd->launches += 3;
    }
    if (nm->damped) {
        // + C (V - 2/dt dU) (NewmarkBeta.cpp:215)
        DevView d = cd->d;
        d.fe = nm->fe_op;
        k_nmg_wdamp<<<(m.ntotal + tb - 1) / tb, tb, 0, cd->stream>>>(d, nm->dUt, 2.0 / dt, nm->pt2);
        bool elem = false;
        if (d.dk0) {
            if (m.ndim == 2) k_element_tan<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->pt2, m.ngp, 0, 1.0);
            else k_element_tan<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->pt2, m.ngp, 0, 1.0);
            elem = true;
            cd->launches += 1;
        }
        if (nm->consistent) {               // am_e M_e with the consistent element mass, not the lumped diagonal
            if (nm->eam) {
                if (m.ndim == 2) k_mass_elem<2, 4><<<eg, 128, 0, cd->stream>>>(d, nm->pt2, nm->fe_op, 0.0, elem ? 1 : 0, nm->eam, 1.0);
                else k_mass_elem<3, 8><<<eg, 128, 0, cd->stream>>>(d, nm->pt2, nm->fe_op, 0.0, elem ? 1 : 0, nm->eam, 1.0);
                elem = true;
                cd->launches += 1;
            }
            d.Cd = nullptr;
        }
        if (m.ndim == 2) k_nmg_damp<2><<<ng, tb, 0, cd->stream>>>(d, nm->pt2, nm->ft, elem ? 1 : 0);
        else k_nmg_damp<3><<<ng, tb, 0, cd->stream>>>(d, nm->pt2, nm->ft, elem ? 1 : 0);
        cd->launches += 2;
    }
    const double* lg = nullptr;
    if (cd->has_sm) {
        // Keff SM (NewmarkBeta::ComputeSupportMotionVector, NewmarkBeta.cpp:180-194)
        TRY(nm_op_total(nm, nm->smv, nm->lg));
        lg = nm->lg;
    }
    k_nmg_reduce<<<(nm->nf + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, nm->ft, lg, nm->b);
    cd->launches += 1;
    CUDA_TRY(cudaGetLastError());
    return SVL_OK;
}

// Linear step with a general T and/or support motion.
static int nmg_step_linear(svl_nm* nm, double* U_hist_row) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double dt = nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb, eg = (m.nelem + 127) / 128, gt = (m.ntotal + tb - 1) / tb;
    k_step_inc<<<1, 1, 0, cd->stream>>>(cd->d.step);
    TRY(nm_drm(nm));
    if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    k_nmg_sm<<<gt, tb, 0, cd->stream>>>(cd->d, nm->smv);
    CUDA_TRY(cudaMemsetAsync(nm->dUt, 0, sizeof(double) * m.ntotal, cd->stream));
    cd->launches += 3;
    TRY(nmg_rhs(nm));
    TRY(nm_solve(nm));
    if (nm->rec_n > 0) TRY(nm_pairs_from_iterates(nm));
    k_nmg_expand<<<gt, tb, 0, cd->stream>>>(cd->d, nm->x, nm->dUt);
    if (m.ndim == 2) k_nmg_update<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, nm->smv, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    else k_nmg_update<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, nm->smv, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    cd->launches += 2;
    CUDA_TRY(cudaGetLastError());
    if (U_hist_row) CUDA_TRY(cudaMemcpyAsync(U_hist_row, cd->d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    return SVL_OK;
}

// One NewtonRaphson step (NewtonRaphson.cpp:24-75 with NewmarkBeta's effective
// force and stiffness): iterate Feff(current states, dU) -> tangent solve ->
// dU += du -> convergence test -> state update from U + dU.
static int nm_step_newton(svl_nm* nm, double* U_hist_row) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double dt = nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb, eg = (m.nelem + 127) / 128, n = nm->nf;
    const int gf = (n + tb - 1) / tb, gt = (m.ntotal + tb - 1) / tb;
    double hs[S_NSCAL];
    k_step_inc<<<1, 1, 0, cd->stream>>>(cd->d.step);
    TRY(nm_drm(nm));
    CUDA_TRY(cudaMemsetAsync(nm->dUf, 0, sizeof(double) * std::max(n, 1), cd->stream));
    if (nm->general) {
        k_nmg_sm<<<gt, tb, 0, cd->stream>>>(cd->d, nm->smv);
        CUDA_TRY(cudaMemsetAsync(nm->dUt, 0, sizeof(double) * m.ntotal, cd->stream));
    }
    double norm0 = 0.0, res = 0.0;
    int it = 0;
    for (;;) {
        if (nm->general) {
            TRY(nmg_rhs(nm));               // K SM with the current tangent, every iteration
        } else {
            TRY(nm_mass_rhs(nm, nm->dUf, 4.0 / dt / dt));
            if (m.ndim == 2) k_nm_rhs<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nm->dUf, 4.0 / dt / dt);
            else k_nm_rhs<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nm->dUf, 4.0 / dt / dt);
        }
        CUDA_TRY(cudaGetLastError());
        TRY(nm_solve(nm));                                  // x = du; b is left as it was
        k_axpy1<<<gf, tb, 0, cd->stream>>>(nm->dUf, nm->x, n);
        // the norms the convergence test reads (Algorithm.cpp:122-188)
        const int test = nm->opts.cnvgtest;
        double fn = 0.0, dn = 0.0, Dn = 0.0, en = 0.0;
        if (test == 1 || test == 4) nm_dot(nm, nm->b, nm->b, S_RP);
        if (test == 2 || test == 5 || test == 7) nm_dot2(nm, nm->x, nm->x, S_RZN, nm->dUf, nm->dUf, S_ZQ);
        if (test == 3 || test == 6) {
            k_vmul<<<gf, tb, 0, cd->stream>>>(nm->x, nm->b, nm->z, n);
            nm_dot(nm, nm->z, nm->z, S_RP);
        }
        if (test != 8) {
            TRY(nm_scalars(nm, hs));
            fn = en = std::sqrt(hs[S_RP]);
            dn = std::sqrt(hs[S_RZN]);
            Dn = std::sqrt(hs[S_ZQ]);
        }
        res = convergence_test(test, it, fn, dn, Dn, en, norm0);
        // UpdateStatesIncrements: element states from U + T dU (Algorithm.cpp:18-56)
        if (nm->general) {
            k_nmg_expand<<<gt, tb, 0, cd->stream>>>(cd->d, nm->dUf, nm->dUt);
            k_nmg_us<<<gt, tb, 0, cd->stream>>>(cd->d, nm->dUt);
        } else {
            k_nm_us<<<gt, tb, 0, cd->stream>>>(cd->d, nm->dUf);
        }
        if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
        else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
        cd->launches += 4;
        CUDA_TRY(cudaGetLastError());
        ++it;
        if (!(res > nm->opts.cnvgtol) || it >= nm->opts.maxit) break;
    }
    nm->newton_iters_last = it;
    nm->newton_iters_total += it;
    nm->newton_res_last = res;
    if (nm->general) {
        if (m.ndim == 2) k_nmg_update<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, nm->smv, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
        else k_nmg_update<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, nm->smv, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    } else {
        if (m.ndim == 2) k_nm_update<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUf, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
        else k_nm_update<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUf, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    }
    cd->launches += 1;
    CUDA_TRY(cudaGetLastError());
    if (U_hist_row) CUDA_TRY(cudaMemcpyAsync(U_hist_row, cd->d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    return SVL_OK;
}

// one step: effective force, solve, state update (d.step already advanced)
// One central-difference step with the non-diagonal K (CentralDifference.cpp:
// 124-152 with the effective force of 204-221): Fint from U, the element and
// diagonal parts of (M/dt^2 - C/2dt)(U - Up), the PCG solve, the update.
static int ncd_step(svl_nm* nm, double* U_hist_row) {
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double c_m = 1.0 / nm->opts.dt / nm->opts.dt, c_c = 1.0 / 2.0 / nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb, eg = (m.nelem + 127) / 128, gt = (m.ntotal + tb - 1) / tb;
    k_step_inc<<<1, 1, 0, cd->stream>>>(cd->d.step);
    if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    k_ncd_w<<<gt, tb, 0, cd->stream>>>(cd->d, nm->wvec);
    cd->launches += 3;
    // element parts of (M/dt^2 - C/2dt)(U - Up)
    const double* blk = ncd_elem(nm, nm->wvec, nm->blk_cd, c_m, -c_c);
    const double* Cd = nm->consistent ? nullptr : cd->d.Cd;
    if (!nm->cd_general) {
        if (m.ndim == 2) k_ncd_rhs<2><<<ng, tb, 0, cd->stream>>>(cd->d, blk, nm->wvec, nm->b, c_m, c_c, Cd);
        else k_ncd_rhs<3><<<ng, tb, 0, cd->stream>>>(cd->d, blk, nm->wvec, nm->b, c_m, c_c, Cd);
        cd->launches += 1;
    } else {
        // Feff = T^T R - T^T (K SM) (CentralDifference.cpp:189-201, 217-220)
        if (m.ndim == 2) k_ncd_rtotal<2><<<ng, tb, 0, cd->stream>>>(cd->d, blk, nm->wvec, nm->ft, c_m, c_c, Cd);
        else k_ncd_rtotal<3><<<ng, tb, 0, cd->stream>>>(cd->d, blk, nm->wvec, nm->ft, c_m, c_c, Cd);
        const double* lg = nullptr;
        if (cd->has_sm) {
            k_ncd_sm<<<gt, tb, 0, cd->stream>>>(cd->d, nm->smv);
            const double* bk = ncd_elem(nm, nm->smv, nm->fe_op, c_m, c_c);
            if (m.ndim == 2) k_ncd_total<2><<<ng, tb, 0, cd->stream>>>(cd->d, bk, nm->smv, nm->lg, c_m, c_c, Cd);
            else k_ncd_total<3><<<ng, tb, 0, cd->stream>>>(cd->d, bk, nm->smv, nm->lg, c_m, c_c, Cd);
            lg = nm->lg;
            cd->launches += 2;
        }
        k_nmg_reduce<<<(nm->nf + tb - 1) / tb, tb, 0, cd->stream>>>(cd->d, nm->ft, lg, nm->b);
        cd->launches += 2;
    }
    CUDA_TRY(cudaGetLastError());
    TRY(nm_solve(nm));
    if (!nm->cd_general) {
        if (m.ndim == 2) k_ncd_update<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->x, c_m, c_c, cd->d.flag);
        else k_ncd_update<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->x, c_m, c_c, cd->d.flag);
        cd->launches += 1;
    } else {
        k_nmg_expand<<<gt, tb, 0, cd->stream>>>(cd->d, nm->x, nm->dUt);
        const double* sm = cd->has_sm ? nm->smv : nullptr;
        if (m.ndim == 2) k_ncd_gupdate<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, sm, c_m, c_c, cd->d.flag);
        else k_ncd_gupdate<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->dUt, sm, c_m, c_c, cd->d.flag);
        cd->launches += 2;
    }
    CUDA_TRY(cudaGetLastError());
    if (U_hist_row) CUDA_TRY(cudaMemcpyAsync(U_hist_row, cd->d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    return SVL_OK;
}

static int nm_step(svl_nm* nm, double* U_hist_row) {
    if (nm->cdmode) return ncd_step(nm, U_hist_row);
    if (nm->newton) return nm_step_newton(nm, U_hist_row);
    if (nm->general) return nmg_step_linear(nm, U_hist_row);
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const double dt = nm->opts.dt;
    const int tb = 256, ng = (m.nnode + tb - 1) / tb, eg = (m.nelem + 127) / 128;
    k_step_inc<<<1, 1, 0, cd->stream>>>(cd->d.step);
    TRY(nm_drm(nm));
    // internal force from the committed state (filtered like the assembler)
    if (m.ndim == 2) k_element<2, 4><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    else k_element<3, 8><<<eg, 128, 0, cd->stream>>>(cd->d, cd->d.Us, m.ngp, 0);
    TRY(nm_mass_rhs(nm, nullptr, 0.0));
    if (m.ndim == 2) k_nm_rhs<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nullptr, 0.0);
    else k_nm_rhs<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->b, 4.0 / dt, nullptr, 0.0);
    cd->launches += 3;
    CUDA_TRY(cudaGetLastError());
    TRY(nm_solve(nm));
    if (nm->rec_n > 0) TRY(nm_pairs_from_iterates(nm));
    if (m.ndim == 2) k_nm_update<2><<<ng, tb, 0, cd->stream>>>(cd->d, nm->x, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    else k_nm_update<3><<<ng, tb, 0, cd->stream>>>(cd->d, nm->x, 4.0 / dt / dt, 4.0 / dt, 2.0 / dt, cd->d.flag);
    cd->launches += 1;
    CUDA_TRY(cudaGetLastError());
    if (U_hist_row) CUDA_TRY(cudaMemcpyAsync(U_hist_row, cd->d.U, sizeof(double) * m.ntotal, cudaMemcpyDeviceToHost, cd->stream));
    return SVL_OK;
}

extern "C" {

int svl_nm_run(svl_nm* nm, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!nm || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    svl_cd* cd = nm->cd;
    const HostModel& m = cd->m;
    const int64_t l0 = cd->launches;
    int kstart = k_first - 1;
    CUDA_TRY(cudaMemcpyAsync(cd->d.step, &kstart, sizeof(int), cudaMemcpyHostToDevice, cd->stream));
    for (int s = 0; s < nsteps; ++s) TRY(nm_step(nm, U_hist ? U_hist + (size_t)s * m.ntotal : nullptr));
    cd->launches_last = cd->launches - l0;
    int flag = 0;
    CUDA_TRY(cudaMemcpyAsync(&flag, cd->d.flag, sizeof(int), cudaMemcpyDeviceToHost, cd->stream));
    CUDA_TRY(cudaStreamSynchronize(cd->stream));
    if (flag) { set_error("non-finite displacement detected"); return SVL_ERR_NONFINITE; }
    return SVL_OK;
}

int svl_nm_run_timed(svl_nm* nm, int32_t k_first, int32_t nsteps, float* ms) {
    if (!nm || !ms) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); set_error("cudaEventCreate failed"); return SVL_ERR_CUDA; }
    int st = SVL_OK;
    if (cudaEventRecord(e0, nm->cd->stream) != cudaSuccess) st = SVL_ERR_CUDA;
    if (!st) st = svl_nm_run(nm, k_first, nsteps, nullptr);
    if (!st && cudaEventRecord(e1, nm->cd->stream) != cudaSuccess) st = SVL_ERR_CUDA;
    if (!st && cudaEventSynchronize(e1) != cudaSuccess) st = SVL_ERR_CUDA;
    if (!st && cudaEventElapsedTime(ms, e0, e1) != cudaSuccess) st = SVL_ERR_CUDA;
    if (st == SVL_ERR_CUDA) set_error("event timing failed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

int svl_nm_train_preconditioner(svl_nm* nm, int32_t k_first, const svl_nn_train_opts* o, float* loss) {
    if (!nm || !o) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("the learned preconditioner needs a hexahedral model whose nodes form a lattice"); return SVL_ERR_UNSUPPORTED; }
    if (o->solve_steps < 0 || o->n_synthetic < 0 || o->iters <= 0 || o->batch <= 0 || !(o->lr > 0.f) ||
        (o->solve_steps > 0 && o->record_every <= 0)) {
        set_error("bad training options");
        return SVL_ERR_INVALID;
    }
    svl_cd* cd = nm->cd;
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, cd->stream, &nm->nn));
    TRY(svl::nn_set_crop(nm->nn, o->crop));
    // 1. Newmark steps with Jacobi-PCG, recording CG iterates
    if (o->solve_steps > 0) {
        while ((int)nm->rec_x.size() < kRecMax) {
            double *xa = nullptr, *ra = nullptr;
            TRY(cd->zeros((size_t)nm->nf, &xa));
            TRY(cd->zeros((size_t)nm->nf, &ra));
            nm->rec_x.push_back(xa);
            nm->rec_r.push_back(ra);
        }
        nm->rec_every = o->record_every;
        nm->rec_n = 0;
        const int st = svl_nm_run(nm, k_first, o->solve_steps, nullptr);
        nm->rec_every = 0;
        nm->rec_n = 0;
        if (st) return st;
    }
    const int k_trial = k_first + o->solve_steps;       // the next step to be run
    // 2. synthetic pairs: e random with 0..5 smoothing sweeps, r_hat = A_hat e
    const int n = nm->nf, tb = 256, g = (n + tb - 1) / tb;
    const int max_sweeps = o->max_sweeps > 0 ? o->max_sweeps : 5;
    double hs[S_NSCAL];
    for (int i = 0; i < o->n_synthetic; ++i) {
        k_randn<<<g, tb, 0, cd->stream>>>(nm->e1, n, o->seed * 0x9E3779B97F4A7C15ull + (uint64_t)i * 0x100000001B3ull);
        // (the single-precision operator where the handle has one: training
        // data need no FP64 accuracy)
        for (int sweep = 0; sweep < i % (max_sweeps + 1); ++sweep) {
            k_vmul<<<g, tb, 0, cd->stream>>>(nm->e1, nm->sdinv, nm->e2, n);
            TRY(nm_apply(nm, nm->e2, nm->q, true));
            k_smooth<<<g, tb, 0, cd->stream>>>(nm->e1, nm->q, nm->sdinv, 0.5, n);
        }
        k_vmul<<<g, tb, 0, cd->stream>>>(nm->e1, nm->sdinv, nm->e2, n);
        TRY(nm_apply(nm, nm->e2, nm->q, true));
        k_vmul<<<g, tb, 0, cd->stream>>>(nm->q, nm->sdinv, nm->e2, n);
        nm_dot(nm, nm->e1, nm->e1, S_RP);
        TRY(nm_scalars(nm, hs));
        TRY(svl::nn_record_pair(nm->nn, nm->e2, nm->e1, 1.0 / std::sqrt(hs[S_RP])));
    }
    CUDA_TRY(cudaGetLastError());
    // 3. Adam in segments; after each, a trial flexible-CG solve on the
    //    effective force of the next step scores the network, and the
    //    best-scoring weights are kept (training loss alone does not track
    //    the iteration count).
    if (nm->jac_ref <= 0) {                 // the trial budget is a plain Jacobi solve
        TRY(nm_trial_rhs(nm, k_trial));
        nm->iters_last = 0;
        const int64_t it_tot = nm->iters_total;
        TRY(nm_solve_jacobi(nm, false, nm->opts.pcg_maxit));
        nm->iters_total = it_tot;
    }
    const int nseg = std::max(1, std::min(o->iters / 250, 16));
    std::vector<float> best_w(svl::kNnWeights);
    int64_t best = INT64_MAX;
    float l = 0.f, best_loss = 0.f;
    for (int sgm = 0; sgm < nseg; ++sgm) {
        const int i0 = (int)((int64_t)o->iters * sgm / nseg), i1 = (int)((int64_t)o->iters * (sgm + 1) / nseg);
        TRY(svl::nn_train_segment(nm->nn, i0, i1, o->iters, o->batch, o->lr, o->seed, &l));
        const int64_t score = nm_trial(nm, k_trial);
        if (score <= best) {
            best = score;
            best_loss = l;
            TRY(svl::nn_get_weights(nm->nn, best_w.data()));
        }
    }
    TRY(svl::nn_set_weights(nm->nn, best_w.data()));
    nm->train_trial_iters = best;
    if (loss) *loss = best_loss;
    nm->precond = SVL_PRECOND_LEARNED;
    return SVL_OK;
}

int svl_nm_set_preconditioner(svl_nm* nm, int32_t precond) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (precond == SVL_PRECOND_JACOBI) { nm->precond = precond; return SVL_OK; }
    if (precond != SVL_PRECOND_LEARNED) { set_error("unknown preconditioner %d", precond); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("the learned preconditioner needs a hexahedral model whose nodes form a lattice"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    nm->precond = precond;
    return SVL_OK;
}

int svl_nn_num_weights(void) { return svl::kNnWeights; }

int svl_nm_preconditioner_weights(svl_nm* nm, float* w_out, const float* w_in) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("no learned preconditioner on this model"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    if (w_in) TRY(svl::nn_set_weights(nm->nn, w_in));
    if (w_out) TRY(svl::nn_get_weights(nm->nn, w_out));
    return SVL_OK;
}

int svl_nm_precond_stats(svl_nm* nm, int64_t* learned_solves, int64_t* fallbacks, int64_t* jacobi_ref_iters) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (learned_solves) *learned_solves = nm->learned_solves;
    if (fallbacks) *fallbacks = nm->fallbacks;
    if (jacobi_ref_iters) *jacobi_ref_iters = nm->jac_ref;
    return SVL_OK;
}

int svl_nm_lattice(svl_nm* nm, int32_t* dims) {
    if (!nm || !dims) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    dims[0] = nm->lattice ? nm->lnx : 0;
    dims[1] = nm->lattice ? nm->lny : 0;
    dims[2] = nm->lattice ? nm->lnz : 0;
    return SVL_OK;
}

int svl_nm_nn_loss_grad(svl_nm* nm, const float* x, const float* t, float* loss, float* grad) {
    if (!nm || !x || !t || !loss || !grad) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("no learned preconditioner on this model"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    return svl::nn_loss_grad_host(nm->nn, x, t, loss, grad);
}

int svl_nm_nn_forward(svl_nm* nm, const float* x, float* y, int32_t path) {
    if (!nm || !x || !y) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("no learned preconditioner on this model"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    return svl::nn_forward_host(nm->nn, x, y, path);
}

int svl_nm_nn_set_path(svl_nm* nm, int32_t path) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (path != 0 && path != 1) { set_error("path must be 0 (CUDA cores) or 1 (tensor cores)"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("no learned preconditioner on this model"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    svl::nn_set_path(nm->nn, path);
    return SVL_OK;
}

int svl_nm_nn_grids(svl_nm* nm, float* rho, float* mask) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (!nm->lattice) { set_error("no learned preconditioner on this model"); return SVL_ERR_UNSUPPORTED; }
    if (!nm->nn) TRY(svl::nn_create(nm->lnx, nm->lny, nm->lnz, nm->gmap, nm->sdinv_h, nm->rho_h, nm->cd->stream, &nm->nn));
    return svl::nn_get_grids(nm->nn, rho, mask);
}

void* svl_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, std::max<size_t>(bytes, 1), cudaHostAllocDefault) != cudaSuccess) {
        set_error("cudaHostAlloc of %zu bytes failed", bytes);
        return nullptr;
    }
    return p;
}

void svl_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

int svl_nm_get(svl_nm* nm, int32_t which, double* out) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    return svl_cd_get(nm->cd, which, out);
}

int svl_nm_reaction(svl_nm* nm, int32_t k, double* R) {
    if (!nm || !R) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    if (nm->consistent || nm->cdmode) {
        set_error("reaction forces are covered with a lumped mass and a diagonal central-difference system");
        return SVL_ERR_UNSUPPORTED;
    }
    return cd_reaction(nm->cd, k, 0, R);
}

int svl_nm_element_response(svl_nm* nm, int32_t response, int32_t nlist, const int32_t* elems, double* out) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    return cd_element_response(nm->cd, nm->cdmode ? 1 : 0, response, nlist, elems, out);
}

int svl_nm_stats(svl_nm* nm, int64_t* iters_total, int64_t* iters_last, double* rel_residual_last) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (iters_total) *iters_total = nm->iters_total;
    if (iters_last) *iters_last = nm->iters_last;
    if (rel_residual_last) *rel_residual_last = nm->res_last;
    return SVL_OK;
}

int svl_nm_newton_stats(svl_nm* nm, int64_t* iters_total, int64_t* iters_last, double* residual_last) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (iters_total) *iters_total = nm->newton_iters_total;
    if (iters_last) *iters_last = nm->newton_iters_last;
    if (residual_last) *residual_last = nm->newton_res_last;
    return SVL_OK;
}

int svl_nm_launch_count(svl_nm* nm, int64_t* launches) {
    if (!nm || !launches) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *launches = nm->cd->launches_last;
    return SVL_OK;
}

int svl_nm_sync(svl_nm* nm) {
    if (!nm) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    return svl_cd_sync(nm->cd);
}

void svl_nm_destroy(svl_nm* nm) { delete nm; }

}  // extern "C"
