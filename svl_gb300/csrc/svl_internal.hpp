// Internal host-side model representation shared by the C-ABI translation
// units.  Not installed; the public interface is include/svl_gb300.h.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/svl_gb300.h"

namespace svl {

void set_error(const char* fmt, ...);

// Algorithm::ComputeConvergence (RP/09-Algorithms/Algorithm.cpp:122-188) from
// the 2-norms of the effective force F, of the iteration's increment du, of
// the accumulated increment dU and of du .* F, at iteration `it` (0-based);
// norm0 holds the first iteration's reference for the relative tests.
//   1 |F|  2 |du|  3 |du.*F|  4 |F|/|F_0|  5 |du|/|dU_0|  6 |du.*F|/|(du.*F)_0|
//   7 |du|/|dU|  8 -1 (the loop stops after one iteration)
inline double convergence_test(int test, int it, double fn, double dn, double Dn, double en, double& norm0) {
    switch (test) {
    case 1: return fn;
    case 2: return dn;
    case 3: return en;
    case 4: if (it == 0) { norm0 = fn; return fn; } return fn / norm0;
    case 5: if (it == 0) { norm0 = Dn; return dn; } return dn / norm0;
    case 6: if (it == 0) { norm0 = en; return en; } return en / norm0;
    case 7: return dn / Dn;
    default: return -1.0;
    }
}

// Gauss abscissa of the 2x2 / 2x2x2 rules, truncated to 15 digits exactly as
// RP/04-Elements/11-Integration/GaussQuadrature.cpp:303-316 tabulates it.
constexpr double kGaussAbscissa = 0.577350269189626;

struct HostModel {
    int ndim = 0, nnode = 0, ndof = 0, ntotal = 0, nfree = 0;   // ndof = ndim (solid dofs per node)
    int etype = 0, nelem = 0, nen = 0, ngp = 0, nstr = 0, nmat = 0;
    std::vector<double> X;
    std::vector<int32_t> tdof, fdof, conn, emat;   // tdof/fdof: the first ndim dofs, [nnode][ndim]
    // every dof of every node (PML nodes carry 5 / 9): [nnode][dstride], count nndof[n]
    int dstride = 0;
    std::vector<int32_t> nndof, tdof_all, fdof_all;
    std::vector<int32_t> epml;        // [nelem] 1 for a PML element (empty: none)
    std::vector<double> pml_par;      // [nelem][3 + 2 ndim] n, L, R, x0, npml
    std::vector<int32_t> dp_dof;      // [ndashpot][2] total dofs of the Lysmer dashpots
    std::vector<double> dp_eta;       // [ndashpot]
    std::vector<double> thick;
    std::vector<int32_t> mtype;
    std::vector<double> mpar;
    std::vector<double> nodemass;
    std::vector<double> ray;          // [nelem][2] Rayleigh (am, ak), empty when undamped
    int nconstraint = 0;
    std::vector<int32_t> cslave, cptr, cmaster;
    std::vector<double> cfactor;
    int lumped = 1;
    // row-sum lumped element masses [(e nen + a) nd + j], filled by the first
    // caller that needs them (the model does not change afterwards)
    mutable std::vector<double> elem_lumped;

    bool has_j2() const;
    bool has_pml() const { return !epml.empty(); }
    int pml_ndof() const { return ndim == 2 ? 5 : 9; }
    const double* param(int e) const { return &mpar[(size_t)emat[e] * SVL_MAT_NPARAM]; }
    int mat_type(int e) const { return mtype[emat[e]]; }
};

// Validates a descriptor and copies it; returns false with svl_last_error set.
bool model_from_desc(const svl_model_desc* d, HostModel& m);

// Physical shape-function derivatives dN_a/dx_j, shape values N_a and the
// Jacobian determinant at Gauss point q of element e.  Same kinematics as
// lin2DQuad4.cpp:648-710 and lin3DHexa8.cpp:756-853.
double gp_geometry(const HostModel& m, int e, int q, double dNx[8][3], double N[8]);

// Integration factor w * t * |detJ| (2D) or w * |detJ| (3D), w = 1.
inline double gp_factor(const HostModel& m, int e, double det) {
    return m.ndim == 2 ? 1.0 * m.thick[e] * (det < 0 ? -det : det) : 1.0 * (det < 0 ? -det : det);
}

// body(begin, end) over [0, n) split across the host's hardware threads.
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& body);

// Diagonal of the assembled row-sum-lumped mass on total dofs.
void lumped_mass_diag(const HostModel& m, double mtol, std::vector<double>& M);
// row-sum lumped mass of every element node and component, [(e nen + a) nd + j]
void element_lumped_masses(const HostModel& m, std::vector<double>& diag);
// Dashpot couplings per total dof, CSR: y_t += c * sum eta (x_t - x_partner)
// for every dashpot that touches t (element order); empty without dashpots.
void dashpot_tables(const HostModel& m, std::vector<int32_t>& ptr, std::vector<int32_t>& col,
                    std::vector<double>& eta);
// Mass-proportional Rayleigh damping on total dofs, sum_e am_e M_e with the
// element row-sum lumped masses (lin2DQuad4.cpp:360-366 with a lumped mass)
void rayleigh_mass_diag(const HostModel& m, std::vector<double>& C);

// Load descriptor as per-total-dof CSR tables: force entries (series, coef)
// and support-motion entries (series, factor) grouped by dof in input order.
struct LoadTables {
    std::vector<int32_t> s_ptr{0};
    std::vector<double> s_val;
    std::vector<int32_t> ld_ptr, ld_ser, sm_ptr, sm_ser;
    std::vector<double> ld_coef, sm_fac;
    bool has_sm = false;
};
// Returns SVL_OK or an error code with svl_last_error set.
int build_load_tables(const HostModel& m, const svl_load_desc* L, LoadTables& out);

// Tables of the explicit central difference with PML layers (see
// explicit_pml_tables in svl_host.cpp): per total dof the stress-dof flag and
// the lumped diagonals of the displacement rows; per free dof 1/(T^T d T)
// (0 on stress dofs); per PML node (in node order) the first total dof of its
// stress block and the ns x ns lumped blocks and the inverse of
// Ms/dt^2 + Cs/2dt; snode_of[n] is the PML node index of node n or -1.
struct ExplicitPmlTables {
    int ns = 0;
    std::vector<int8_t> sdof;
    std::vector<int32_t> sfirst, snode_of;
    std::vector<double> Mu, Cu, Ku, Gu, kinv;
    std::vector<double> Ms, Cs, Ks, Gs, Dinv;
};
int explicit_pml_tables(const HostModel& m, double dt, double mtol, const LoadTables& lt, ExplicitPmlTables& out);

// PML element action y_e = coef_M M u_M + coef_C C u_C + coef_K K u_K + coef_G G u_G
// (PML2DQuad4 / PML3DHexa8), one thread per element; see svl_pml.cu.
struct PmlArgs {
    int nelem;
    const double* X;       // [nelem][nen][nd]
    const double* mat;     // [nelem][3]  E, nu, rho
    const double* thick;   // [nelem] (2D) or null
    const double* par;     // [nelem][3 + 2 nd]  m, L, R, x0[nd], n[nd]
    double coef[4];        // M, C, K, G
    const double* u[4];    // [nelem][nc] each, or total-dof vectors when edof is set (null when the coefficient is 0)
    const int32_t* edof;   // [nelem][nc] total dof of each element dof (gather mode), or null
    double* y;             // [nelem][nc]
    double ftol;           // >= 0: entries with |y| <= ftol are dropped (force filter)
    double yscale;         // y is scaled by this after the filter
    int accumulate;        // 1: y += result
    int single;            // 1: single-precision arithmetic (inner solver iterations)
    const float* tab;      // [nelem][pml_tab_stride(nd)] single-precision element constants
                           // (pml_tab_fill), or null; used by the single-precision operator
    float coef_f[4];       // coef in single precision (set by pml_action_launch)
    const float* u_f;      // single precision, gather mode: the input vector in float and
    float* y_f;            // the element vectors in float (no filter, scale or accumulate)
};
// per element: node coordinates relative to node 0 [nen][nd], node 0 - x0 [nd],
// n [nd], then mu, lambda, rho, a0, b0, m, L, thickness
inline int pml_tab_stride(int nd) { return ((nd == 2 ? 4 : 8) * nd + 2 * nd + 8 + 3) / 4 * 4; }
void pml_tab_fill(int nd, int nelem, const double* X, const double* mat, const double* thick, const double* par,
                  std::vector<float>& tab);
int pml_action_launch(int ndim, const PmlArgs& A, cudaStream_t st);

// T (total <- free) rows as CSR over total dofs, sorted columns, duplicates summed.
void build_total_to_free(const HostModel& m, std::vector<int32_t>& ptr,
                         std::vector<int32_t>& col, std::vector<double>& val);

}  // namespace svl
