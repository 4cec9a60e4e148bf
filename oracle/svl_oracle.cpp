/*
 * svl_oracle.cpp -- CPU FP64 restatement of SeismoVLAB's time-stepping hot
 * path.  TEST INFRASTRUCTURE ONLY: this file is the checker the GPU path is
 * compared against (tests/, __graft_entry__.smoke(), bench.py's CPU baseline
 * arm).  Nothing in the svl_gb300 product links or calls it.
 *
 * It follows the reference's structure on purpose ("reference-faithful"):
 * Jacobian, its inverse and the strain-displacement matrix are recomputed at
 * every Gauss point on every call; element contributions are summed in
 * element-tag order with the assembler's tolerance filters; the central
 * difference update is the diagonal solve of (M/dt^2) with Eigen's
 * (1/d)*b convention.  A second, "fast" internal-force routine (precomputed
 * Gauss-point geometry, OpenMP over elements, same summation order) exists
 * only to time a multi-core CPU baseline.
 *
 * Parity status: pinned against the reference's own artefacts where they
 * exist -- the pre-processor's numbering (tests/golden/, generated by running
 * PP/ on small models) and the OpenSees histories shipped with the
 * validation cases F02/F03/J02 (03-Validations/01-Debugging) -- but not
 * against the SVL binary, which cannot be built without Eigen/PETSc/MUMPS.
 *
 * Citations are relative to the SVL tree: RP/ = 02-Run_Process/.
 * Compile with -ffp-contract=off so x86 and Arm hosts round identically.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <string>
#include <algorithm>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/svl_gb300.h"

namespace {

/* Gauss points: RP/04-Elements/11-Integration/GaussQuadrature.cpp:303-316
 * (quad, r fastest) and the hexa table below it (r, then s, then t); the
 * abscissa is the 15-digit truncated 1/sqrt(3) with unit weights. */
const double kGauss = 0.577350269189626;

struct Model {
    int ndim, nnode, ndof, ntotal, nfree, nelem, nen, ngp, nstr, etype;
    std::vector<double> X;            // [nnode][ndim]
    std::vector<int> tdof, fdof;      // [nnode][ndof] the first ndim dofs (ndof = ndim)
    int dstride;                      // stride of the descriptor's dof rows
    std::vector<int> nndof, tdof_all, fdof_all;   // every dof of a node (PML nodes 5 / 9)
    std::vector<int> epml;            // [nelem] PML flag, empty without PML
    std::vector<double> pml_par;      // [nelem][3 + 2 ndim]
    std::vector<int> dp_dof;          // [ndashpot][2] Lysmer dashpots (ZeroLength1D + Viscous1DLinear)
    std::vector<double> dp_eta;
    std::vector<int> conn, emat;
    std::vector<double> thick;
    std::vector<int> mtype;
    std::vector<double> mpar;
    std::vector<double> nodemass;     // [ntotal] or empty
    std::vector<double> ray;          // [nelem][2] Rayleigh (am, ak) or empty
    int nconstraint;
    std::vector<int> cslave, cptr, cmaster;
    std::vector<double> cfactor;
    int lumped;
};

struct Loads {
    std::vector<int> sptr; std::vector<double> sval;
    std::vector<int> fdof, fser; std::vector<double> fcoef;
    std::vector<int> smdof, smser; std::vector<double> smfac;
    // domain reduction: entries (element, factor), node rows into the motion, exterior flags
    std::vector<int> drm_elem; std::vector<double> drm_factor;
    int drm_nt = 0;
    std::vector<int> drm_row, drm_ext;
    std::vector<double> drm_motion;
    double series(int s, int k) const {            // Load::GetLoadVector (Load.cpp:69-71)
        int n = sptr[s + 1] - sptr[s];
        return (k >= 0 && k < n) ? sval[sptr[s] + k] : 0.0;
    }
    double support(int s, int k) const {           // Node::GetSupportMotion (Node.cpp:228-247)
        int n = sptr[s + 1] - sptr[s];
        if (n <= 0) return 0.0;
        return (k >= 0 && k < n) ? sval[sptr[s] + k] : sval[sptr[s]];   // k < 0: out of range (unsigned)
    }
};

bool load_model(const svl_model_desc* d, Model& m) {
    if (!d) return false;
    m.ndim = d->ndim; m.nnode = d->nnode; m.ndof = d->ndof;
    m.ntotal = d->ntotal; m.nfree = d->nfree; m.nelem = d->nelem; m.etype = d->elem_type;
    if (m.etype == SVL_ELEM_LIN2DQUAD4) { m.nen = 4; m.ngp = 4; m.nstr = 3; if (m.ndim != 2) return false; }
    else if (m.etype == SVL_ELEM_LIN3DHEXA8) { m.nen = 8; m.ngp = 8; m.nstr = 6; if (m.ndim != 3) return false; }
    else return false;
    const int pnd = m.ndim == 2 ? 5 : 9;
    m.dstride = d->ndof;
    if (m.dstride != m.ndim && m.dstride != pnd) return false;
    m.ndof = m.ndim;
    m.X.assign(d->coords, d->coords + (size_t)m.nnode * m.ndim);
    m.nndof.assign(m.nnode, m.dstride);
    if (d->node_ndof) m.nndof.assign(d->node_ndof, d->node_ndof + m.nnode);
    m.tdof_all.assign((size_t)m.nnode * m.dstride, -1);
    m.fdof_all.assign((size_t)m.nnode * m.dstride, -1);
    m.tdof.assign((size_t)m.nnode * m.ndim, -1);
    m.fdof.assign((size_t)m.nnode * m.ndim, -1);
    for (int n = 0; n < m.nnode; ++n)
        for (int j = 0; j < m.nndof[n]; ++j) {
            const size_t i = (size_t)n * m.dstride + j;
            m.tdof_all[i] = d->totaldof[i]; m.fdof_all[i] = d->freedof[i];
            if (j < m.ndim) { m.tdof[(size_t)n * m.ndim + j] = d->totaldof[i]; m.fdof[(size_t)n * m.ndim + j] = d->freedof[i]; }
        }
    m.epml.clear(); m.pml_par.clear();
    if (d->elem_pml) {
        bool any = false;
        for (int e = 0; e < m.nelem; ++e) any |= d->elem_pml[e] != 0;
        if (any) {
            if (!d->elem_pml_param) return false;
            m.epml.assign(m.nelem, 0);
            for (int e = 0; e < m.nelem; ++e) m.epml[e] = d->elem_pml[e] != 0;
            m.pml_par.assign(d->elem_pml_param, d->elem_pml_param + (size_t)m.nelem * (3 + 2 * m.ndim));
        }
    }
    m.conn.assign(d->conn, d->conn + (size_t)m.nelem * m.nen);
    m.emat.assign(d->elem_mat, d->elem_mat + m.nelem);
    m.thick.assign(m.nelem, 1.0);
    if (d->elem_thickness) m.thick.assign(d->elem_thickness, d->elem_thickness + m.nelem);
    m.mtype.assign(d->mat_type, d->mat_type + d->nmat);
    m.mpar.assign(d->mat_param, d->mat_param + (size_t)d->nmat * SVL_MAT_NPARAM);
    if (d->node_mass) m.nodemass.assign(d->node_mass, d->node_mass + m.ntotal);
    if (d->elem_rayleigh) m.ray.assign(d->elem_rayleigh, d->elem_rayleigh + (size_t)2 * m.nelem);
    m.dp_dof.clear(); m.dp_eta.clear();
    if (d->ndashpot > 0) {
        m.dp_dof.assign(d->dashpot_dof, d->dashpot_dof + 2 * (size_t)d->ndashpot);
        m.dp_eta.assign(d->dashpot_eta, d->dashpot_eta + d->ndashpot);
    }
    m.nconstraint = d->nconstraint;
    if (m.nconstraint > 0) {
        m.cslave.assign(d->con_slave, d->con_slave + m.nconstraint);
        m.cptr.assign(d->con_ptr, d->con_ptr + m.nconstraint + 1);
        m.cmaster.assign(d->con_master, d->con_master + m.cptr.back());
        m.cfactor.assign(d->con_factor, d->con_factor + m.cptr.back());
    }
    m.lumped = d->lumped;
    return true;
}

void load_loads(const svl_load_desc* l, Loads& L, int nnode, int ndim) {
    L.sptr.assign(1, 0);
    if (!l) return;
    if (l->ndrm > 0) {
        L.drm_elem.assign(l->drm_elem, l->drm_elem + l->ndrm);
        L.drm_factor.assign(l->drm_factor, l->drm_factor + l->ndrm);
        L.drm_nt = l->drm_nt;
        L.drm_row.assign(l->drm_node_row, l->drm_node_row + nnode);
        L.drm_ext.assign(l->drm_node_ext, l->drm_node_ext + nnode);
        int nb = 0;
        for (int r : L.drm_row) nb = std::max(nb, r + 1);
        L.drm_motion.assign(l->drm_motion, l->drm_motion + (size_t)nb * l->drm_nt * 3 * ndim);
    }
    if (l->nseries > 0) {
        L.sptr.assign(l->series_ptr, l->series_ptr + l->nseries + 1);
        L.sval.assign(l->series_val, l->series_val + L.sptr.back());
    }
    if (l->nforce > 0) {
        L.fdof.assign(l->force_dof, l->force_dof + l->nforce);
        L.fser.assign(l->force_series, l->force_series + l->nforce);
        L.fcoef.assign(l->force_coef, l->force_coef + l->nforce);
    }
    if (l->nsupport > 0) {
        L.smdof.assign(l->sm_dof, l->sm_dof + l->nsupport);
        L.smser.assign(l->sm_series, l->sm_series + l->nsupport);
        L.smfac.assign(l->sm_factor, l->sm_factor + l->nsupport);
    }
}

/* ---------------- materials (per Gauss point) ---------------------------- */

struct MatState {                  // committed + trial state of one Gauss point
    double strain[6], stress[6], ep[6], back[6], alpha;
    double ep_n[6], back_n[6], alpha_n, strain_n[6], stress_n[6];
    double tangent[36], tangent_n[36];
};

// 6x6 helpers of the J2 models (PlasticPlaneStrainJ2.cpp:282-350).
void j2_identity_tensor(double D[36]) {          // 1 (x) 1 on the normal block
    for (int i = 0; i < 36; ++i) D[i] = 0.0;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) D[i * 6 + j] = 1.0;
}
void j2_identity_operator(double I[36]) {        // symmetric identity, 1/2 on shear
    for (int i = 0; i < 36; ++i) I[i] = 0.0;
    for (int i = 0; i < 3; ++i) I[i * 6 + i] = 1.0;
    for (int i = 3; i < 6; ++i) I[i * 6 + i] = 0.5;
}
double j2_norm(const double T[6]) {
    return std::sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2] + 2.0 * (T[3] * T[3] + T[4] * T[4] + T[5] * T[5]));
}

void j2_elastic_tangent(double K, double G, double C[36]) {
    double D[36], I[36];
    j2_identity_tensor(D); j2_identity_operator(I);
    for (int i = 0; i < 36; ++i) C[i] = K * D[i] + 2.0 * G * (I[i] - 1.0 / 3.0 * D[i]);
}

void mat_init(MatState& s, int type, const double* p) {
    std::memset(&s, 0, sizeof(s));
    if (type == SVL_MAT_PLASTICPLANESTRAINJ2 || type == SVL_MAT_PLASTIC3DJ2) {
        j2_elastic_tangent(p[0], p[1], s.tangent);
        std::memcpy(s.tangent_n, s.tangent, sizeof(s.tangent));
    }
}

/* J2 radial return on the 6-vector tensor strain E (shear = 1/2 gamma):
 * PlasticPlaneStrainJ2::UpdateState (PlasticPlaneStrainJ2.cpp:227-279) and
 * Plastic3DJ2::UpdateState (Plastic3DJ2.cpp:206-255) share this arithmetic.
 * Like the reference, the update starts from the current (not the last
 * committed) plastic strain, back stress and hardening variable. */
void j2_update(MatState& s, const double* p, const double E[6]) {
    const double K = p[0], G = p[1], H = p[3], beta = p[4], SY = p[5];
    const double one[6] = {1, 1, 1, 0, 0, 0};
    double D[36], I[36], Id[36];
    j2_identity_tensor(D); j2_identity_operator(I);
    for (int i = 0; i < 36; ++i) Id[i] = I[i] - 1.0 / 3.0 * D[i];
    for (int i = 0; i < 6; ++i) s.strain[i] = E[i];
    double tr = E[0] + E[1] + E[2];
    double dev[6], trial[6], rel[6];
    for (int i = 0; i < 6; ++i) dev[i] = E[i] - 1.0 / 3.0 * tr * one[i];
    for (int i = 0; i < 6; ++i) trial[i] = 2.0 * G * (dev[i] - s.ep[i]);
    for (int i = 0; i < 6; ++i) rel[i] = trial[i] - s.back[i];
    double nrm = j2_norm(rel);
    double f = nrm - std::sqrt(2.0 / 3.0) * (SY + s.alpha * beta * H);
    if (f <= 0) {
        for (int i = 0; i < 36; ++i) s.tangent[i] = K * D[i] + 2.0 * G * Id[i];
        for (int i = 0; i < 6; ++i) s.stress[i] = K * tr * one[i] + trial[i];
    } else {
        double n[6];
        for (int i = 0; i < 6; ++i) n[i] = rel[i] / nrm;
        double dg = f / (2.0 * G + 2.0 / 3.0 * H);
        s.alpha += std::sqrt(2.0 / 3.0) * dg;
        for (int i = 0; i < 6; ++i) s.back[i] += 2.0 / 3.0 * (1.0 - beta) * H * dg * n[i];
        for (int i = 0; i < 6; ++i) s.ep[i] += dg * n[i];
        for (int i = 0; i < 6; ++i) s.stress[i] = K * tr * one[i] + trial[i] - 2.0 * G * dg * n[i];
        double c1 = 1.0 / (1.0 + H / G / 3.0), c2 = 4.0 * G * G * dg / nrm;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double nn = n[i] * n[j];
                s.tangent[i * 6 + j] = K * D[i * 6 + j] + 2.0 * G * (Id[i * 6 + j] - c1 * nn) - c2 * (Id[i * 6 + j] - nn);
            }
    }
}

/* Material::UpdateState(strain, 1) for the engineering strain vector of the
 * element (3 entries in 2D: xx, yy, gamma_xy; 6 in 3D). */
void mat_update(MatState& s, int type, const double* p, const double* eps) {
    if (type == SVL_MAT_ELASTIC2DPLANESTRAIN) {
        for (int i = 0; i < 3; ++i) s.strain[i] = eps[i];
    } else if (type == SVL_MAT_ELASTIC3DLINEAR) {
        for (int i = 0; i < 6; ++i) s.strain[i] = eps[i];
    } else if (type == SVL_MAT_PLASTICPLANESTRAINJ2) {
        // plane strain mapped to [0, exx, eyy, 0, gxy/2, 0] (PlasticPlaneStrainJ2.cpp:236)
        double E[6] = {0.0, eps[0], eps[1], 0.0, 0.5 * eps[2], 0.0};
        j2_update(s, p, E);
    } else {
        // (Plastic3DJ2.cpp:215)
        double E[6] = {eps[0], eps[1], eps[2], 0.5 * eps[3], 0.5 * eps[4], 0.5 * eps[5]};
        j2_update(s, p, E);
    }
}

void elastic_coeffs(const double* p, double& c1, double& c2, double& c3) {
    const double E = p[0], nu = p[1];
    c1 = E * (1.0 - nu) / (1.0 - 2.0 * nu) / (1.0 + nu);
    c2 = E * nu / (1.0 - 2.0 * nu) / (1.0 + nu);
    c3 = E / (2.0 * (1.0 + nu));
}

// Material::GetStress (Elastic2DPlaneStrain.cpp:96-99, Elastic3DLinear.cpp:97,
// PlasticPlaneStrainJ2.cpp:123-128 returns indices 1,2,4).
void mat_stress(const MatState& s, int type, const double* p, double* sig) {
    if (type == SVL_MAT_ELASTIC2DPLANESTRAIN) {
        double c1, c2, c3; elastic_coeffs(p, c1, c2, c3);
        sig[0] = c1 * s.strain[0] + c2 * s.strain[1];
        sig[1] = c2 * s.strain[0] + c1 * s.strain[1];
        sig[2] = c3 * s.strain[2];
    } else if (type == SVL_MAT_ELASTIC3DLINEAR) {
        double c1, c2, c3; elastic_coeffs(p, c1, c2, c3);
        const double* e = s.strain;
        sig[0] = c1 * e[0] + c2 * e[1] + c2 * e[2];
        sig[1] = c2 * e[0] + c1 * e[1] + c2 * e[2];
        sig[2] = c2 * e[0] + c2 * e[1] + c1 * e[2];
        sig[3] = c3 * e[3]; sig[4] = c3 * e[4]; sig[5] = c3 * e[5];
    } else if (type == SVL_MAT_PLASTICPLANESTRAINJ2) {
        sig[0] = s.stress[1]; sig[1] = s.stress[2]; sig[2] = s.stress[4];
    } else {
        for (int i = 0; i < 6; ++i) sig[i] = s.stress[i];
    }
}

// Material::GetTangentStiffness (nstr x nstr, row-major).
void mat_tangent(const MatState& s, int type, const double* p, double* C) {
    if (type == SVL_MAT_ELASTIC2DPLANESTRAIN) {
        double c1, c2, c3; elastic_coeffs(p, c1, c2, c3);
        double T[9] = {c1, c2, 0, c2, c1, 0, 0, 0, c3};
        std::memcpy(C, T, sizeof(T));
    } else if (type == SVL_MAT_ELASTIC3DLINEAR) {
        double c1, c2, c3; elastic_coeffs(p, c1, c2, c3);
        for (int i = 0; i < 36; ++i) C[i] = 0.0;
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C[i * 6 + j] = (i == j) ? c1 : c2;
        for (int i = 3; i < 6; ++i) C[i * 6 + i] = c3;
    } else if (type == SVL_MAT_PLASTICPLANESTRAINJ2) {
        // (PlasticPlaneStrainJ2.cpp:151-159) rows/cols 1,2,4 of the 6x6 tangent
        const int ix[3] = {1, 2, 4};
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C[i * 3 + j] = s.tangent[ix[i] * 6 + ix[j]];
    } else {
        std::memcpy(C, s.tangent, sizeof(double) * 36);
    }
}

void mat_commit(MatState& s) {
    std::memcpy(s.ep_n, s.ep, sizeof(s.ep)); std::memcpy(s.back_n, s.back, sizeof(s.back));
    s.alpha_n = s.alpha;
    std::memcpy(s.strain_n, s.strain, sizeof(s.strain)); std::memcpy(s.stress_n, s.stress, sizeof(s.stress));
    std::memcpy(s.tangent_n, s.tangent, sizeof(s.tangent));
}

double mat_density(int type, const double* p) { (void)type; return p[2]; }

/* ---------------- element kinematics ------------------------------------- */

void gauss_point(int nd, int q, double xi[3]) {
    xi[0] = (q & 1) ? kGauss : -kGauss;
    xi[1] = (q & 2) ? kGauss : -kGauss;
    xi[2] = (q & 4) ? kGauss : -kGauss;
    if (nd == 2) xi[2] = 0.0;
}

// Natural derivatives dN_a/dr_i of the bilinear / trilinear shape functions,
// node order of lin2DQuad4.cpp:648-667 and lin3DHexa8.cpp:756-807.
void shape_derivs(int nd, const double* xi, double dN[8][3], double N[8]) {
    if (nd == 2) {
        const double sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
        for (int a = 0; a < 4; ++a) {
            N[a] = 0.25 * (1.0 + sr[a] * xi[0]) * (1.0 + ss[a] * xi[1]);
            dN[a][0] = 0.25 * sr[a] * (1.0 + ss[a] * xi[1]);
            dN[a][1] = 0.25 * ss[a] * (1.0 + sr[a] * xi[0]);
            dN[a][2] = 0.0;
        }
    } else {
        const double sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
        const double ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
        const double st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        for (int a = 0; a < 8; ++a) {
            double fr = 1.0 + sr[a] * xi[0], fs = 1.0 + ss[a] * xi[1], ft = 1.0 + st[a] * xi[2];
            N[a] = 0.125 * fr * fs * ft;
            dN[a][0] = 0.125 * sr[a] * fs * ft;
            dN[a][1] = 0.125 * ss[a] * fr * ft;
            dN[a][2] = 0.125 * st[a] * fr * fs;
        }
    }
}

/* Jacobian J_ij = d x_j / d r_i, its determinant and the physical shape
 * derivatives dN_a/dx_j = sum_i Jinv_ji dN_a/dr_i (the B coefficients of
 * lin2DQuad4.cpp:688-710 / lin3DHexa8.cpp:811-853). */
double element_gp(const Model& m, int e, int q, double dNx[8][3], double N[8]) {
    const int nd = m.ndim, nen = m.nen;
    double xi[3], dN[8][3];
    gauss_point(nd, q, xi);
    shape_derivs(nd, xi, dN, N);
    double J[3][3] = {{0}};
    for (int a = 0; a < nen; ++a) {
        const double* x = &m.X[(size_t)m.conn[(size_t)e * nen + a] * nd];
        for (int i = 0; i < nd; ++i) for (int j = 0; j < nd; ++j) J[i][j] += dN[a][i] * x[j];
    }
    double det, Ji[3][3];
    if (nd == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
        Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
    } else {
        double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        Ji[0][0] = c00 / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][0] = c01 / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][0] = c02 / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    for (int a = 0; a < nen; ++a)
        for (int j = 0; j < nd; ++j) {
            double v = 0.0;
            for (int i = 0; i < nd; ++i) v += Ji[j][i] * dN[a][i];
            dNx[a][j] = v;
        }
    return det;
}

// Engineering strain B u at one Gauss point.
void strain_of(int nd, int nen, const double dNx[8][3], const double* ue, double* eps) {
    if (nd == 2) {
        double exx = 0, eyy = 0, gxy = 0;
        for (int a = 0; a < nen; ++a) {
            exx += dNx[a][0] * ue[2 * a];
            eyy += dNx[a][1] * ue[2 * a + 1];
            gxy += dNx[a][1] * ue[2 * a] + dNx[a][0] * ue[2 * a + 1];
        }
        eps[0] = exx; eps[1] = eyy; eps[2] = gxy;
    } else {
        double e[6] = {0, 0, 0, 0, 0, 0};
        for (int a = 0; a < nen; ++a) {
            const double* u = ue + 3 * a;
            e[0] += dNx[a][0] * u[0];
            e[1] += dNx[a][1] * u[1];
            e[2] += dNx[a][2] * u[2];
            e[3] += dNx[a][1] * u[0] + dNx[a][0] * u[1];
            e[4] += dNx[a][2] * u[1] + dNx[a][1] * u[2];
            e[5] += dNx[a][2] * u[0] + dNx[a][0] * u[2];
        }
        for (int i = 0; i < 6; ++i) eps[i] = e[i];
    }
}

// fe += c * B^T sig.
void add_BTsig(int nd, int nen, const double dNx[8][3], const double* sig, double c, double* fe) {
    if (nd == 2) {
        for (int a = 0; a < nen; ++a) {
            fe[2 * a]     += c * (dNx[a][0] * sig[0] + dNx[a][1] * sig[2]);
            fe[2 * a + 1] += c * (dNx[a][1] * sig[1] + dNx[a][0] * sig[2]);
        }
    } else {
        for (int a = 0; a < nen; ++a) {
            const double bx = dNx[a][0], by = dNx[a][1], bz = dNx[a][2];
            fe[3 * a]     += c * (bx * sig[0] + by * sig[3] + bz * sig[5]);
            fe[3 * a + 1] += c * (by * sig[1] + bx * sig[3] + bz * sig[4]);
            fe[3 * a + 2] += c * (bz * sig[2] + by * sig[4] + bx * sig[5]);
        }
    }
}

// B as an nstr x (nen*nd) dense matrix (for stiffness assembly).
void B_matrix(int nd, int nen, const double dNx[8][3], double* B) {
    const int nc = nen * nd;
    if (nd == 2) {
        for (int i = 0; i < 3 * nc; ++i) B[i] = 0.0;
        for (int a = 0; a < nen; ++a) {
            B[0 * nc + 2 * a] = dNx[a][0];
            B[1 * nc + 2 * a + 1] = dNx[a][1];
            B[2 * nc + 2 * a] = dNx[a][1]; B[2 * nc + 2 * a + 1] = dNx[a][0];
        }
    } else {
        for (int i = 0; i < 6 * nc; ++i) B[i] = 0.0;
        for (int a = 0; a < nen; ++a) {
            const double bx = dNx[a][0], by = dNx[a][1], bz = dNx[a][2];
            B[0 * nc + 3 * a] = bx; B[1 * nc + 3 * a + 1] = by; B[2 * nc + 3 * a + 2] = bz;
            B[3 * nc + 3 * a] = by; B[3 * nc + 3 * a + 1] = bx;
            B[4 * nc + 3 * a + 1] = bz; B[4 * nc + 3 * a + 2] = by;
            B[5 * nc + 3 * a] = bz; B[5 * nc + 3 * a + 2] = bx;
        }
    }
}

/* ---------------- the simulated mesh ------------------------------------- */

struct Sim {
    Model m; Loads L;
    std::vector<MatState> gp;          // [nelem][ngp]
    std::vector<int> edofs;            // [nelem][nen*ndof] total dofs
    // T (total <- free) as row lists: for every total dof the (free, factor) pairs.
    std::vector<int> Tptr, Tcol; std::vector<double> Tval;
    std::vector<int> smflag;
    double ftol = 1e-12, mtol = 1e-12, ktol = 1e-12;

    bool init(const svl_model_desc* d, const svl_load_desc* l) {
        if (!load_model(d, m)) return false;
        load_loads(l, L, m.nnode, m.ndim);
        const int nc = m.nen * m.ndof;
        edofs.resize((size_t)m.nelem * nc);
        for (int e = 0; e < m.nelem; ++e)
            for (int a = 0; a < m.nen; ++a)
                for (int j = 0; j < m.ndof; ++j)
                    edofs[(size_t)e * nc + a * m.ndof + j] = m.tdof[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndof + j];
        gp.resize((size_t)m.nelem * m.ngp);
        for (int e = 0; e < m.nelem; ++e)
            for (int q = 0; q < m.ngp; ++q)
                mat_init(gp[(size_t)e * m.ngp + q], m.mtype[m.emat[e]], &m.mpar[(size_t)m.emat[e] * SVL_MAT_NPARAM]);
        build_T();
        smflag.assign(m.ntotal, 0);
        for (int d0 : L.smdof) smflag[d0] = 1;
        return true;
    }

    // Mesh::GetTotalToFreeMatrix (Mesh.cpp:328-383): identity rows for free
    // dofs, factor rows for constrained dofs, zero rows for restrained ones.
    void build_T() {
        std::vector<std::vector<std::pair<int, double>>> rows(m.ntotal);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j) {
                int f = m.fdof_all[(size_t)n * m.dstride + j], t = m.tdof_all[(size_t)n * m.dstride + j];
                if (f > -1) rows[t].push_back({f, 1.0});
            }
        for (int c = 0; c < m.nconstraint; ++c)
            for (int i = m.cptr[c]; i < m.cptr[c + 1]; ++i)
                rows[m.cslave[c]].push_back({m.cmaster[i], m.cfactor[i]});
        Tptr.assign(m.ntotal + 1, 0);
        for (int t = 0; t < m.ntotal; ++t) {
            std::sort(rows[t].begin(), rows[t].end());
            // setFromTriplets sums duplicates
            std::vector<std::pair<int, double>> r;
            for (auto& p : rows[t]) { if (!r.empty() && r.back().first == p.first) r.back().second += p.second; else r.push_back(p); }
            for (auto& p : r) { Tcol.push_back(p.first); Tval.push_back(p.second); }
            Tptr[t + 1] = (int)Tcol.size();
        }
    }
    // x_total = T x_free
    void T_apply(const std::vector<double>& xf, std::vector<double>& xt) const {
        xt.assign(m.ntotal, 0.0);
        for (int t = 0; t < m.ntotal; ++t) {
            double s = 0.0;
            for (int i = Tptr[t]; i < Tptr[t + 1]; ++i) s += Tval[i] * xf[Tcol[i]];
            xt[t] = s;
        }
    }
    // y_free = T^T y_total, summed in ascending total-dof order.
    void TT_apply(const std::vector<double>& yt, std::vector<double>& yf) const {
        yf.assign(m.nfree, 0.0);
        for (int t = 0; t < m.ntotal; ++t)
            for (int i = Tptr[t]; i < Tptr[t + 1]; ++i) yf[Tcol[i]] += Tval[i] * yt[t];
    }

    const double* mp(int e) const { return &m.mpar[(size_t)m.emat[e] * SVL_MAT_NPARAM]; }
    int mt(int e) const { return m.mtype[m.emat[e]]; }

    // Element::ComputeInternalForces (lin2DQuad4.cpp:383-412, lin3DHexa8.cpp:383-412).
    void element_fint(int e, double* fe) const {
        const int nc = m.nen * m.ndof;
        for (int i = 0; i < nc; ++i) fe[i] = 0.0;
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            double det = element_gp(m, e, q, dNx, N);
            double sig[6];
            mat_stress(gp[(size_t)e * m.ngp + q], mt(e), mp(e), sig);
            double c = (m.ndim == 2) ? 1.0 * m.thick[e] * std::fabs(det) : 1.0 * std::fabs(det);
            add_BTsig(m.ndim, m.nen, dNx, sig, c, fe);
        }
    }
    // ELEMENT recorder values of element e (Recorder.cpp:272-323): 0 strain and
    // 1 total stress per Gauss point (Material::GetStrain / GetTotalStress:
    // elastic the engineering strain and C eps; J2 the material strain with
    // tensor shears, 2D components 1 2 4, PlasticPlaneStrainJ2.cpp:114-147),
    // 2 the internal force, 3 the strain rate (zeros for these materials).
    void element_response(int e, int response, double* out) const {
        const int ns = m.ndim == 2 ? 3 : 6;
        if (response == 2) { element_fint(e, out); return; }
        for (int q = 0; q < m.ngp; ++q) {
            const MatState& st = gp[(size_t)e * m.ngp + q];
            double* o = out + (size_t)q * ns;
            const int t = mt(e);
            if (response == 3) { for (int c = 0; c < ns; ++c) o[c] = 0.0; continue; }
            if (response == 1) { mat_stress(st, t, mp(e), o); continue; }
            if (t == SVL_MAT_PLASTICPLANESTRAINJ2) { o[0] = st.strain[1]; o[1] = st.strain[2]; o[2] = st.strain[4]; }
            else for (int c = 0; c < ns; ++c) o[c] = st.strain[c];
        }
    }
    // Element::UpdateState with strain B (U + dU) (lin2DQuad4.cpp:87-107, 618-633).
    void element_update(int e, const std::vector<double>& Ustrain) {
        const int nc = m.nen * m.ndof;
        double ue[24];
        for (int i = 0; i < nc; ++i) ue[i] = Ustrain[edofs[(size_t)e * nc + i]];
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            element_gp(m, e, q, dNx, N);
            double eps[6];
            strain_of(m.ndim, m.nen, dNx, ue, eps);
            mat_update(gp[(size_t)e * m.ngp + q], mt(e), mp(e), eps);
        }
    }
    void commit_all() { for (auto& s : gp) mat_commit(s); }

    // Element::ComputeStiffnessMatrix with the current tangent.
    void element_K(int e, double* Ke) const {
        const int nc = m.nen * m.ndof, ns = m.nstr;
        for (int i = 0; i < nc * nc; ++i) Ke[i] = 0.0;
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            double det = element_gp(m, e, q, dNx, N);
            double B[6 * 24], C[36], CB[6 * 24];
            B_matrix(m.ndim, m.nen, dNx, B);
            mat_tangent(gp[(size_t)e * m.ngp + q], mt(e), mp(e), C);
            double c = (m.ndim == 2) ? 1.0 * m.thick[e] * std::fabs(det) : 1.0 * std::fabs(det);
            for (int i = 0; i < ns; ++i)
                for (int j = 0; j < nc; ++j) {
                    double v = 0.0;
                    for (int k = 0; k < ns; ++k) v += C[i * ns + k] * B[k * nc + j];
                    CB[i * nc + j] = v;
                }
            for (int i = 0; i < nc; ++i)
                for (int j = 0; j < nc; ++j) {
                    double v = 0.0;
                    for (int k = 0; k < ns; ++k) v += B[k * nc + i] * CB[k * nc + j];
                    Ke[i * nc + j] += c * v;
                }
        }
    }
    // Element::ComputeInitialStiffnessMatrix (lin2DQuad4.cpp:714-739): B^T C0 B
    // with the material's initial tangent (J2: K 1(x)1 + 2G Id, PlasticPlaneStrainJ2.cpp:163-180).
    void element_K0(int e, double* Ke) const {
        const int nc = m.nen * m.ndof, ns = m.nstr;
        for (int i = 0; i < nc * nc; ++i) Ke[i] = 0.0;
        const int type = mt(e);
        const double* p = mp(e);
        double C[36];
        if (type == SVL_MAT_PLASTICPLANESTRAINJ2 || type == SVL_MAT_PLASTIC3DJ2) {
            double C6[36];
            j2_elastic_tangent(p[0], p[1], C6);
            if (type == SVL_MAT_PLASTICPLANESTRAINJ2) {
                const int ix[3] = {1, 2, 4};
                for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) C[i * 3 + j] = C6[ix[i] * 6 + ix[j]];
            } else std::memcpy(C, C6, sizeof(C6));
        } else {
            MatState z; mat_init(z, type, p);
            mat_tangent(z, type, p, C);
        }
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            double det = element_gp(m, e, q, dNx, N);
            double B[6 * 24], CB[6 * 24];
            B_matrix(m.ndim, m.nen, dNx, B);
            double c = (m.ndim == 2) ? 1.0 * m.thick[e] * std::fabs(det) : 1.0 * std::fabs(det);
            for (int i = 0; i < ns; ++i)
                for (int j = 0; j < nc; ++j) {
                    double v = 0.0;
                    for (int k = 0; k < ns; ++k) v += C[i * ns + k] * B[k * nc + j];
                    CB[i * nc + j] = v;
                }
            for (int i = 0; i < nc; ++i)
                for (int j = 0; j < nc; ++j) {
                    double v = 0.0;
                    for (int k = 0; k < ns; ++k) v += B[k * nc + i] * CB[k * nc + j];
                    Ke[i * nc + j] += c * v;
                }
        }
    }
    // Element::ComputeMassMatrix with row-sum lumping (lin2DQuad4.cpp:243-285).
    void element_M(int e, double* Me, bool lump) const {
        const int nc = m.nen * m.ndof, nd = m.ndim;
        for (int i = 0; i < nc * nc; ++i) Me[i] = 0.0;
        const double rho = mat_density(mt(e), mp(e));
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            double det = element_gp(m, e, q, dNx, N);
            double c = (nd == 2) ? 1.0 * rho * m.thick[e] * std::fabs(det) : 1.0 * rho * std::fabs(det);
            for (int a = 0; a < m.nen; ++a)
                for (int b = 0; b < m.nen; ++b)
                    for (int j = 0; j < nd; ++j) Me[(a * nd + j) * nc + (b * nd + j)] += c * (N[a] * N[b]);
        }
        if (lump)
            for (int i = 0; i < nc; ++i)
                for (int j = 0; j < nc; ++j)
                    if (i != j) { Me[i * nc + i] += Me[i * nc + j]; Me[i * nc + j] = 0.0; }
    }
    // Element body force rho int(H^T q) (lin2DQuad4.cpp:528-560).
    void element_body(int e, const double* qv, double* fe) const {
        const int nc = m.nen * m.ndof, nd = m.ndim;
        for (int i = 0; i < nc; ++i) fe[i] = 0.0;
        const double rho = mat_density(mt(e), mp(e));
        for (int q = 0; q < m.ngp; ++q) {
            double dNx[8][3], N[8];
            double det = element_gp(m, e, q, dNx, N);
            double c = (nd == 2) ? 1.0 * rho * m.thick[e] * std::fabs(det) : 1.0 * rho * std::fabs(det);
            for (int a = 0; a < m.nen; ++a)
                for (int j = 0; j < nd; ++j) fe[a * nd + j] += c * (N[a] * qv[j]);
        }
    }

    // Assembler::ComputeInternalForceVector (Assembler.cpp:240-269).
    void assemble_fint(std::vector<double>& F) const {
        F.assign(m.ntotal, 0.0);
        const int nc = m.nen * m.ndof;
        double fe[24];
        for (int e = 0; e < m.nelem; ++e) {
            element_fint(e, fe);
            for (int j = 0; j < nc; ++j)
                if (std::fabs(fe[j]) > ftol) F[edofs[(size_t)e * nc + j]] += fe[j];
        }
    }
    // Diagonal of the assembled lumped mass (Assembler.cpp:48-67, 623-697).
    void assemble_mass_diag(std::vector<double>& M) const {
        std::vector<double> Me_e(m.ntotal, 0.0), Mn(m.ntotal, 0.0);
        const int nc = m.nen * m.ndof;
        std::vector<double> Me((size_t)nc * nc);
        for (int e = 0; e < m.nelem; ++e) {
            element_M(e, Me.data(), true);
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    double v = Me[(size_t)i * nc + j];
                    if (std::fabs(v) > mtol && i == j) Me_e[edofs[(size_t)e * nc + i]] += v;
                }
        }
        if (!m.nodemass.empty())
            for (int t = 0; t < m.ntotal; ++t) if (std::fabs(m.nodemass[t]) > mtol) Mn[t] = m.nodemass[t];
        M.resize(m.ntotal);
        for (int t = 0; t < m.ntotal; ++t) M[t] = Me_e[t] + Mn[t];
    }
    // Assembler::ComputeExternalForceVector (Assembler.cpp:291-489), in the
    // pre-resolved (dof, series, coef) form.
    void fext(int k, std::vector<double>& F) const {
        F.assign(m.ntotal, 0.0);
        for (size_t i = 0; i < L.fdof.size(); ++i) F[L.fdof[i]] += L.fcoef[i] * L.series(L.fser[i], k);
        if (!L.drm_elem.empty()) drm_forces(k, F);
    }
    // lin2DQuad4::ComputeDomainReductionForces (lin2DQuad4.cpp:564-614,
    // lin3DHexa8.cpp:661-718): M~ Ao + C~ Vo + K~ Uo with the entries between
    // two dofs of equal boundary/exterior condition set to zero; motion rows past
    // the end of the signals read as zero (the reference reads them unchecked).
    void drm_forces(int k, std::vector<double>& F) const {
        const int nc = m.nen * m.ndof, nd = m.ndim;
        std::vector<double> Me((size_t)nc * nc), Ce((size_t)nc * nc, 0.0), Ke((size_t)nc * nc), K0((size_t)nc * nc);
        std::vector<double> Uo(nc), Vo(nc), Ao(nc), fe(nc);
        std::vector<int> cond(nc);
        for (size_t i = 0; i < L.drm_elem.size(); ++i) {
            const int e = L.drm_elem[i];
            for (int a = 0; a < m.nen; ++a) {
                const int n = m.conn[(size_t)e * m.nen + a];
                const int r = L.drm_row[n];
                const double sg = L.drm_ext[n] ? -1.0 : 1.0;
                for (int c = 0; c < nd; ++c) {
                    double u = 0, v = 0, acc = 0;
                    if (r >= 0 && k >= 0 && k < L.drm_nt) {
                        const double* row = &L.drm_motion[((size_t)r * L.drm_nt + k) * 3 * nd];
                        u = row[c]; v = row[nd + c]; acc = row[2 * nd + c];
                    }
                    Uo[a * nd + c] = sg * u; Vo[a * nd + c] = sg * v; Ao[a * nd + c] = sg * acc;
                    cond[a * nd + c] = L.drm_ext[n];
                }
            }
            element_M(e, Me.data(), m.lumped != 0);
            element_K(e, Ke.data());
            std::fill(Ce.begin(), Ce.end(), 0.0);
            if (!m.ray.empty()) {
                element_K0(e, K0.data());
                for (int j = 0; j < nc * nc; ++j) Ce[j] = m.ray[2 * e] * Me[j] + m.ray[2 * e + 1] * K0[j];
            }
            for (int r = 0; r < nc; ++r) {
                double v = 0.0;
                for (int c = 0; c < nc; ++c) {
                    if (cond[r] == cond[c]) continue;
                    const size_t ij = (size_t)r * nc + c;
                    v += Me[ij] * Ao[c] + Ce[ij] * Vo[c] + Ke[ij] * Uo[c];
                }
                fe[r] = v;
            }
            for (int r = 0; r < nc; ++r) F[edofs[(size_t)e * nc + r]] += L.drm_factor[i] * fe[r];
        }
    }
    // Assembler::ComputeSupportMotionIncrement (Assembler.cpp:493-532).
    // Reaction forces after a step (DynamicAnalysis::UpdateDomain,
    // DynamicAnalysis.cpp:128-150): Integrator::ComputeReactionForce =
    // ComputeDynamicInternalForceVector - Fext(k) - Fbar (CentralDifference.cpp:
    // 156-171, NewmarkBeta.cpp), the dynamic vector being the node inertia m A
    // (Assembler.cpp:569-592) and then, in element order, Fint_e + C_e V_e +
    // M_e A_e of every element with a fixed node (lin2DQuad4.cpp:416-434,
    // ZeroLength1D.cpp:257-277; Assembler.cpp:596-619, unfiltered).  A node is
    // fixed when one of its free-dof entries is -1 (Driver.hpp:338-341); the
    // other nodes report zeros (Node::GetReaction).  Element states are the
    // ones of the last update; C_e = am M_e + ak K0_e, dashpots eta a a^T.
    void reaction(int k, const std::vector<double>& V, const std::vector<double>& A, std::vector<double>& R) const {
        const int nt = m.ntotal, nen = m.nen, nc = nen * m.ndof;
        std::vector<char> fixed(m.nnode, 0), dof_fixed(nt, 0);
        for (int n = 0; n < m.nnode; ++n) {
            for (int j = 0; j < m.nndof[n]; ++j) if (m.fdof_all[(size_t)n * m.dstride + j] == -1) fixed[n] = 1;
            if (fixed[n]) for (int j = 0; j < m.nndof[n]; ++j) dof_fixed[m.tdof_all[(size_t)n * m.dstride + j]] = 1;
        }
        std::vector<double> F(nt, 0.0);
        if (!m.nodemass.empty()) for (int t = 0; t < nt; ++t) F[t] += m.nodemass[t] * A[t];
        std::vector<double> fe(72), Me((size_t)nc * nc), K0((size_t)nc * nc);
        for (int e = 0; e < m.nelem; ++e) {
            bool hf = false;
            for (int a = 0; a < nen; ++a) hf = hf || fixed[m.conn[(size_t)e * nen + a]];
            if (!hf) continue;
            element_fint(e, fe.data());
            element_M(e, Me.data(), m.lumped != 0);
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * e], ak = m.ray.empty() ? 0.0 : m.ray[2 * e + 1];
            if (ak != 0.0) element_K0(e, K0.data());
            const int* ed = &edofs[(size_t)e * nc];
            for (int i = 0; i < nc; ++i) {
                double cv = 0.0, ma = 0.0;
                for (int j = 0; j < nc; ++j) {
                    const double c = am * Me[(size_t)i * nc + j] + (ak != 0.0 ? ak * K0[(size_t)i * nc + j] : 0.0);
                    cv += c * V[ed[j]];
                    ma += Me[(size_t)i * nc + j] * A[ed[j]];
                }
                F[ed[i]] += (fe[i] + cv) + ma;
            }
        }
        std::vector<int> node_of(nt, -1);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j) node_of[m.tdof_all[(size_t)n * m.dstride + j]] = n;
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
            if (!fixed[node_of[a]] && !fixed[node_of[b]]) continue;
            const double eta = m.dp_eta[i];
            F[a] += eta * (V[a] - V[b]);
            F[b] += eta * (V[b] - V[a]);
        }
        std::vector<double> Fx;
        fext(k, Fx);
        R.assign(nt, 0.0);
        for (int t = 0; t < nt; ++t) if (dof_fixed[t]) R[t] = (F[t] - Fx[t]) - 0.0;
    }
    void support_increment(int k, std::vector<double>& SM) const {
        SM.assign(m.ntotal, 0.0);
        for (size_t i = 0; i < L.smdof.size(); ++i) {
            double g = L.support(L.smser[i], k);
            if (k > 0) g -= L.support(L.smser[i], k - 1);
            SM[L.smdof[i]] += L.smfac[i] * g;
        }
    }
};

/* ---------------- central difference (CentralDifference.cpp) ------------- */

struct CD {
    Sim s; double dt;
    std::vector<double> U, V, A, Up, Md, Kd, Kff_inv, Us;
    std::vector<double> Cd;    // damping diagonal (mass-proportional Rayleigh, dashpots), empty when undamped
    std::vector<int> dpa, dpb; std::vector<double> dpe;   // dashpot off-diagonal couplings C_ab = -eta
    bool fast = false;
    std::vector<double> geo;   // fast mode: [nelem][ngp][nen*ndim + 1]
    std::vector<double> fe_all;  // fast mode: element force blocks

    bool init(const svl_model_desc* d, const svl_load_desc* l, double dt_, double ftol, double mtol) {
        if (!s.init(d, l)) return false;
        if (!s.m.lumped || !s.m.epml.empty()) return false;
        dt = dt_; s.ftol = ftol; s.mtol = mtol;
        const int nt = s.m.ntotal;
        U.assign(nt, 0); V.assign(nt, 0); A.assign(nt, 0); Up.assign(nt, 0); Us.assign(nt, 0);
        s.assemble_mass_diag(Md);
        // C = sum_e am_e M_e + ak_e K0_e (lin2DQuad4.cpp:355-366); with a lumped
        // mass it is diagonal only when every ak_e is zero, which the diagonal
        // solve below needs
        if (!s.m.ray.empty()) {
            const int nc = s.m.nen * s.m.ndof;
            std::vector<double> Me((size_t)nc * nc);
            Cd.assign(nt, 0.0);
            for (int e = 0; e < s.m.nelem; ++e) {
                const double am = s.m.ray[2 * e], ak = s.m.ray[2 * e + 1];
                if (ak != 0.0) return false;
                if (am == 0.0) continue;
                s.element_M(e, Me.data(), true);
                for (int i = 0; i < nc; ++i) {
                    const double v = am * Me[(size_t)i * nc + i];
                    if (std::fabs(v) > s.ktol) Cd[s.edofs[(size_t)e * nc + i]] += v;
                }
            }
        }
        // dashpots: C_e = eta [1 -1; -1 1] (ZeroLength1D.cpp:210-228).  The
        // diagonal solve holds when no dashpot couples two free (or constrained) dofs
        for (size_t i = 0; i < s.m.dp_eta.size(); ++i) {
            const int a = s.m.dp_dof[2 * i], b = s.m.dp_dof[2 * i + 1];
            const double eta = s.m.dp_eta[i];
            if (!(std::fabs(eta) > s.ktol)) continue;
            const int na = s.Tptr[a + 1] - s.Tptr[a], nb = s.Tptr[b + 1] - s.Tptr[b];
            if (na > 0 && nb > 0) return false;
            if ((na > 0 && (na != 1 || s.Tval[s.Tptr[a]] != 1.0)) || (nb > 0 && (nb != 1 || s.Tval[s.Tptr[b]] != 1.0))) return false;
            if (Cd.empty()) Cd.assign(nt, 0.0);
            Cd[a] += eta; Cd[b] += eta;
            dpa.push_back(a); dpb.push_back(b); dpe.push_back(eta);
            dpa.push_back(b); dpb.push_back(a); dpe.push_back(eta);
        }
        // K = 1/dt/dt*M + 1/2/dt*C (CentralDifference.cpp:70)
        Kd.resize(nt);
        for (int t = 0; t < nt; ++t) Kd[t] = Cd.empty() ? 1.0 / dt / dt * Md[t] : 1.0 / dt / dt * Md[t] + 1.0 / 2.0 / dt * Cd[t];
        // Keff = T^T K T (diagonal when every slave has one master)
        std::vector<double> kf(s.m.nfree, 0.0);
        for (int t = 0; t < nt; ++t)
            for (int i = s.Tptr[t]; i < s.Tptr[t + 1]; ++i) kf[s.Tcol[i]] += s.Tval[i] * Kd[t] * s.Tval[i];
        Kff_inv.resize(s.m.nfree);
        for (int f = 0; f < s.m.nfree; ++f) Kff_inv[f] = 1.0 / kf[f];
        return true;
    }
    void set_initial(const double* U0, const double* V0, const double* A0) {
        for (int t = 0; t < s.m.ntotal; ++t) {
            U[t] = U0 ? U0[t] : 0.0; V[t] = V0 ? V0[t] : 0.0; A[t] = A0 ? A0[t] : 0.0;
            Up[t] = U[t] - dt * V[t] + dt * dt / 2.0 * A[t];
        }
    }
    void enable_fast() {
        const Model& m = s.m;
        const int per = m.nen * m.ndim + 1;
        geo.resize((size_t)m.nelem * m.ngp * per);
        for (int e = 0; e < m.nelem; ++e)
            for (int q = 0; q < m.ngp; ++q) {
                double dNx[8][3], N[8];
                double det = element_gp(m, e, q, dNx, N);
                double* g = &geo[((size_t)e * m.ngp + q) * per];
                for (int a = 0; a < m.nen; ++a) for (int j = 0; j < m.ndim; ++j) g[a * m.ndim + j] = dNx[a][j];
                g[per - 1] = (m.ndim == 2) ? 1.0 * m.thick[e] * std::fabs(det) : 1.0 * std::fabs(det);
            }
        fast = true;
    }
    // Fast internal force: precomputed geometry, elements in parallel, then a
    // serial element-order scatter so the sums match the faithful routine.
    void fint_fast(std::vector<double>& F) {
        const Model& m = s.m;
        const int nc = m.nen * m.ndof, per = m.nen * m.ndim + 1;
        fe_all.resize((size_t)m.nelem * nc);
        #pragma omp parallel for schedule(static)
        for (int e = 0; e < m.nelem; ++e) {
            double* fe = &fe_all[(size_t)e * nc];
            for (int i = 0; i < nc; ++i) fe[i] = 0.0;
            for (int q = 0; q < m.ngp; ++q) {
                const double* g = &geo[((size_t)e * m.ngp + q) * per];
                double dNx[8][3];
                for (int a = 0; a < m.nen; ++a) for (int j = 0; j < m.ndim; ++j) dNx[a][j] = g[a * m.ndim + j];
                double sig[6];
                mat_stress(s.gp[(size_t)e * m.ngp + q], s.mt(e), s.mp(e), sig);
                add_BTsig(m.ndim, m.nen, dNx, sig, g[per - 1], fe);
            }
        }
        F.assign(m.ntotal, 0.0);
        for (int e = 0; e < m.nelem; ++e)
            for (int j = 0; j < nc; ++j) {
                double v = fe_all[(size_t)e * nc + j];
                if (std::fabs(v) > s.ftol) F[s.edofs[(size_t)e * nc + j]] += v;
            }
    }
    void update_fast(const std::vector<double>& Ustr) {
        const Model& m = s.m;
        const int nc = m.nen * m.ndof, per = m.nen * m.ndim + 1;
        #pragma omp parallel for schedule(static)
        for (int e = 0; e < m.nelem; ++e) {
            double ue[24];
            for (int i = 0; i < nc; ++i) ue[i] = Ustr[s.edofs[(size_t)e * nc + i]];
            for (int q = 0; q < m.ngp; ++q) {
                const double* g = &geo[((size_t)e * m.ngp + q) * per];
                double dNx[8][3];
                for (int a = 0; a < m.nen; ++a) for (int j = 0; j < m.ndim; ++j) dNx[a][j] = g[a * m.ndim + j];
                double eps[6];
                strain_of(m.ndim, m.nen, dNx, ue, eps);
                mat_update(s.gp[(size_t)e * m.ngp + q], s.mt(e), s.mp(e), eps);
            }
        }
    }

    // One CentralDifference::ComputeNewStep(k) with Linear + diagonal solve,
    // followed by the CommitState of DynamicAnalysis::UpdateDomain.
    void step(int k) {
        const int nt = s.m.ntotal;
        std::vector<double> Fint, Fext, R(nt), Feff, SM, du, dUt;
        if (fast) fint_fast(Fint); else s.assemble_fint(Fint);
        s.fext(k, Fext);
        // Fext + Fbar - Fint + (1/dt/dt*M - 1/2/dt*C)*(U - Up)   (CentralDifference.cpp:217)
        for (int t = 0; t < nt; ++t) {
            const double c = Cd.empty() ? 1.0 / dt / dt * Md[t] : 1.0 / dt / dt * Md[t] - 1.0 / 2.0 / dt * Cd[t];
            R[t] = (Fext[t] + 0.0 - Fint[t]) + c * (U[t] - Up[t]);
        }
        for (size_t i = 0; i < dpa.size(); ++i)          // off-diagonal dashpot terms: -1/2/dt * (-eta)
            R[dpa[i]] += 1.0 / 2.0 / dt * dpe[i] * (U[dpb[i]] - Up[dpb[i]]);
        s.TT_apply(R, Feff);
        // support motion: Feff -= T^T (K SM)   (CentralDifference.cpp:190-202)
        s.support_increment(k, SM);
        {
            std::vector<double> KSM(nt), lg;
            for (int t = 0; t < nt; ++t) KSM[t] = Kd[t] * SM[t];
            for (size_t i = 0; i < dpa.size(); ++i) KSM[dpa[i]] -= 1.0 / 2.0 / dt * dpe[i] * SM[dpb[i]];
            s.TT_apply(KSM, lg);
            for (int f = 0; f < s.m.nfree; ++f) Feff[f] -= lg[f];
        }
        // diagonal LDL^T solve: x = (1/d) * b
        du.resize(s.m.nfree);
        for (int f = 0; f < s.m.nfree; ++f) du[f] = Kff_inv[f] * Feff[f];
        // Algorithm::UpdateStatesIncrements: strain from U + T du (no support motion)
        s.T_apply(du, dUt);
        for (int t = 0; t < nt; ++t) Us[t] = U[t] + dUt[t];
        if (fast) update_fast(Us); else for (int e = 0; e < s.m.nelem; ++e) s.element_update(e, Us);
        // CentralDifference::ComputeNewStep (CentralDifference.cpp:138-148)
        for (int t = 0; t < nt; ++t) {
            double dU = dUt[t] + SM[t];
            V[t] = 1.0 / 2.0 / dt * (U[t] + dU - Up[t]);
            A[t] = 1.0 / dt / dt * (dU - U[t] + Up[t]);
            Up[t] = U[t];
            U[t] += dU;
        }
        s.commit_all();
    }
};

/* ---------------- sparse matrices and solvers (Newmark) ------------------ */

struct CSR { int n = 0; std::vector<int> ptr, col; std::vector<double> val; };

// Triplets summed in insertion order per entry (setFromTriplets), free dofs only.
struct Trip { int r, c; double v; };
void csr_from_triplets(int n, std::vector<Trip>& tr, CSR& A) {
    std::stable_sort(tr.begin(), tr.end(), [](const Trip& a, const Trip& b) { return a.r < b.r || (a.r == b.r && a.c < b.c); });
    A.n = n; A.ptr.assign(n + 1, 0); A.col.clear(); A.val.clear();
    for (size_t i = 0; i < tr.size();) {
        size_t j = i; double v = 0.0;
        while (j < tr.size() && tr[j].r == tr[i].r && tr[j].c == tr[i].c) { v += tr[j].v; ++j; }
        A.col.push_back(tr[i].c); A.val.push_back(v); A.ptr[tr[i].r + 1]++;
        i = j;
    }
    for (int r = 0; r < n; ++r) A.ptr[r + 1] += A.ptr[r];
}

void csr_mv(const CSR& A, const std::vector<double>& x, std::vector<double>& y) {
    y.assign(A.n, 0.0);
    for (int r = 0; r < A.n; ++r) { double s = 0; for (int i = A.ptr[r]; i < A.ptr[r + 1]; ++i) s += A.val[i] * x[A.col[i]]; y[r] = s; }
}

// Dense LDL^T (small systems only; stands in for SimplicialLDLT).
bool dense_ldlt_solve(const CSR& A, const std::vector<double>& b, std::vector<double>& x) {
    const int n = A.n;
    std::vector<double> M((size_t)n * n, 0.0);
    for (int r = 0; r < n; ++r) for (int i = A.ptr[r]; i < A.ptr[r + 1]; ++i) M[(size_t)r * n + A.col[i]] = A.val[i];
    std::vector<double> D(n);
    for (int j = 0; j < n; ++j) {
        double d = M[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= M[(size_t)j * n + k] * M[(size_t)j * n + k] * D[k];
        if (d == 0.0 || !std::isfinite(d)) return false;
        D[j] = d;
        for (int i = j + 1; i < n; ++i) {
            double v = M[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) v -= M[(size_t)i * n + k] * M[(size_t)j * n + k] * D[k];
            M[(size_t)i * n + j] = v / d;
        }
    }
    x = b;
    for (int i = 0; i < n; ++i) for (int k = 0; k < i; ++k) x[i] -= M[(size_t)i * n + k] * x[k];
    for (int i = 0; i < n; ++i) x[i] = x[i] / D[i];
    for (int i = n - 1; i >= 0; --i) for (int k = i + 1; k < n; ++k) x[i] -= M[(size_t)k * n + i] * x[k];
    return true;
}

// Jacobi-preconditioned CG to a true relative residual tolerance.
int pcg_solve(const CSR& A, const std::vector<double>& b, std::vector<double>& x, double rtol, int maxit, int* iters) {
    const int n = A.n;
    std::vector<double> dinv(n, 1.0), r(n), z(n), p(n), q;
    for (int i = 0; i < n; ++i) for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) if (A.col[k] == i) dinv[i] = 1.0 / A.val[k];
    x.assign(n, 0.0);
    double bn = 0; for (double v : b) bn += v * v; bn = std::sqrt(bn);
    if (bn == 0.0) { if (iters) *iters = 0; return 0; }
    r = b;
    for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    p = z;
    double rz = 0; for (int i = 0; i < n; ++i) rz += r[i] * z[i];
    for (int it = 1; it <= maxit; ++it) {
        csr_mv(A, p, q);
        double pq = 0; for (int i = 0; i < n; ++i) pq += p[i] * q[i];
        if (!(pq > 0)) { if (iters) *iters = it; return SVL_ERR_BREAKDOWN; }
        double al = rz / pq;
        for (int i = 0; i < n; ++i) { x[i] += al * p[i]; r[i] -= al * q[i]; }
        double rn = 0; for (double v : r) rn += v * v;
        if (std::sqrt(rn) <= rtol * bn) {
            // confirm with the true residual
            std::vector<double> Ax; csr_mv(A, x, Ax);
            double tr = 0; for (int i = 0; i < n; ++i) { double d = b[i] - Ax[i]; tr += d * d; }
            if (std::sqrt(tr) <= rtol * bn) { if (iters) *iters = it; return 0; }
            for (int i = 0; i < n; ++i) r[i] = b[i] - Ax[i];
        }
        for (int i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
        double rz2 = 0; for (int i = 0; i < n; ++i) rz2 += r[i] * z[i];
        double be = rz2 / rz; rz = rz2;
        for (int i = 0; i < n; ++i) p[i] = z[i] + be * p[i];
    }
    if (iters) *iters = maxit;
    return SVL_ERR_MAXITER;
}

/* ---------------- Newmark (NewmarkBeta.cpp, beta=1/4, gamma=1/2) -------- */

/* Algorithm::ComputeConvergence (Algorithm.cpp:122-188).  The run entry
 * points encode the algorithm as algo 0 Linear, 1 Newton with test 5, 2
 * Newton with test 4, 10 + t Newton with test t (1..8). */
int newton_test(int algo) { return algo == 1 ? 5 : algo == 2 ? 4 : algo - 10; }
double convergence(int test, int it, const std::vector<double>& F, const std::vector<double>& dU,
                   const std::vector<double>& du, double& norm0) {
    auto nrm = [](const std::vector<double>& v) { double s2 = 0; for (double x : v) s2 += x * x; return std::sqrt(s2); };
    std::vector<double> en(du.size());
    for (size_t i = 0; i < du.size(); ++i) en[i] = du[i] * F[i];
    switch (test) {
    case 1: return nrm(F);
    case 2: return nrm(du);
    case 3: return nrm(en);
    case 4: if (it == 0) { norm0 = nrm(F); return norm0; } return nrm(F) / norm0;
    case 5: if (it == 0) { norm0 = nrm(dU); return nrm(du); } return nrm(du) / norm0;
    case 6: if (it == 0) { norm0 = nrm(en); return norm0; } return nrm(en) / norm0;
    case 7: return nrm(du) / nrm(dU);
    default: return -1.0;        // 8: maximum number of iterations
    }
}

struct Newmark {
    Sim s; double dt;
    std::vector<double> U, V, A, Mfull_diag;
    CSR Mt;                      // total-dof mass (lumped or consistent)
    CSR Ct;                      // total-dof Rayleigh damping (empty when undamped)
    int solver = 0;              // 0 dense LDL^T, 1 Jacobi-PCG
    double pcg_tol = 1e-12; int pcg_maxit = 100000; long pcg_iters = 0;

    bool init(const svl_model_desc* d, const svl_load_desc* l, double dt_) {
        if (!s.init(d, l)) return false;
        if (!s.m.epml.empty()) return false;       // PML: XNewmark
        dt = dt_;
        const int nt = s.m.ntotal;
        U.assign(nt, 0); V.assign(nt, 0); A.assign(nt, 0);
        // total mass matrix triplets in element order with the mass filter
        std::vector<Trip> tr;
        const int nc = s.m.nen * s.m.ndof;
        std::vector<double> Me((size_t)nc * nc);
        for (int e = 0; e < s.m.nelem; ++e) {
            s.element_M(e, Me.data(), s.m.lumped != 0);
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    double v = Me[(size_t)i * nc + j];
                    if (std::fabs(v) > s.mtol) tr.push_back({s.edofs[(size_t)e * nc + i], s.edofs[(size_t)e * nc + j], v});
                }
        }
        if (!s.m.nodemass.empty())
            for (int t = 0; t < nt; ++t) if (std::fabs(s.m.nodemass[t]) > s.mtol) tr.push_back({t, t, s.m.nodemass[t]});
        csr_from_triplets(nt, tr, Mt);
        // Rayleigh C_e = am M_e + ak K0_e (lin2DQuad4.cpp:355-366), assembled with
        // the stiffness tolerance (Assembler.cpp:117-158)
        if (!s.m.ray.empty()) {
            std::vector<Trip> ct;
            std::vector<double> K0((size_t)nc * nc);
            for (int e = 0; e < s.m.nelem; ++e) {
                const double am = s.m.ray[2 * e], ak = s.m.ray[2 * e + 1];
                if (am == 0.0 && ak == 0.0) continue;
                s.element_M(e, Me.data(), s.m.lumped != 0);
                s.element_K0(e, K0.data());
                for (int j = 0; j < nc; ++j)
                    for (int i = 0; i < nc; ++i) {
                        const double v = am * Me[(size_t)i * nc + j] + ak * K0[(size_t)i * nc + j];
                        if (std::fabs(v) > s.ktol) ct.push_back({s.edofs[(size_t)e * nc + i], s.edofs[(size_t)e * nc + j], v});
                    }
            }
            push_dashpots(ct);
            csr_from_triplets(nt, ct, Ct);
        } else if (!s.m.dp_eta.empty()) {
            std::vector<Trip> ct;
            push_dashpots(ct);
            csr_from_triplets(nt, ct, Ct);
        }
        return true;
    }
    // ZeroLength1D damping eta a a^T, a = (-1, +1) on its two dofs, column by column
    // with the stiffness tolerance (Assembler.cpp:117-158)
    void push_dashpots(std::vector<Trip>& ct) const {
        for (size_t i = 0; i < s.m.dp_eta.size(); ++i) {
            const int a = s.m.dp_dof[2 * i], b = s.m.dp_dof[2 * i + 1];
            const double eta = s.m.dp_eta[i];
            if (!(std::fabs(eta) > s.ktol)) continue;
            ct.push_back({a, a, eta}); ct.push_back({b, a, -eta});
            ct.push_back({a, b, -eta}); ct.push_back({b, b, eta});
        }
    }
    // T^T K T as free-dof CSR
    void reduce(const std::vector<Trip>& totalTr, CSR& Kff) const {
        std::vector<Trip> tr;
        for (const Trip& t : totalTr)
            for (int i = s.Tptr[t.r]; i < s.Tptr[t.r + 1]; ++i)
                for (int j = s.Tptr[t.c]; j < s.Tptr[t.c + 1]; ++j)
                    tr.push_back({s.Tcol[i], s.Tcol[j], s.Tval[i] * t.v * s.Tval[j]});
        csr_from_triplets(s.m.nfree, tr, Kff);
    }
    // Effective stiffness K + 4/dt^2 M (NewmarkBeta.cpp:224-235), C = 0.
    void keff(CSR& Kff) const {
        std::vector<Trip> tr;
        const int nc = s.m.nen * s.m.ndof;
        std::vector<double> Ke((size_t)nc * nc);
        for (int e = 0; e < s.m.nelem; ++e) {
            s.element_K(e, Ke.data());
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    double v = Ke[(size_t)i * nc + j];
                    if (std::fabs(v) > s.ktol) tr.push_back({s.edofs[(size_t)e * nc + i], s.edofs[(size_t)e * nc + j], v});
                }
        }
        for (int r = 0; r < Mt.n; ++r)
            for (int i = Mt.ptr[r]; i < Mt.ptr[r + 1]; ++i) tr.push_back({r, Mt.col[i], 4.0 / dt / dt * Mt.val[i]});
        for (int r = 0; r < Ct.n; ++r)
            for (int i = Ct.ptr[r]; i < Ct.ptr[r + 1]; ++i) tr.push_back({r, Ct.col[i], 2.0 / dt * Ct.val[i]});
        reduce(tr, Kff);
    }
    bool solve(const CSR& K, const std::vector<double>& b, std::vector<double>& x) {
        if (solver == 0) return dense_ldlt_solve(K, b, x);
        int it = 0;
        int st = pcg_solve(K, b, x, pcg_tol, pcg_maxit, &it);
        pcg_iters += it;
        return st == 0;
    }
    // One NewmarkBeta::ComputeNewStep with Linear (algo 0) or Newton (algo 1).
    int step(int k, int algo, int maxit, double cnvgtol) {
        const int nt = s.m.ntotal, nf = s.m.nfree;
        std::vector<double> dUf(nf, 0.0), du, dUt, Fint, Fext, SM, F(nt), Feff, MV, Us(nt);
        double norm0 = 0.0;
        int it = 0;
        for (;;) {
            s.T_apply(dUf, dUt);
            s.assemble_fint(Fint);
            s.fext(k, Fext);
            std::vector<double> w(nt);
            for (int t = 0; t < nt; ++t) w[t] = 4.0 / dt * V[t] + A[t] - 4.0 / dt / dt * dUt[t];
            csr_mv(Mt, w, MV);
            // Fext + Fbar - Fint + M*(4/dt V + A - 4/dt^2 dU) + C*(V - 2/dt dU) (NewmarkBeta.cpp:215)
            for (int t = 0; t < nt; ++t) F[t] = (Fext[t] + 0.0 - Fint[t]) + MV[t];
            if (Ct.n) {
                std::vector<double> w2(nt), CV;
                for (int t = 0; t < nt; ++t) w2[t] = V[t] - 2.0 / dt * dUt[t];
                csr_mv(Ct, w2, CV);
                for (int t = 0; t < nt; ++t) F[t] += CV[t];
            }
            s.TT_apply(F, Feff);
            CSR K; keff(K);
            // support motion term: Feff -= T^T (K_total SM).  K_total SM needs
            // the total stiffness; restrained rows only couple through K.
            // NewmarkBeta takes the increment of step k-1 (NewmarkBeta.cpp:186),
            // unlike CentralDifference (CentralDifference.cpp:196).
            s.support_increment(k - 1, SM);
            bool anySM = false; for (double v : SM) if (v != 0.0) { anySM = true; break; }
            if (anySM) {
                std::vector<Trip> tr; const int nc = s.m.nen * s.m.ndof;
                std::vector<double> Ke((size_t)nc * nc);
                for (int e = 0; e < s.m.nelem; ++e) {
                    s.element_K(e, Ke.data());
                    for (int j = 0; j < nc; ++j) for (int i = 0; i < nc; ++i) {
                        double v = Ke[(size_t)i * nc + j];
                        if (std::fabs(v) > s.ktol) tr.push_back({s.edofs[(size_t)e * nc + i], s.edofs[(size_t)e * nc + j], v});
                    }
                }
                for (int r = 0; r < Mt.n; ++r) for (int i = Mt.ptr[r]; i < Mt.ptr[r + 1]; ++i) tr.push_back({r, Mt.col[i], 4.0 / dt / dt * Mt.val[i]});
                for (int r = 0; r < Ct.n; ++r) for (int i = Ct.ptr[r]; i < Ct.ptr[r + 1]; ++i) tr.push_back({r, Ct.col[i], 2.0 / dt * Ct.val[i]});
                CSR Kt; csr_from_triplets(nt, tr, Kt);
                std::vector<double> KS, lg; csr_mv(Kt, SM, KS); s.TT_apply(KS, lg);
                for (int f = 0; f < nf; ++f) Feff[f] -= lg[f];
            }
            if (!solve(K, Feff, du)) return SVL_ERR_BREAKDOWN;
            for (int f = 0; f < nf; ++f) dUf[f] += du[f];
            // convergence on the effective force this iteration solved for
            const double res = algo == 0 ? 0.0 : convergence(newton_test(algo), it, Feff, dUf, du, norm0);
            s.T_apply(dUf, dUt);
            for (int t = 0; t < nt; ++t) Us[t] = U[t] + dUt[t];
            for (int e = 0; e < s.m.nelem; ++e) s.element_update(e, Us);
            ++it;
            if (algo == 0 || !(res > cnvgtol) || it >= maxit) {
                // NewmarkBeta::ComputeNewStep (NewmarkBeta.cpp:130-139)
                for (int t = 0; t < nt; ++t) {
                    double d = dUt[t];
                    U[t] += (d + SM[t]);
                    A[t] = 4.0 / dt / dt * d - 4.0 / dt * V[t] - A[t];
                    V[t] = 2.0 / dt * d - V[t];
                }
                s.commit_all();
                last_iters = it;
                return 0;
            }
        }
    }
    int last_iters = 0;
};

/* ---------------- PML elements (PML2DQuad4, PML3DHexa8) ------------------ */

/* Stretching factors at a point (PML2DQuad4.cpp:655-693,
 * PML3DHexa8.cpp:952-996): a_i = 1 + a0 ((x_i - x0_i) n_i / L)^m,
 * b_i = b0 (...)^m, a0 = (m+1) (L/10) / (2L) ln(1/R), b0 = (m+1) Vp / (2L) ln(1/R). */
void pml_stretch(int nd, const double* x, const double* par, double rho, double mu, double lambda, double* a, double* b) {
    const double m = par[0], L = par[1], R = par[2];
    const double* x0 = par + 3;
    const double* n = par + 3 + nd;
    const double Vp = std::sqrt((lambda + 2.0 * mu) / rho);
    const double bpml = L / 10.0;
    const double a0 = (m + 1.0) * bpml / 2.0 / L * std::log(1.0 / R);
    const double b0 = (m + 1.0) * Vp / 2.0 / L * std::log(1.0 / R);
    for (int i = 0; i < nd; ++i) {
        const double r = std::pow((x[i] - x0[i]) * n[i] / L, m);
        a[i] = 1.0 + a0 * r;
        b[i] = b0 * r;
    }
}

/* Element matrices of PML2DQuad4 (5 dofs/node: ux uy s11 s22 s12;
 * PML2DQuad4.cpp:233-470) and PML3DHexa8 (9 dofs/node: ux uy uz s11 s22 s33
 * s12 s23 s13; PML3DHexa8.cpp:214-712), row-major nc x nc.  Each matrix is a
 * scalar s times the displacement block rho N N and the stress-compliance
 * block, plus (not for M) the displacement-stress coupling dN_j N_k q_d for
 * derivative direction d:
 *   3D  M: s = ax ay az,                          q = 0
 *       C: s = ax ay bz + ax by az + bx ay az,    q = (ay az, ax az, ax ay)
 *       K: s = ax by bz + bx by az + bx ay bz,    q = (ay bz + az by, ax bz + az bx, ax by + ay bx)
 *       G: s = bx by bz,                          q = (by bz, bx bz, bx by)
 *   2D  M: s = ax ay, C: s = ax by + ay bx, q = (ay, ax); K: s = bx by, q = (by, bx); G empty.
 * Same Gauss points and accumulation order as the lin elements; mu =
 * E / 2 / (1 + nu) and lambda = E nu / (1 + nu) / (1 - 2 nu) as in the
 * reference.  par: m, L, R, x0[nd], n[nd]. */
void pml_matrices(int nd, const double* X, double E, double nu, double rho, double t, const double* par,
                  double* Mo, double* Co, double* Ko, double* Go) {
    const int nen = nd == 2 ? 4 : 8, nn = nd == 2 ? 5 : 9, nc = nen * nn, ngp = nen;
    double* out[4] = {Mo, Co, Ko, Go};
    for (double* o : out) if (o) std::fill(o, o + (size_t)nc * nc, 0.0);
    const double mu = E / 2.0 / (1 + nu);
    const double lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    for (int q = 0; q < ngp; ++q) {
        double xi[3], dN[8][3], N[8];
        gauss_point(nd, q, xi);
        shape_derivs(nd, xi, dN, N);
        double J[3][3] = {{0}}, xg[3] = {0, 0, 0};
        for (int a = 0; a < nen; ++a)
            for (int i = 0; i < nd; ++i) {
                xg[i] += N[a] * X[a * nd + i];
                for (int j = 0; j < nd; ++j) J[i][j] += dN[a][i] * X[a * nd + j];
            }
        double det, Ji[3][3];
        if (nd == 2) {
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
            Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
        } else {
            const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            Ji[0][0] = c00 / det;
            Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
            Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
            Ji[1][0] = c01 / det;
            Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
            Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
            Ji[2][0] = c02 / det;
            Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
            Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        }
        double dx[8][3];
        for (int a = 0; a < nen; ++a)
            for (int j = 0; j < nd; ++j) {
                double v = 0.0;
                for (int i = 0; i < nd; ++i) v += Ji[j][i] * dN[a][i];
                dx[a][j] = v;
            }
        const double D = std::fabs(det);
        const double f = nd == 2 ? t * 1.0 * D : 1.0 * D;
        double a[3] = {1, 1, 1}, b[3] = {0, 0, 0};
        pml_stretch(nd, xg, par, rho, mu, lambda, a, b);
        double sc[4], qd[4][3];
        if (nd == 2) {
            sc[0] = a[0] * a[1];                 qd[0][0] = 0.0;  qd[0][1] = 0.0;
            sc[1] = a[0] * b[1] + a[1] * b[0];   qd[1][0] = a[1]; qd[1][1] = a[0];
            sc[2] = b[0] * b[1];                 qd[2][0] = b[1]; qd[2][1] = b[0];
            sc[3] = 0.0;                         qd[3][0] = 0.0;  qd[3][1] = 0.0;
        } else {
            sc[0] = a[0] * a[1] * a[2];
            sc[1] = a[0] * a[1] * b[2] + a[0] * b[1] * a[2] + b[0] * a[1] * a[2];
            sc[2] = a[0] * b[1] * b[2] + b[0] * b[1] * a[2] + b[0] * a[1] * b[2];
            sc[3] = b[0] * b[1] * b[2];
            qd[0][0] = qd[0][1] = qd[0][2] = 0.0;
            qd[1][0] = a[1] * a[2]; qd[1][1] = a[0] * a[2]; qd[1][2] = a[0] * a[1];
            qd[2][0] = a[1] * b[2] + a[2] * b[1]; qd[2][1] = a[0] * b[2] + a[2] * b[0]; qd[2][2] = a[0] * b[1] + a[1] * b[0];
            qd[3][0] = b[1] * b[2]; qd[3][1] = b[0] * b[2]; qd[3][2] = b[0] * b[1];
        }
        for (int mi = 0; mi < 4; ++mi) {
            double* Mx = out[mi];
            if (!Mx || (nd == 2 && mi == 3)) continue;
            const double s = sc[mi];
            auto at = [&](int r, int c) -> double& { return Mx[(size_t)r * nc + c]; };
            for (int j = 0; j < nen; ++j)
                for (int k = 0; k < nen; ++k) {
                    const double NN = N[j] * N[k] * f;
                    if (nd == 2) {
                        const int r = 5 * j, c = 5 * k;
                        at(r, c) += rho * s * NN;
                        at(r + 1, c + 1) += rho * s * NN;
                        at(r + 2, c + 2) += -s * (lambda + 2.0 * mu) / 4.0 / mu / (lambda + mu) * NN;
                        at(r + 3, c + 3) += -s * (lambda + 2.0 * mu) / 4.0 / mu / (lambda + mu) * NN;
                        at(r + 4, c + 4) += -s / mu * NN;
                        at(r + 2, c + 3) += s * lambda / 4.0 / mu / (lambda + mu) * NN;
                        at(r + 3, c + 2) += s * lambda / 4.0 / mu / (lambda + mu) * NN;
                        if (mi == 0) continue;
                        const double qx = qd[mi][0], qy = qd[mi][1];
                        at(r, c + 2) += qx * dx[j][0] * N[k] * f;
                        at(r + 2, c) += qx * dx[k][0] * N[j] * f;
                        at(r, c + 4) += qy * dx[j][1] * N[k] * f;
                        at(r + 4, c) += qy * dx[k][1] * N[j] * f;
                        at(r + 1, c + 3) += qy * dx[j][1] * N[k] * f;
                        at(r + 3, c + 1) += qy * dx[k][1] * N[j] * f;
                        at(r + 1, c + 4) += qx * dx[j][0] * N[k] * f;
                        at(r + 4, c + 1) += qx * dx[k][0] * N[j] * f;
                    } else {
                        const int r = 9 * j, c = 9 * k;
                        const double kap = s * (lambda + mu) / mu / (3.0 * lambda + 2.0 * mu);
                        const double lam = s * lambda / 2.0 / mu / (3.0 * lambda + 2.0 * mu);
                        for (int d = 0; d < 3; ++d) at(r + d, c + d) += rho * s * NN;
                        for (int d = 3; d < 6; ++d) at(r + d, c + d) += -kap * NN;
                        for (int d = 6; d < 9; ++d) at(r + d, c + d) += -s / mu * NN;
                        at(r + 3, c + 4) += lam * NN; at(r + 3, c + 5) += lam * NN; at(r + 4, c + 5) += lam * NN;
                        at(r + 4, c + 3) += lam * NN; at(r + 5, c + 3) += lam * NN; at(r + 5, c + 4) += lam * NN;
                        if (mi == 0) continue;
                        const double qx = qd[mi][0], qy = qd[mi][1], qz = qd[mi][2];
                        // displacement rows x stress columns and the transposes
                        const struct { int u, sg, dir; } cp[9] = {{0, 3, 0}, {0, 6, 1}, {0, 8, 2}, {1, 4, 1}, {1, 6, 0},
                                                                  {1, 7, 2}, {2, 5, 2}, {2, 8, 0}, {2, 7, 1}};
                        for (const auto& e : cp) {
                            const double qv = e.dir == 0 ? qx : (e.dir == 1 ? qy : qz);
                            at(r + e.u, c + e.sg) += dx[j][e.dir] * N[k] * qv * f;
                            at(r + e.sg, c + e.u) += dx[k][e.dir] * N[j] * qv * f;
                        }
                    }
                }
        }
    }
}

}  // namespace

/* ---------------- ExtendedNewmarkBeta with PML (ExtendedNewmarkBeta.cpp) -- */

/* ExtendedNewmarkBeta::ComputeNewStep with the Linear or NewtonRaphson
 * algorithm on a mesh of elastic or J2 solid elements (lin2DQuad4/lin3DHexa8,
 * first ndim dofs of their nodes) and PML elements (PML2DQuad4/PML3DHexa8,
 * every dof of their nodes):
 *   M, C, K, G assembled once (ExtendedNewmarkBeta.cpp:64-70, Assembler.cpp
 *   48-205) in element-tag order, M with the mass tolerance, C, K, G with the
 *   stiffness tolerance; PML mass consistent (PML3DHexa8.cpp:214-284, the 2D
 *   lumping is a TODO in PML2DQuad4.cpp:286-289); solid C Rayleigh, PML C its own;
 *   Feff = Fext - Fint - G (Ubar + dt U + dt^2/6 V) + C V + M (4/dt V + A)  (:208-229)
 *   Keff = K + 4/dt^2 M + 2/dt C + dt/3 G                                   (:233-245)
 *   Feff -= T^T Keff SM(k)                                                  (:190-204)
 *   dU = T du; Ubar += dt U + dt/3 (dU + SM) + dt^2/6 V; U += dU + SM;
 *   A = 4/dt^2 dU - 4/dt V - A; V = 2/dt dU - V                             (:123-153)
 * Fint: solid elements from their material state (strain of U + T du of the
 * last step), PML elements K_e U_e with U the displacement after the last
 * step (PML3DHexa8.cpp:716-742 with zero node increments after UpdateDomain).
 * With J2 elements K is re-assembled with their current tangents at every
 * iteration (Rayleigh C keeps the initial stiffness). */
// CentralDifference with a non-diagonal K = 1/dt/dt*M + 1/2/dt*C
// (CentralDifference.cpp:64-151, K at :70): a consistent mass (massform
// Consistent, lin2DQuad4.cpp:243-285 / lin3DHexa8.cpp:243-285 without the
// lumping branch) or stiffness-proportional Rayleigh damping.  M and C are
// assembled in element order with the tolerance filters, T^T K T is factorised
// once (dense LDL^T: SimplicialLDLT with its factor-once flag,
// EigenSolver.cpp:19-59) and every step solves it for
// T^T [Fext(k) - Fint + (1/dt/dt*M - 1/2/dt*C)(U - Up)] (:206-221); support
// motion adds -T^T K SM (:190-202).
struct CDGen {
    Sim s; double dt = 0;
    std::vector<double> U, V, A, Up, Us;
    CSR Mt, Ct;
    int nf = 0;
    std::vector<double> L, D;            // T^T K T = L D L^T, L unit lower [nf][nf]

    static bool needed(const Model& m) {
        if (!m.lumped) return true;
        for (size_t e = 0; e < m.ray.size() / 2; ++e) if (m.ray[2 * e + 1] != 0.0) return true;
        return false;
    }
    bool init(const svl_model_desc* d, const svl_load_desc* l, double dt_, double ftol, double mtol) {
        if (!s.init(d, l)) return false;
        if (!s.m.epml.empty()) return false;
        dt = dt_; s.ftol = ftol; s.mtol = mtol;
        const Model& m = s.m;
        const int nt = m.ntotal, nc = m.nen * m.ndof;
        U.assign(nt, 0); V.assign(nt, 0); A.assign(nt, 0); Up.assign(nt, 0); Us.assign(nt, 0);
        std::vector<Trip> tm, tc;
        std::vector<double> Me((size_t)nc * nc), K0((size_t)nc * nc);
        for (int e = 0; e < m.nelem; ++e) {
            s.element_M(e, Me.data(), m.lumped != 0);
            const int* ed = &s.edofs[(size_t)e * nc];
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    const double v = Me[(size_t)i * nc + j];
                    if (std::fabs(v) > s.mtol) tm.push_back({ed[i], ed[j], v});
                }
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * e], ak = m.ray.empty() ? 0.0 : m.ray[2 * e + 1];
            if (am == 0.0 && ak == 0.0) continue;
            if (ak != 0.0) s.element_K0(e, K0.data());
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    const double v = am * Me[(size_t)i * nc + j] + (ak != 0.0 ? ak * K0[(size_t)i * nc + j] : 0.0);
                    if (std::fabs(v) > s.ktol) tc.push_back({ed[i], ed[j], v});
                }
        }
        if (!m.nodemass.empty())
            for (int t = 0; t < nt; ++t) if (std::fabs(m.nodemass[t]) > s.mtol) tm.push_back({t, t, m.nodemass[t]});
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
            const double eta = m.dp_eta[i];
            if (!(std::fabs(eta) > s.ktol)) continue;
            tc.push_back({a, a, eta}); tc.push_back({b, a, -eta}); tc.push_back({a, b, -eta}); tc.push_back({b, b, eta});
        }
        csr_from_triplets(nt, tm, Mt);
        csr_from_triplets(nt, tc, Ct);
        // dense T^T K T and its factorisation
        nf = m.nfree;
        L.assign((size_t)nf * nf, 0.0);
        auto addK = [&](const CSR& Mx, double c) {
            for (int r = 0; r < nt; ++r)
                for (int p = Mx.ptr[r]; p < Mx.ptr[r + 1]; ++p) {
                    const int col = Mx.col[p];
                    const double v = c * Mx.val[p];
                    for (int i = s.Tptr[r]; i < s.Tptr[r + 1]; ++i)
                        for (int j = s.Tptr[col]; j < s.Tptr[col + 1]; ++j)
                            L[(size_t)s.Tcol[i] * nf + s.Tcol[j]] += s.Tval[i] * v * s.Tval[j];
                }
        };
        addK(Mt, 1.0 / dt / dt);
        addK(Ct, 1.0 / 2.0 / dt);
        D.assign(nf, 0.0);
        for (int j = 0; j < nf; ++j) {
            double dj = L[(size_t)j * nf + j];
            for (int k = 0; k < j; ++k) dj -= L[(size_t)j * nf + k] * L[(size_t)j * nf + k] * D[k];
            if (!(dj > 0.0) || !std::isfinite(dj)) return false;
            D[j] = dj;
            for (int i = j + 1; i < nf; ++i) {
                double v = L[(size_t)i * nf + j];
                for (int k = 0; k < j; ++k) v -= L[(size_t)i * nf + k] * L[(size_t)j * nf + k] * D[k];
                L[(size_t)i * nf + j] = v / dj;
            }
        }
        return true;
    }
    void set_initial(const double* U0, const double* V0, const double* A0) {
        for (int t = 0; t < s.m.ntotal; ++t) {
            U[t] = U0 ? U0[t] : 0.0; V[t] = V0 ? V0[t] : 0.0; A[t] = A0 ? A0[t] : 0.0;
            Up[t] = U[t] - dt * V[t] + dt * dt / 2.0 * A[t];
        }
    }
    void step(int k) {
        const int nt = s.m.ntotal;
        std::vector<double> Fint, Fext, w(nt), Mw, Cw, R(nt), Feff, SM, Ksm(nt), MS, CS, lg, dUt;
        s.assemble_fint(Fint);
        s.fext(k, Fext);
        for (int t = 0; t < nt; ++t) w[t] = U[t] - Up[t];
        csr_mv(Mt, w, Mw);
        csr_mv(Ct, w, Cw);
        for (int t = 0; t < nt; ++t) R[t] = (Fext[t] + 0.0 - Fint[t]) + (1.0 / dt / dt * Mw[t] - 1.0 / 2.0 / dt * Cw[t]);
        s.TT_apply(R, Feff);
        s.support_increment(k, SM);
        csr_mv(Mt, SM, MS);
        csr_mv(Ct, SM, CS);
        for (int t = 0; t < nt; ++t) Ksm[t] = 1.0 / dt / dt * MS[t] + 1.0 / 2.0 / dt * CS[t];
        s.TT_apply(Ksm, lg);
        for (int f = 0; f < nf; ++f) Feff[f] -= lg[f];
        // L D L^T du = Feff
        std::vector<double> du(Feff);
        for (int i = 0; i < nf; ++i) for (int k2 = 0; k2 < i; ++k2) du[i] -= L[(size_t)i * nf + k2] * du[k2];
        for (int i = 0; i < nf; ++i) du[i] /= D[i];
        for (int i = nf - 1; i >= 0; --i) for (int k2 = i + 1; k2 < nf; ++k2) du[i] -= L[(size_t)k2 * nf + i] * du[k2];
        s.T_apply(du, dUt);
        for (int t = 0; t < nt; ++t) Us[t] = U[t] + dUt[t];
        for (int e = 0; e < s.m.nelem; ++e) s.element_update(e, Us);
        for (int t = 0; t < nt; ++t) {
            const double dU = dUt[t] + SM[t];
            V[t] = 1.0 / 2.0 / dt * (U[t] + dU - Up[t]);
            A[t] = 1.0 / dt / dt * (dU - U[t] + Up[t]);
            Up[t] = U[t];
            U[t] += dU;
        }
        s.commit_all();
    }
};

struct XNewmark {
    Sim s; double dt;
    std::vector<double> U, V, A, Ubar;
    CSR Kt, Mt, Ct, Gt;                      // Kt: initial K (re-assembled per iteration with J2 tangents)
    std::vector<std::vector<int>> edof;      // per element: solid nen*ndim, PML nen*(5|9)
    int solver = 0; double pcg_tol = 1e-12;
    bool nonlinear = false;                  // J2 solid elements present
    bool newmark = false;                    // NewmarkBeta's force, stiffness and update
    int last_iters = 0;
    double last_res = 0.0;

    bool pml(int e) const { return !s.m.epml.empty() && s.m.epml[e]; }
    void pml_elem(int e, double* Me, double* Ce, double* Ke, double* Ge) const {
        const Model& m = s.m;
        double X[8 * 3];
        for (int a = 0; a < m.nen; ++a)
            for (int i = 0; i < m.ndim; ++i) X[a * m.ndim + i] = m.X[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndim + i];
        const double* p = s.mp(e);
        pml_matrices(m.ndim, X, p[0], p[1], p[2], m.ndim == 2 ? m.thick[e] : 1.0,
                     &m.pml_par[(size_t)e * (3 + 2 * m.ndim)], Me, Ce, Ke, Ge);
    }
    bool init(const svl_model_desc* d, const svl_load_desc* l, double dt_) {
        if (!s.init(d, l)) return false;
        dt = dt_;
        const Model& m = s.m;
        // PML elements take the elastic constants of their material; solid
        // elements may be elastic or J2
        for (int e = 0; e < m.nelem; ++e) {
            const int t = s.mt(e);
            const bool el = t == SVL_MAT_ELASTIC2DPLANESTRAIN || t == SVL_MAT_ELASTIC3DLINEAR;
            if (!el && pml(e)) return false;
            if (!el) nonlinear = true;
        }
        const int nt = m.ntotal, pnd = m.ndim == 2 ? 5 : 9;
        U.assign(nt, 0); V.assign(nt, 0); A.assign(nt, 0); Ubar.assign(nt, 0);
        edof.resize(m.nelem);
        for (int e = 0; e < m.nelem; ++e) {
            const int k = pml(e) ? pnd : m.ndim;
            for (int a = 0; a < m.nen; ++a) {
                const int n = m.conn[(size_t)e * m.nen + a];
                if (k > m.nndof[n]) return false;
                for (int j = 0; j < k; ++j) edof[e].push_back(m.tdof_all[(size_t)n * m.dstride + j]);
            }
        }
        std::vector<Trip> tk, tm, tc, tg;
        const int ncmax = m.nen * pnd;
        std::vector<double> Me((size_t)ncmax * ncmax), Ce(Me.size()), Ke(Me.size()), Ge(Me.size()), K0(Me.size());
        auto push = [&](std::vector<Trip>& tr, int e, const double* A_, double tol) {
            const int nc = (int)edof[e].size();
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    const double v = A_[(size_t)i * nc + j];
                    if (std::fabs(v) > tol) tr.push_back({edof[e][i], edof[e][j], v});
                }
        };
        for (int e = 0; e < m.nelem; ++e) {
            const int nc = (int)edof[e].size();
            if (pml(e)) {
                pml_elem(e, Me.data(), Ce.data(), Ke.data(), Ge.data());
                push(tm, e, Me.data(), s.mtol);
                push(tc, e, Ce.data(), s.ktol);
                push(tk, e, Ke.data(), s.ktol);
                if (m.ndim == 3) push(tg, e, Ge.data(), s.ktol);     // PML2DQuad4 has no history matrix
            } else {
                s.element_M(e, Me.data(), m.lumped != 0);
                s.element_K(e, Ke.data());
                push(tm, e, Me.data(), s.mtol);
                push(tk, e, Ke.data(), s.ktol);
                if (!m.ray.empty()) {
                    const double am = m.ray[2 * e], ak = m.ray[2 * e + 1];
                    s.element_K0(e, K0.data());
                    for (int i = 0; i < nc * nc; ++i) Ce[i] = am * Me[i] + ak * K0[i];
                    push(tc, e, Ce.data(), s.ktol);
                }
            }
        }
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {       // ZeroLength1D dashpots
            const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
            const double eta = m.dp_eta[i];
            if (!(std::fabs(eta) > s.ktol)) continue;
            tc.push_back({a, a, eta}); tc.push_back({b, a, -eta}); tc.push_back({a, b, -eta}); tc.push_back({b, b, eta});
        }
        if (!m.nodemass.empty())
            for (int t = 0; t < nt; ++t) if (std::fabs(m.nodemass[t]) > s.mtol) tm.push_back({t, t, m.nodemass[t]});
        csr_from_triplets(nt, tk, Kt); csr_from_triplets(nt, tm, Mt);
        csr_from_triplets(nt, tc, Ct); csr_from_triplets(nt, tg, Gt);
        return true;
    }
    void set_initial(const double* U0, const double* V0, const double* A0, const double* Ub0) {
        const int nt = s.m.ntotal;
        for (int t = 0; t < nt; ++t) {
            U[t] = U0 ? U0[t] : 0.0; V[t] = V0 ? V0[t] : 0.0; A[t] = A0 ? A0[t] : 0.0; Ubar[t] = Ub0 ? Ub0[t] : 0.0;
        }
        // solid element states from the initial displacement
        for (int e = 0; e < s.m.nelem; ++e) if (!pml(e)) s.element_update(e, U);
        s.commit_all();
    }
    // K with the solid elements' current tangents, in element order
    void assemble_K(CSR& K) const {
        const Model& m = s.m;
        std::vector<Trip> tk;
        std::vector<double> Ke(72 * 72);
        for (int e = 0; e < m.nelem; ++e) {
            const int nc = (int)edof[e].size();
            if (pml(e)) pml_elem(e, nullptr, nullptr, Ke.data(), nullptr);
            else s.element_K(e, Ke.data());
            for (int j = 0; j < nc; ++j)
                for (int i = 0; i < nc; ++i) {
                    const double v = Ke[(size_t)i * nc + j];
                    if (std::fabs(v) > s.ktol) tk.push_back({edof[e][i], edof[e][j], v});
                }
        }
        csr_from_triplets(m.ntotal, tk, K);
    }
    // total effective stiffness K + 4/dt^2 M + 2/dt C + dt/3 G
    void keff_total(CSR& Kt_eff) const {
        std::vector<Trip> tr;
        auto add = [&](const CSR& A_, double c) {
            for (int r = 0; r < A_.n; ++r) for (int i = A_.ptr[r]; i < A_.ptr[r + 1]; ++i) tr.push_back({r, A_.col[i], c * A_.val[i]});
        };
        add(Kt, 1.0); add(Mt, 4.0 / dt / dt); add(Ct, 2.0 / dt);
        if (!newmark) add(Gt, dt / 3.0);
        csr_from_triplets(s.m.ntotal, tr, Kt_eff);
    }
    // Reaction forces after step k (DynamicAnalysis::UpdateDomain,
    // DynamicAnalysis.cpp:128-150) through ExtendedNewmarkBeta /
    // NewmarkBeta::ComputeReactionForce (ExtendedNewmarkBeta.cpp:158-172,
    // NewmarkBeta.cpp:148-162): Fint_dyn - Fext(k) - Fbar (Fbar = 0), Fint_dyn
    // the node inertia m A (Assembler.cpp:569-592) and then, in element order,
    // the dynamic force of every element with a fixed node: solids Fint_e +
    // C_e V_e + M_e A_e (lin3DHexa8 / lin2DQuad4 ComputeInternalDynamicForces),
    // PML elements K_e u_e + C_e v_e + M_e a_e over all their dofs
    // (PML3DHexa8.cpp:746-767, PML2DQuad4: no history term), dashpots
    // eta a a^T V; reported on the dofs of fixed nodes (a node with a free-dof
    // entry of -1), zeros elsewhere.
    void reaction(int k, std::vector<double>& R) const {
        const Model& m = s.m;
        const int nt = m.ntotal, nen = m.nen;
        std::vector<char> fixed(m.nnode, 0), dof_fixed(nt, 0);
        for (int n = 0; n < m.nnode; ++n) {
            for (int j = 0; j < m.nndof[n]; ++j) if (m.fdof_all[(size_t)n * m.dstride + j] == -1) fixed[n] = 1;
            if (fixed[n]) for (int j = 0; j < m.nndof[n]; ++j) dof_fixed[m.tdof_all[(size_t)n * m.dstride + j]] = 1;
        }
        std::vector<double> F(nt, 0.0);
        if (!m.nodemass.empty()) for (int t = 0; t < nt; ++t) F[t] += m.nodemass[t] * A[t];
        std::vector<double> fe(72), Me(72 * 72), Ce(72 * 72), Ke(72 * 72), K0(72 * 72);
        for (int e = 0; e < m.nelem; ++e) {
            bool hf = false;
            for (int a = 0; a < nen; ++a) hf = hf || fixed[m.conn[(size_t)e * nen + a]];
            if (!hf) continue;
            const std::vector<int>& ed = edof[e];
            const int nc = (int)ed.size();
            if (pml(e)) {
                pml_elem(e, Me.data(), Ce.data(), Ke.data(), nullptr);
                for (int i = 0; i < nc; ++i) {
                    double ku = 0.0, cv = 0.0, ma = 0.0;
                    for (int j = 0; j < nc; ++j) {
                        ku += Ke[(size_t)i * nc + j] * U[ed[j]];
                        cv += Ce[(size_t)i * nc + j] * V[ed[j]];
                        ma += Me[(size_t)i * nc + j] * A[ed[j]];
                    }
                    F[ed[i]] += (ku + cv) + ma;
                }
                continue;
            }
            s.element_fint(e, fe.data());
            s.element_M(e, Me.data(), m.lumped != 0);
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * e], ak = m.ray.empty() ? 0.0 : m.ray[2 * e + 1];
            if (ak != 0.0) s.element_K0(e, K0.data());
            for (int i = 0; i < nc; ++i) {
                double cv = 0.0, ma = 0.0;
                for (int j = 0; j < nc; ++j) {
                    const double c = am * Me[(size_t)i * nc + j] + (ak != 0.0 ? ak * K0[(size_t)i * nc + j] : 0.0);
                    cv += c * V[ed[j]];
                    ma += Me[(size_t)i * nc + j] * A[ed[j]];
                }
                F[ed[i]] += (fe[i] + cv) + ma;
            }
        }
        std::vector<int> node_of(nt, -1);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j) node_of[m.tdof_all[(size_t)n * m.dstride + j]] = n;
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            const int a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
            if (!fixed[node_of[a]] && !fixed[node_of[b]]) continue;
            const double eta = m.dp_eta[i];
            F[a] += eta * (V[a] - V[b]);
            F[b] += eta * (V[b] - V[a]);
        }
        std::vector<double> Fx;
        s.fext(k, Fx);
        R.assign(nt, 0.0);
        for (int t = 0; t < nt; ++t) if (dof_fixed[t]) R[t] = F[t] - Fx[t];
    }
    // One ExtendedNewmarkBeta::ComputeNewStep with Linear (algo 0) or
    // NewtonRaphson (algo 1: test 5, algo 2: test 4).  Every iteration
    // re-evaluates ComputeEffectiveForce (:208-229, which has no increment
    // terms: only Fint follows the iterate through the element states),
    // ComputeEffectiveStiffness (:233-245, K with the current tangents) and
    // the support-motion term (:190-204), solves, accumulates dU and updates
    // the solid elements from U + T dU (NewtonRaphson.cpp:24-75,
    // Algorithm.cpp:18-56).
    int step(int k, int algo = 0, int maxit = 1, double cnvgtol = 0.0) {
        const Model& m = s.m;
        const int nt = m.ntotal, nf = m.nfree;
        std::vector<double> Fint(nt), Fext, w(nt), MW, CV, GW, F(nt), Feff, SM, du, dUt, dUf(nf, 0.0), Us(nt);
        double fe[72], ue[72];
        std::vector<double> Ke(72 * 72);
        double norm0 = 0.0, res = 0.0;
        int it = 0;
        s.support_increment(newmark ? k - 1 : k, SM);
        bool anySM = false; for (double v : SM) if (v != 0.0) { anySM = true; break; }
        Us = U;                                  // node displacements + increments T dU
        dUt.assign(nt, 0.0);
        for (;;) {
            // Fint in element order with the force filter; a PML element takes
            // K_e (U + T dU) of its nodes (PML3DHexa8.cpp:716-742: the node
            // increments are T dU of the iterate, Algorithm.cpp:18-56, zero
            // after UpdateDomain)
            std::fill(Fint.begin(), Fint.end(), 0.0);
            for (int e = 0; e < m.nelem; ++e) {
                const int nc = (int)edof[e].size();
                if (pml(e)) {
                    pml_elem(e, nullptr, nullptr, Ke.data(), nullptr);
                    for (int i = 0; i < nc; ++i) ue[i] = Us[edof[e][i]];
                    for (int i = 0; i < nc; ++i) {
                        double v = 0.0;
                        for (int j = 0; j < nc; ++j) v += Ke[(size_t)i * nc + j] * ue[j];
                        fe[i] = v;
                    }
                } else {
                    s.element_fint(e, fe);
                }
                for (int j = 0; j < nc; ++j) if (std::fabs(fe[j]) > s.ftol) Fint[edof[e][j]] += fe[j];
            }
            s.fext(k, Fext);
            if (newmark) {
                // Fext + Fbar - Fint + M (4/dt V + A - 4/dt^2 dU) + C (V - 2/dt dU) (NewmarkBeta.cpp:215)
                for (int t = 0; t < nt; ++t) w[t] = 4.0 / dt * V[t] + A[t] - 4.0 / dt / dt * dUt[t];
                csr_mv(Mt, w, MW);
                for (int t = 0; t < nt; ++t) w[t] = V[t] - 2.0 / dt * dUt[t];
                csr_mv(Ct, w, CV);
                for (int t = 0; t < nt; ++t) F[t] = ((Fext[t] + 0.0 - Fint[t]) + MW[t]) + CV[t];
            } else {
                for (int t = 0; t < nt; ++t) w[t] = 4.0 / dt * V[t] + A[t];
                csr_mv(Mt, w, MW);
                csr_mv(Ct, V, CV);
                for (int t = 0; t < nt; ++t) w[t] = Ubar[t] + dt * U[t] + dt * dt / 6.0 * V[t];
                csr_mv(Gt, w, GW);
                for (int t = 0; t < nt; ++t) F[t] = (((Fext[t] + 0.0 - Fint[t]) - GW[t]) + CV[t]) + MW[t];
            }
            s.TT_apply(F, Feff);
            if (nonlinear) assemble_K(Kt);
            CSR Ktot; keff_total(Ktot);
            if (anySM) {
                std::vector<double> KS, lg; csr_mv(Ktot, SM, KS); s.TT_apply(KS, lg);
                for (int f = 0; f < nf; ++f) Feff[f] -= lg[f];
            }
            // T^T Keff T
            std::vector<Trip> tr;
            for (int r = 0; r < Ktot.n; ++r)
                for (int i = Ktot.ptr[r]; i < Ktot.ptr[r + 1]; ++i)
                    for (int a = s.Tptr[r]; a < s.Tptr[r + 1]; ++a)
                        for (int b = s.Tptr[Ktot.col[i]]; b < s.Tptr[Ktot.col[i] + 1]; ++b)
                            tr.push_back({s.Tcol[a], s.Tcol[b], s.Tval[a] * Ktot.val[i] * s.Tval[b]});
            CSR Kff; csr_from_triplets(nf, tr, Kff);
            if (solver == 0) { if (!dense_ldlt_solve(Kff, Feff, du)) return SVL_ERR_BREAKDOWN; }
            else return SVL_ERR_INVALID;
            for (int f = 0; f < nf; ++f) dUf[f] += du[f];
            if (algo != 0) res = convergence(newton_test(algo), it, Feff, dUf, du, norm0);
            s.T_apply(dUf, dUt);
            for (int t = 0; t < nt; ++t) Us[t] = U[t] + dUt[t];
            for (int e = 0; e < m.nelem; ++e) if (!pml(e)) s.element_update(e, Us);
            ++it;
            if (algo == 0 || !(res > cnvgtol) || it >= maxit) break;
        }
        last_iters = it;
        last_res = res;
        for (int t = 0; t < nt; ++t) {
            const double d = dUt[t], D = d + SM[t];
            if (!newmark) Ubar[t] = Ubar[t] + dt * U[t] + dt / 3.0 * D + dt * dt / 6.0 * V[t];
            U[t] += D;
            A[t] = 4.0 / dt / dt * d - 4.0 / dt * V[t] - A[t];
            V[t] = 2.0 / dt * d - V[t];
        }
        s.commit_all();
        return 0;
    }
};

/* ---------------- Explicit central difference with PML layers -------------- */

/* A scheme of this library, not a restatement: the reference's
 * CentralDifference never applies the PML history matrix G
 * (CentralDifference::GetPMLHistoryVector returns an empty vector,
 * CentralDifference.cpp:114-120) and keeps the PML mass consistent with a
 * negative stress block (PML3DHexa8.cpp:214-284), so M/dt^2 + C/2dt is sparse
 * and indefinite there.  This scheme advances the same semi-discrete system
 *   M x'' + C x' + K x + G xbar = F,   xbar = integral of x,
 * with the element matrices M, C, K, G of PML2DQuad4 / PML3DHexa8
 * (pml_matrices above, PML3DHexa8.cpp:214-712) and of the solid elements
 * (lumped mass, internal force from the material state), explicitly:
 *
 * 1. Split of the PML element matrices.  Every PML matrix is a "mass-like"
 *    part (the displacement-displacement and stress-stress blocks, which are
 *    N_j N_k integrals) plus the displacement-stress coupling (dN N blocks).
 *    The mass-like parts are row-sum lumped per node: diagonal on the
 *    displacement dofs (Mu, Cu, Ku, Gu) and one ns x ns block per node on its
 *    stress dofs (Ms, Cs, Ks, Gs; ns = 3 in 2D, 6 in 3D).  The couplings act
 *    as element matrix products.  Solid elements contribute their lumped mass
 *    (with the mass tolerance, as CentralDifference) to Mu and their internal
 *    force to the displacement rows.
 * 2. Staggered time levels.  Displacements u live at the integer steps,
 *    the PML stress dofs S (the time integral of the stress, so S' is the
 *    stress) at the half steps: at the start of step k the state holds u^k,
 *    u^(k-1), S^(k+1/2), S^(k-1/2), ubar^k and Sbar^k.
 * 3. Displacement rows at t_k (central differences; the increment form of
 *    CentralDifference.cpp:206-221, diagonal solve):
 *      (Mu/dt^2 + Cu/2dt) du = Fext(k) - Fint_solid(u^k)
 *          - [C_uS sdot + K_uS smid + G_uS Sbar^k]_elements
 *          - Ku u^k - Gu ubar^k + (Mu/dt^2 - Cu/2dt)(u^k - u^(k-1)),
 *    sdot = (S^(k+1/2) - S^(k-1/2))/dt, smid = (S^(k+1/2) + S^(k-1/2))/2;
 *    u^(k+1) = u^k + du on free dofs (restrained: 0, or the support-motion
 *    increment).
 * 4. ubar^(k+1) = ubar^k + dt (u^k + u^(k+1))/2, Sbar^(k+1) = Sbar^k + dt S^(k+1/2).
 * 5. Stress rows at t_(k+1/2):
 *      (Ms/dt^2 + Cs/2dt) dS = - [C_Su udot + K_Su umid + G_Su ubar^(k+1/2)]_elements
 *          - Ks S^(k+1/2) - Gs Sbar^(k+1/2) + (Ms/dt^2 - Cs/2dt)(S^(k+1/2) - S^(k-1/2)),
 *    udot = (u^(k+1) - u^k)/dt, umid = (u^(k+1) + u^k)/2,
 *    ubar^(k+1/2) = (ubar^k + ubar^(k+1))/2, Sbar^(k+1/2) = Sbar^k + dt/2 S^(k+1/2);
 *    S^(k+3/2) = S^(k+1/2) + dS (one ns x ns solve per PML node).
 * Away from the PML (a = 1, b = c = d = 0) this is the leapfrog scheme of the
 * velocity-stress system, stable for dt below the lumped-mass limit.  Element
 * contributions are summed per dof in element order, unfiltered; the total-dof
 * vector U holds u^k on displacement dofs and S^(k+1/2) on stress dofs, Up
 * u^(k-1) and S^(k-1/2), Ubar ubar^k and Sbar^k.  V and A are the central
 * difference formulas of CentralDifference.cpp:141-144 on every dof.
 * Restrictions: constraints only with one master per constrained dof (the
 * EQUAL ties of mergeDomain) and not on stress dofs, no dashpots, no
 * domain-reduction loads, no restrained stress dofs, support motion only on displacement dofs, Rayleigh
 * damping only mass-proportional on solid elements. */
struct CDPml {
    Sim s; double dt;
    int ns = 0, pnd = 0;
    std::vector<double> U, Up, Ubar, V, A;
    std::vector<char> sdof;                 // [ntotal] 1 for a PML stress dof
    std::vector<double> Mu, Cu, Ku, Gu;     // [ntotal] lumped diagonals of the displacement rows
    std::vector<int> sfirst;                // [nnode] first total dof of the node's stress block, or -1
    std::vector<int> snodes;                // nodes with a stress block
    std::vector<int> snode_idx;             // [nnode] index into snodes, or -1
    std::vector<double> Ms, Cs, Ks, Gs, Dinv;   // [snodes][ns*ns]
    std::vector<double> Kff_inv;            // [nfree] 1 / (T^T d T) on displacement free dofs, 0 on stress ones
    std::vector<std::vector<int>> edof;
    bool pml(int e) const { return !s.m.epml.empty() && s.m.epml[e]; }

    void pml_elem(int e, double* Me, double* Ce, double* Ke, double* Ge) const {
        const Model& m = s.m;
        double X[8 * 3];
        for (int a = 0; a < m.nen; ++a)
            for (int i = 0; i < m.ndim; ++i) X[a * m.ndim + i] = m.X[(size_t)m.conn[(size_t)e * m.nen + a] * m.ndim + i];
        const double* p = s.mp(e);
        pml_matrices(m.ndim, X, p[0], p[1], p[2], m.ndim == 2 ? m.thick[e] : 1.0,
                     &m.pml_par[(size_t)e * (3 + 2 * m.ndim)], Me, Ce, Ke, Ge);
    }

    int init(const svl_model_desc* d, const svl_load_desc* l, double dt_, double mtol) {
        if (!s.init(d, l)) return SVL_ERR_INVALID;
        Model& m = s.m;
        dt = dt_; s.mtol = mtol;
        if (!m.lumped || !m.dp_eta.empty() || !s.L.drm_elem.empty()) return SVL_ERR_UNSUPPORTED;
        pnd = m.ndim == 2 ? 5 : 9;
        ns = pnd - m.ndim;
        const int nt = m.ntotal;
        for (int e = 0; e < m.nelem; ++e) {
            const int t = s.mt(e);
            const bool el = t == SVL_MAT_ELASTIC2DPLANESTRAIN || t == SVL_MAT_ELASTIC3DLINEAR;
            if (!el && pml(e)) return SVL_ERR_UNSUPPORTED;
            if (!m.ray.empty() && (m.ray[2 * e + 1] != 0.0 || (pml(e) && m.ray[2 * e] != 0.0))) return SVL_ERR_UNSUPPORTED;
        }
        U.assign(nt, 0); Up.assign(nt, 0); Ubar.assign(nt, 0); V.assign(nt, 0); A.assign(nt, 0);
        sdof.assign(nt, 0);
        sfirst.assign(m.nnode, -1);
        edof.resize(m.nelem);
        std::vector<char> pnode(m.nnode, 0);
        for (int e = 0; e < m.nelem; ++e) {
            const int k = pml(e) ? pnd : m.ndim;
            for (int a = 0; a < m.nen; ++a) {
                const int n = m.conn[(size_t)e * m.nen + a];
                if (k > m.nndof[n]) return SVL_ERR_INVALID;
                if (pml(e)) pnode[n] = 1;
                for (int j = 0; j < k; ++j) edof[e].push_back(m.tdof_all[(size_t)n * m.dstride + j]);
            }
        }
        for (int n = 0; n < m.nnode; ++n) {
            if (!pnode[n]) continue;
            snodes.push_back(n);
            sfirst[n] = m.tdof_all[(size_t)n * m.dstride + m.ndim];
            for (int j = 0; j < ns; ++j) {
                const int t = m.tdof_all[(size_t)n * m.dstride + m.ndim + j];
                if (t != sfirst[n] + j) return SVL_ERR_UNSUPPORTED;       // stress dofs consecutive
                if (m.fdof_all[(size_t)n * m.dstride + m.ndim + j] < 0) return SVL_ERR_UNSUPPORTED;
                sdof[t] = 1;
            }
        }
        for (int d0 : s.L.smdof) if (sdof[d0]) return SVL_ERR_UNSUPPORTED;
        // lumped mass-like parts, summed in element order; the element row sums
        // are formed in parallel in chunks of elements, then added in order
        Mu.assign(nt, 0); Cu.assign(nt, 0); Ku.assign(nt, 0); Gu.assign(nt, 0);
        const size_t nb = (size_t)ns * ns;
        snode_idx.assign(m.nnode, -1);
        for (size_t i = 0; i < snodes.size(); ++i) snode_idx[snodes[i]] = (int)i;
        Ms.assign(snodes.size() * nb, 0); Cs = Ms; Ks = Ms; Gs = Ms; Dinv = Ms;
        const int ncmax = m.nen * pnd;
        const int ncs = m.nen * m.ndim;
        const int nw = m.ndim == 3 ? 4 : 3;
        const size_t per = (size_t)nw * (ncs + m.nen * nb);      // row sums of one element
        const int chunk = 4096;
        std::vector<double> rs((size_t)chunk * per);
        for (int e0 = 0; e0 < m.nelem; e0 += chunk) {
            const int e1 = std::min(m.nelem, e0 + chunk);
            std::vector<double> Xe0((size_t)ncmax * ncmax), Xe1(Xe0.size()), Xe2(Xe0.size()), Xe3(Xe0.size());
            std::vector<double> Me((size_t)ncs * ncs);
            #pragma omp parallel for schedule(dynamic, 16) firstprivate(Xe0, Xe1, Xe2, Xe3, Me)
            for (int e = e0; e < e1; ++e) {
                double* r = &rs[(size_t)(e - e0) * per];
                if (!pml(e)) {
                    s.element_M(e, Me.data(), true);
                    for (int i = 0; i < ncs; ++i) r[i] = Me[(size_t)i * ncs + i];
                    continue;
                }
                pml_elem(e, Xe0.data(), Xe1.data(), Xe2.data(), m.ndim == 3 ? Xe3.data() : nullptr);
                const double* Xs[4] = {Xe0.data(), Xe1.data(), Xe2.data(), Xe3.data()};
                const int nc = m.nen * pnd;
                for (int w = 0; w < nw; ++w) {
                    const double* X = Xs[w];
                    double* ru = r + (size_t)w * (ncs + m.nen * nb);
                    double* rb = ru + ncs;
                    for (int j = 0; j < m.nen; ++j) {
                        for (int c = 0; c < m.ndim; ++c) {
                            double v = 0.0;
                            for (int k = 0; k < m.nen; ++k) v += X[(size_t)(j * pnd + c) * nc + k * pnd + c];
                            ru[j * m.ndim + c] = v;
                        }
                        for (int rr = 0; rr < ns; ++rr)
                            for (int c = 0; c < ns; ++c) {
                                double v = 0.0;
                                for (int k = 0; k < m.nen; ++k) v += X[(size_t)(j * pnd + m.ndim + rr) * nc + k * pnd + m.ndim + c];
                                rb[(size_t)j * nb + rr * ns + c] = v;
                            }
                    }
                }
            }
            for (int e = e0; e < e1; ++e) {
                const double* r = &rs[(size_t)(e - e0) * per];
                if (!pml(e)) {
                    // lumped solid mass with the mass tolerance (Assembler.cpp:623-697)
                    for (int i = 0; i < ncs; ++i) if (std::fabs(r[i]) > mtol) Mu[edof[e][i]] += r[i];
                    if (!m.ray.empty() && m.ray[2 * e] != 0.0)
                        for (int i = 0; i < ncs; ++i) {
                            const double v = m.ray[2 * e] * r[i];
                            if (std::fabs(v) > s.ktol) Cu[edof[e][i]] += v;
                        }
                    continue;
                }
                std::vector<double>* du[4] = {&Mu, &Cu, &Ku, &Gu};
                std::vector<double>* bs[4] = {&Ms, &Cs, &Ks, &Gs};
                for (int w = 0; w < nw; ++w) {
                    const double* ru = r + (size_t)w * (ncs + m.nen * nb);
                    const double* rb = ru + ncs;
                    for (int j = 0; j < m.nen; ++j) {
                        const int n = m.conn[(size_t)e * m.nen + j];
                        for (int c = 0; c < m.ndim; ++c) (*du[w])[edof[e][j * pnd + c]] += ru[j * m.ndim + c];
                        double* B = &(*bs[w])[(size_t)snode_idx[n] * nb];
                        for (size_t k = 0; k < nb; ++k) B[k] += rb[(size_t)j * nb + k];
                    }
                }
            }
        }
        if (!m.nodemass.empty())
            for (int t = 0; t < nt; ++t) if (std::fabs(m.nodemass[t]) > mtol) Mu[t] += m.nodemass[t];
        // T^T (Mu/dt^2 + Cu/2dt) T, diagonal when every constrained dof has one
        // master (the EQUAL constraints of mergeDomain); stress dofs are free and
        // unconstrained, solved per node below
        {
            std::vector<double> kf(m.nfree, 0.0);
            std::vector<int> ncol(nt, 0);
            for (int t = 0; t < nt; ++t) {
                if (sdof[t]) continue;
                ncol[t] = s.Tptr[t + 1] - s.Tptr[t];
                if (ncol[t] > 1) return SVL_ERR_UNSUPPORTED;
                const double d = 1.0 / dt / dt * Mu[t] + 1.0 / 2.0 / dt * Cu[t];
                for (int i = s.Tptr[t]; i < s.Tptr[t + 1]; ++i) kf[s.Tcol[i]] += s.Tval[i] * d * s.Tval[i];
            }
            Kff_inv.assign(m.nfree, 0.0);
            std::vector<char> sfree(m.nfree, 0);
            for (int t = 0; t < nt; ++t)
                if (sdof[t]) for (int i = s.Tptr[t]; i < s.Tptr[t + 1]; ++i) sfree[s.Tcol[i]] = 1;
            for (int f = 0; f < m.nfree; ++f) {
                if (sfree[f]) continue;
                if (!(kf[f] > 0.0)) return SVL_ERR_INVALID;
                Kff_inv[f] = 1.0 / kf[f];
            }
        }
        // inverse of Ms/dt^2 + Cs/2dt per node (Gauss-Jordan with partial pivoting)
        for (int n : snodes) {
            const size_t sb = (size_t)snode_idx[n] * nb;
            double Aa[36], B[36];
            for (size_t i = 0; i < nb; ++i) {
                Aa[i] = Ms[sb + i] / dt / dt + Cs[sb + i] / 2.0 / dt;
                B[i] = 0.0;
            }
            for (int i = 0; i < ns; ++i) B[i * ns + i] = 1.0;
            for (int c = 0; c < ns; ++c) {
                int p = c;
                for (int r = c + 1; r < ns; ++r) if (std::fabs(Aa[r * ns + c]) > std::fabs(Aa[p * ns + c])) p = r;
                if (!(std::fabs(Aa[p * ns + c]) > 0.0)) return SVL_ERR_INVALID;
                if (p != c) for (int j = 0; j < ns; ++j) { std::swap(Aa[p * ns + j], Aa[c * ns + j]); std::swap(B[p * ns + j], B[c * ns + j]); }
                const double piv = Aa[c * ns + c];
                for (int j = 0; j < ns; ++j) { Aa[c * ns + j] /= piv; B[c * ns + j] /= piv; }
                for (int r = 0; r < ns; ++r) {
                    if (r == c) continue;
                    const double f = Aa[r * ns + c];
                    if (f == 0.0) continue;
                    for (int j = 0; j < ns; ++j) { Aa[r * ns + j] -= f * Aa[c * ns + j]; B[r * ns + j] -= f * B[c * ns + j]; }
                }
            }
            for (size_t i = 0; i < nb; ++i) Dinv[sb + i] = B[i];
        }
        return SVL_OK;
    }
    void set_initial(const double* U0, const double* V0, const double* A0) {
        for (int t = 0; t < s.m.ntotal; ++t) {
            const double u = U0 ? U0[t] : 0.0, v = V0 ? V0[t] : 0.0, a = A0 ? A0[t] : 0.0;
            U[t] = u; V[t] = v; A[t] = a;
            Up[t] = u - dt * v + dt * dt / 2.0 * a;
            Ubar[t] = 0.0;
        }
        for (int e = 0; e < s.m.nelem; ++e) if (!pml(e)) s.element_update(e, U);
        s.commit_all();
    }
    // u-rows (which = 0) or S-rows (which = 1) of X_e w_e summed over the three
    // (2D: two) coupling matrices C, K, G with the inputs in0, in1, in2
    // (entries of the other class are zero), element order, into F.
    void couple(int which, const std::vector<double>& in0, const std::vector<double>& in1,
                const std::vector<double>& in2, std::vector<double>& F) const {
        const Model& m = s.m;
        const int nc = m.nen * pnd;
        std::vector<double> Ce((size_t)nc * nc), Ke(Ce.size()), Ge(Ce.size());
        std::vector<double> fe_all;
        std::vector<int> pe;
        for (int e = 0; e < m.nelem; ++e) if (pml(e)) pe.push_back(e);
        fe_all.assign(pe.size() * nc, 0.0);
        #pragma omp parallel for schedule(dynamic, 16) firstprivate(Ce, Ke, Ge)
        for (long ii = 0; ii < (long)pe.size(); ++ii) {
            const int e = pe[ii];
            pml_elem(e, nullptr, Ce.data(), Ke.data(), m.ndim == 3 ? Ge.data() : nullptr);
            double* fe = &fe_all[(size_t)ii * nc];
            const std::vector<double>* ins[3] = {&in0, &in1, &in2};
            const double* mats[3] = {Ce.data(), Ke.data(), Ge.data()};
            for (int w = 0; w < (m.ndim == 3 ? 3 : 2); ++w) {
                double x[72];
                for (int i = 0; i < nc; ++i) {
                    const int t = edof[e][i];
                    const bool is_s = (i % pnd) >= m.ndim;
                    x[i] = (which == 0) == is_s ? (*ins[w])[t] : 0.0;
                }
                for (int r = 0; r < nc; ++r) {
                    if (((r % pnd) >= m.ndim) != (which == 1)) continue;
                    double acc = 0.0;
                    for (int c = 0; c < nc; ++c) acc += mats[w][(size_t)r * nc + c] * x[c];
                    fe[r] += acc;
                }
            }
        }
        for (size_t ii = 0; ii < pe.size(); ++ii) {
            const int e = pe[ii];
            for (int r = 0; r < nc; ++r)
                if (((r % pnd) >= m.ndim) == (which == 1)) F[edof[e][r]] += fe_all[ii * nc + r];
        }
    }
    void step(int k) {
        const Model& m = s.m;
        const int nt = m.ntotal;
        const size_t nb = (size_t)ns * ns;
        const int ncs = m.nen * m.ndim, nc = m.nen * pnd;
        std::vector<double> Fext, SM, sdot(nt, 0.0), smid(nt, 0.0), dU(nt, 0.0), Us(nt), Ubn(nt), Ubh(nt);
        // -- displacement rows ------------------------------------------------
        for (int t = 0; t < nt; ++t)
            if (sdof[t]) { sdot[t] = (U[t] - Up[t]) / dt; smid[t] = (U[t] + Up[t]) / 2.0; }
        // element forces on the displacement rows: solid internal force from the
        // material state, PML couplings C_uS sdot + K_uS smid + G_uS Sbar; summed in
        // element order with the force filter (Assembler.cpp:240-269)
        std::vector<double> Fc(nt, 0.0), fe_all((size_t)m.nelem * nc, 0.0);
        {
            std::vector<double> Ce((size_t)nc * nc), Ke(Ce.size()), Ge(Ce.size());
            #pragma omp parallel for schedule(dynamic, 16) firstprivate(Ce, Ke, Ge)
            for (int e = 0; e < m.nelem; ++e) {
                double* fe = &fe_all[(size_t)e * nc];
                if (!pml(e)) { s.element_fint(e, fe); continue; }
                pml_elem(e, nullptr, Ce.data(), Ke.data(), m.ndim == 3 ? Ge.data() : nullptr);
                double x0[72], x1[72], x2[72];
                for (int i = 0; i < nc; ++i) {
                    const int t = edof[e][i];
                    const bool is_s = (i % pnd) >= m.ndim;
                    x0[i] = is_s ? sdot[t] : 0.0; x1[i] = is_s ? smid[t] : 0.0; x2[i] = is_s ? Ubar[t] : 0.0;
                }
                for (int r = 0; r < nc; ++r) {
                    if ((r % pnd) >= m.ndim) continue;
                    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
                    for (int c = 0; c < nc; ++c) {
                        a0 += Ce[(size_t)r * nc + c] * x0[c];
                        a1 += Ke[(size_t)r * nc + c] * x1[c];
                        if (m.ndim == 3) a2 += Ge[(size_t)r * nc + c] * x2[c];
                    }
                    fe[r] = a0 + a1 + a2;
                }
            }
        }
        for (int e = 0; e < m.nelem; ++e) {
            const double* fe = &fe_all[(size_t)e * nc];
            const int n_e = pml(e) ? nc : ncs;
            for (int r = 0; r < n_e; ++r) {
                if (pml(e) && (r % pnd) >= m.ndim) continue;
                if (std::fabs(fe[r]) > s.ftol) Fc[edof[e][r]] += fe[r];
            }
        }
        s.fext(k, Fext);
        s.support_increment(k, SM);
        // the increment form of the plain central difference (CentralDifference.cpp:206-221)
        // with the lumped PML terms, reduced to the free dofs by T^T, the diagonal
        // (1/d) b solve, and expanded by T
        std::vector<double> Rt(nt, 0.0), Feff, du_f, dUt;
        for (int t = 0; t < nt; ++t) {
            if (sdof[t]) continue;
            const double c = 1.0 / dt / dt * Mu[t] - 1.0 / 2.0 / dt * Cu[t];
            Rt[t] = ((Fext[t] + 0.0 - Fc[t]) - Ku[t] * U[t] - Gu[t] * Ubar[t]) + c * (U[t] - Up[t]);
        }
        s.TT_apply(Rt, Feff);
        du_f.assign(m.nfree, 0.0);
        for (int f = 0; f < m.nfree; ++f) du_f[f] = Kff_inv[f] * Feff[f];
        s.T_apply(du_f, dUt);
        for (int t = 0; t < nt; ++t) {
            if (sdof[t]) continue;
            const double du = dUt[t];
            Us[t] = U[t] + du;                 // strain without the support-motion increment (Algorithm.cpp:23)
            dU[t] = du + SM[t];
            const double un = U[t] + dU[t];
            Ubn[t] = Ubar[t] + dt * (U[t] + un) / 2.0;
            Ubh[t] = (Ubar[t] + Ubn[t]) / 2.0;
        }
        for (int e = 0; e < m.nelem; ++e) if (!pml(e)) s.element_update(e, Us);
        // -- stress rows --------------------------------------------------------
        std::vector<double> udot(nt, 0.0), umid(nt, 0.0), ubh(nt, 0.0), Fs(nt, 0.0);
        for (int t = 0; t < nt; ++t)
            if (!sdof[t]) {
                const double un = U[t] + dU[t];
                udot[t] = (un - U[t]) / dt; umid[t] = (un + U[t]) / 2.0; ubh[t] = Ubh[t];
            }
        couple(1, udot, umid, ubh, Fs);
        for (int n : snodes) {
            const int t0 = sfirst[n];
            const size_t sb = (size_t)snode_idx[n] * nb;
            double R[6];
            for (int r = 0; r < ns; ++r) {
                double v = -Fs[t0 + r];
                for (int c = 0; c < ns; ++c) {
                    const size_t i = sb + r * ns + c;
                    const double sc = U[t0 + c], sp = Up[t0 + c], sbh = Ubar[t0 + c] + dt / 2.0 * sc;
                    v += -Ks[i] * sc - Gs[i] * sbh + (Ms[i] / dt / dt - Cs[i] / 2.0 / dt) * (sc - sp);
                }
                R[r] = v;
            }
            for (int r = 0; r < ns; ++r) {
                double v = 0.0;
                for (int c = 0; c < ns; ++c) v += Dinv[sb + r * ns + c] * R[c];
                dU[t0 + r] = v;
                Ubn[t0 + r] = Ubar[t0 + r] + dt * U[t0 + r];
            }
        }
        // -- new state (CentralDifference.cpp:138-148 on every dof) -------------
        for (int t = 0; t < nt; ++t) {
            V[t] = 1.0 / 2.0 / dt * (U[t] + dU[t] - Up[t]);
            A[t] = 1.0 / dt / dt * (dU[t] - U[t] + Up[t]);
            Up[t] = U[t];
            U[t] += dU[t];
            Ubar[t] = Ubn[t];
        }
        s.commit_all();
    }
};

/* ---------------- C ABI of the oracle ------------------------------------ */
extern "C" {

/* Central difference run.  hist_U: [nsteps][ntotal] or NULL; V/A out: [ntotal]
 * or NULL.  mode 0 = reference-faithful single thread, 1 = fast (OpenMP). */
int oracle_cd_run(const svl_model_desc* model, const svl_load_desc* loads, double dt,
                  double ftol, double mtol, int k_first, int nsteps, int mode,
                  const double* U0, const double* V0, const double* A0,
                  double* hist_U, double* U_out, double* V_out, double* A_out, double* step_seconds) {
    {
        // a consistent mass or stiffness-proportional damping: the factorised
        // non-diagonal K (CDGen), one faithful mode
        Model probe;
        if (!load_model(model, probe)) return SVL_ERR_INVALID;
        if (probe.epml.empty() && CDGen::needed(probe)) {
            CDGen g;
            if (!g.init(model, loads, dt, ftol, mtol)) return SVL_ERR_INVALID;
            g.set_initial(U0, V0, A0);
            const int nt = g.s.m.ntotal;
            const auto t0 = std::chrono::steady_clock::now();
            for (int i = 0; i < nsteps; ++i) {
                g.step(k_first + i);
                if (hist_U) std::memcpy(hist_U + (size_t)i * nt, g.U.data(), sizeof(double) * nt);
            }
            if (step_seconds) step_seconds[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (U_out) std::memcpy(U_out, g.U.data(), sizeof(double) * nt);
            if (V_out) std::memcpy(V_out, g.V.data(), sizeof(double) * nt);
            if (A_out) std::memcpy(A_out, g.A.data(), sizeof(double) * nt);
            return 0;
        }
    }
    CD cd;
    if (!cd.init(model, loads, dt, ftol, mtol)) return SVL_ERR_INVALID;
    cd.set_initial(U0, V0, A0);
    if (mode == 1) cd.enable_fast();
    const int nt = cd.s.m.ntotal;
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < nsteps; ++i) {
        cd.step(k_first + i);
        if (hist_U) std::memcpy(hist_U + (size_t)i * nt, cd.U.data(), sizeof(double) * nt);
    }
    if (step_seconds) step_seconds[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (U_out) std::memcpy(U_out, cd.U.data(), sizeof(double) * nt);
    if (V_out) std::memcpy(V_out, cd.V.data(), sizeof(double) * nt);
    if (A_out) std::memcpy(A_out, cd.A.data(), sizeof(double) * nt);
    return 0;
}

/* Explicit central difference with PML layers (the staggered scheme of
 * CDPml above).  hist_U [nsteps][ntotal] or NULL; U/V/A/Ubar out [ntotal] or
 * NULL.  Returns an SVL_* status (UNSUPPORTED for models outside its scope). */
int oracle_cdpml_run(const svl_model_desc* model, const svl_load_desc* loads, double dt, double ftol, double mtol,
                     int k_first, int nsteps, const double* U0, const double* V0, const double* A0,
                     double* hist_U, double* U_out, double* V_out, double* A_out, double* Ubar_out,
                     double* step_seconds) {
    CDPml c;
    c.s.ftol = ftol;
    const int st = c.init(model, loads, dt, mtol);
    if (st) return st;
    c.s.ftol = ftol;
    c.set_initial(U0, V0, A0);
    const int nt = c.s.m.ntotal;
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < nsteps; ++i) {
        c.step(k_first + i);
        if (hist_U) std::memcpy(hist_U + (size_t)i * nt, c.U.data(), sizeof(double) * nt);
    }
    if (step_seconds) step_seconds[0] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (U_out) std::memcpy(U_out, c.U.data(), sizeof(double) * nt);
    if (V_out) std::memcpy(V_out, c.V.data(), sizeof(double) * nt);
    if (A_out) std::memcpy(A_out, c.A.data(), sizeof(double) * nt);
    if (Ubar_out) std::memcpy(Ubar_out, c.Ubar.data(), sizeof(double) * nt);
    return 0;
}

/* Newmark (average acceleration) run with Linear (algo 0) or Newton (algo 1)
 * iterations and a dense LDL^T (solver 0) or Jacobi-PCG (solver 1) solve. */
int oracle_newmark_run(const svl_model_desc* model, const svl_load_desc* loads, double dt,
                       int k_first, int nsteps, int algo, int maxit, double cnvgtol,
                       int solver, double pcg_tol, double* hist_U, long* pcg_iters, int* step_iters) {
    Newmark nm;
    if (!nm.init(model, loads, dt)) return SVL_ERR_INVALID;
    nm.solver = solver; nm.pcg_tol = pcg_tol;
    const int nt = nm.s.m.ntotal;
    for (int i = 0; i < nsteps; ++i) {
        int st = nm.step(k_first + i, algo, maxit, cnvgtol);
        if (st) return st;
        if (step_iters) step_iters[i] = nm.last_iters;
        if (hist_U) std::memcpy(hist_U + (size_t)i * nt, nm.U.data(), sizeof(double) * nt);
    }
    if (pcg_iters) *pcg_iters = nm.pcg_iters;
    return 0;
}

/* ExtendedNewmarkBeta (newmark 0) or NewmarkBeta (newmark 1: the effective
 * force with the increment terms, K + 4/dt^2 M + 2/dt C, the support-motion
 * increment of step k - 1, no PML history; NewmarkBeta.cpp:117-235) on models
 * with PML elements (dense LDL^T solve): algo 0 Linear, 1 Newton with test 5,
 * 2 Newton with test 4; step_iters [nsteps] or NULL. */
int oracle_xnewmark_run(const svl_model_desc* model, const svl_load_desc* loads, double dt, int k_first, int nsteps,
                        int algo, int maxit, double cnvgtol, int newmark,
                        double* hist_U, double* U_out, double* V_out, double* A_out, double* Ubar_out, int* step_iters,
                        double* last_res) {
    XNewmark x;
    x.newmark = newmark != 0;
    if (!x.init(model, loads, dt)) return SVL_ERR_INVALID;
    x.set_initial(nullptr, nullptr, nullptr, nullptr);
    const int nt = x.s.m.ntotal;
    for (int i = 0; i < nsteps; ++i) {
        int st = x.step(k_first + i, algo, algo == 0 ? 1 : maxit, cnvgtol);
        if (st) return st;
        if (step_iters) step_iters[i] = x.last_iters;
        if (last_res) *last_res = x.last_res;
        if (hist_U) std::memcpy(hist_U + (size_t)i * nt, x.U.data(), sizeof(double) * nt);
    }
    if (U_out) std::memcpy(U_out, x.U.data(), sizeof(double) * nt);
    if (V_out) std::memcpy(V_out, x.V.data(), sizeof(double) * nt);
    if (A_out) std::memcpy(A_out, x.A.data(), sizeof(double) * nt);
    if (Ubar_out) std::memcpy(Ubar_out, x.Ubar.data(), sizeof(double) * nt);
    return 0;
}

/* Reaction forces after `nsteps` steps from k_first of the central-difference
 * (integrator 0), NewmarkBeta (1, algo/maxit/cnvgtol as oracle_newmark_run),
 * ExtendedNewmarkBeta (2) or the NewmarkBeta mode of the PML model's
 * integrator (3) run; R_out [ntotal]. */
int oracle_reaction_run(const svl_model_desc* model, const svl_load_desc* loads, double dt, int k_first, int nsteps,
                        int integrator, int algo, int maxit, double cnvgtol, double* R_out) {
    std::vector<double> R;
    const int klast = k_first + nsteps - 1;
    if (integrator >= 2) {
        XNewmark x;
        x.newmark = integrator == 3;
        if (!x.init(model, loads, dt)) return SVL_ERR_INVALID;
        x.set_initial(nullptr, nullptr, nullptr, nullptr);
        for (int i = 0; i < nsteps; ++i) {
            int st = x.step(k_first + i, algo, algo == 0 ? 1 : maxit, cnvgtol);
            if (st) return st;
        }
        x.reaction(klast, R);
    } else if (integrator == 0) {
        CD cd;
        if (!cd.init(model, loads, dt, 1e-12, 1e-12)) return SVL_ERR_INVALID;
        cd.set_initial(nullptr, nullptr, nullptr);
        for (int i = 0; i < nsteps; ++i) cd.step(k_first + i);
        cd.s.reaction(klast, cd.V, cd.A, R);
    } else {
        Newmark nm;
        if (!nm.init(model, loads, dt)) return SVL_ERR_INVALID;
        for (int i = 0; i < nsteps; ++i) {
            int st = nm.step(k_first + i, algo, algo == 0 ? 1 : maxit, cnvgtol);
            if (st) return st;
        }
        nm.s.reaction(klast, nm.V, nm.A, R);
    }
    std::memcpy(R_out, R.data(), sizeof(double) * R.size());
    return 0;
}

/* ELEMENT recorder values (Sim::element_response) of the listed elements
 * after `nsteps` steps of central difference (integrator 0) or NewmarkBeta
 * (1, algo/maxit/cnvgtol as oracle_newmark_run); out [nlist][ngp*3|6] or
 * [nlist][NC]. */
int oracle_element_response_run(const svl_model_desc* model, const svl_load_desc* loads, double dt, int k_first,
                                 int nsteps, int integrator, int algo, int maxit, double cnvgtol, int response,
                                 int nlist, const int* elems, double* out) {
    auto emit = [&](const Sim& s) {
        const int per = response == 2 ? s.m.nen * s.m.ndof : s.m.ngp * (s.m.ndim == 2 ? 3 : 6);
        for (int i = 0; i < nlist; ++i) s.element_response(elems[i], response, out + (size_t)i * per);
    };
    Model probe;
    if (!load_model(model, probe)) return SVL_ERR_INVALID;
    if (integrator == 0 && probe.epml.empty() && CDGen::needed(probe)) {
        CDGen g;                            // non-diagonal K (consistent mass or ak != 0)
        if (!g.init(model, loads, dt, 1e-12, 1e-12)) return SVL_ERR_INVALID;
        g.set_initial(nullptr, nullptr, nullptr);
        for (int i = 0; i < nsteps; ++i) g.step(k_first + i);
        emit(g.s);
    } else if (integrator == 0) {
        CD cd;
        if (!cd.init(model, loads, dt, 1e-12, 1e-12)) return SVL_ERR_INVALID;
        cd.set_initial(nullptr, nullptr, nullptr);
        for (int i = 0; i < nsteps; ++i) cd.step(k_first + i);
        emit(cd.s);
    } else {
        Newmark nm;
        if (!nm.init(model, loads, dt)) return SVL_ERR_INVALID;
        for (int i = 0; i < nsteps; ++i) {
            int st = nm.step(k_first + i, algo, algo == 0 ? 1 : maxit, cnvgtol);
            if (st) return st;
        }
        emit(nm.s);
    }
    return 0;
}

/* Total-dof matrices K, M, C, G of the ExtendedNewmark model as dense arrays
 * (small models; the tests check structure and the time stepping with them). */
int oracle_xnewmark_matrices(const svl_model_desc* model, double* K, double* M, double* C, double* G) {
    XNewmark x;
    if (!x.init(model, nullptr, 1.0)) return SVL_ERR_INVALID;
    const int nt = x.s.m.ntotal;
    const CSR* src[4] = {&x.Kt, &x.Mt, &x.Ct, &x.Gt};
    double* dst[4] = {K, M, C, G};
    for (int q = 0; q < 4; ++q) {
        if (!dst[q]) continue;
        std::fill(dst[q], dst[q] + (size_t)nt * nt, 0.0);
        for (int r = 0; r < nt; ++r)
            for (int i = src[q]->ptr[r]; i < src[q]->ptr[r + 1]; ++i) dst[q][(size_t)r * nt + src[q]->col[i]] = src[q]->val[i];
    }
    return 0;
}

/* Element-level probes used by the tests. */
int oracle_element_fint(const svl_model_desc* model, const double* U_total, double* fe_all) {
    Sim s;
    if (!s.init(model, nullptr)) return SVL_ERR_INVALID;
    std::vector<double> U(U_total, U_total + s.m.ntotal);
    for (int e = 0; e < s.m.nelem; ++e) s.element_update(e, U);
    const int nc = s.m.nen * s.m.ndof;
    for (int e = 0; e < s.m.nelem; ++e) s.element_fint(e, fe_all + (size_t)e * nc);
    return 0;
}

int oracle_element_matrices(const svl_model_desc* model, int e, double* Ke, double* Me_lumped, double* Me_consistent) {
    Sim s;
    if (!s.init(model, nullptr)) return SVL_ERR_INVALID;
    if (Ke) s.element_K(e, Ke);
    if (Me_lumped) s.element_M(e, Me_lumped, true);
    if (Me_consistent) s.element_M(e, Me_consistent, false);
    return 0;
}

int oracle_body_force(const svl_model_desc* model, int e, const double* q, double* fe) {
    Sim s;
    if (!s.init(model, nullptr)) return SVL_ERR_INVALID;
    s.element_body(e, q, fe);
    return 0;
}

int oracle_lumped_mass(const svl_model_desc* model, double mtol, double* M) {
    Sim s;
    if (!s.init(model, nullptr)) return SVL_ERR_INVALID;
    s.mtol = mtol;
    std::vector<double> Md;
    s.assemble_mass_diag(Md);
    std::memcpy(M, Md.data(), sizeof(double) * Md.size());
    return 0;
}

/* PML element matrices (row-major nc x nc; any output may be NULL). */
int oracle_pml_matrices(int ndim, const double* X, double E, double nu, double rho, double t, const double* par,
                        double* M, double* C, double* K, double* G) {
    if (ndim != 2 && ndim != 3) return SVL_ERR_INVALID;
    pml_matrices(ndim, X, E, nu, rho, t, par, M, C, K, G);
    return 0;
}

/* Single Gauss-point J2 driver: applies `n` strain increments (engineering
 * strain rows of size 3 or 6) with a commit after each, returning the stress
 * after each increment. */
int oracle_j2_path(int mat_type, const double* param, int n, const double* strains, double* stresses) {
    MatState s; mat_init(s, mat_type, param);
    const int ns = (mat_type == SVL_MAT_PLASTICPLANESTRAINJ2 || mat_type == SVL_MAT_ELASTIC2DPLANESTRAIN) ? 3 : 6;
    for (int i = 0; i < n; ++i) {
        mat_update(s, mat_type, param, strains + (size_t)i * ns);
        mat_stress(s, mat_type, param, stresses + (size_t)i * ns);
        mat_commit(s);
    }
    return 0;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
