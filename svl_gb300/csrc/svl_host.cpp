// Host-side pieces of the C ABI: model validation, element geometry,
// lumped mass, the T operator, the structured-grid generator with the
// pre-processor's PlainScheme numbering, and element body loads.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <utility>

#include <functional>
#include <thread>

#include "svl_internal.hpp"

namespace svl {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

bool HostModel::has_j2() const {
    for (int t : mtype)
        if (t == SVL_MAT_PLASTICPLANESTRAINJ2 || t == SVL_MAT_PLASTIC3DJ2) return true;
    return false;
}

bool model_from_desc(const svl_model_desc* d, HostModel& m) {
    if (!d) { set_error("model descriptor is NULL"); return false; }
    m.ndim = d->ndim; m.nnode = d->nnode; m.ndof = d->ndof;
    m.ntotal = d->ntotal; m.nfree = d->nfree; m.etype = d->elem_type;
    m.nelem = d->nelem; m.nmat = d->nmat;
    if (m.etype == SVL_ELEM_LIN2DQUAD4) { m.nen = 4; m.ngp = 4; m.nstr = 3; }
    else if (m.etype == SVL_ELEM_LIN3DHEXA8) { m.nen = 8; m.ngp = 8; m.nstr = 6; }
    else { set_error("unsupported element type %d", m.etype); return false; }
    if ((m.etype == SVL_ELEM_LIN2DQUAD4 && m.ndim != 2) || (m.etype == SVL_ELEM_LIN3DHEXA8 && m.ndim != 3)) {
        set_error("element type %d does not match ndim %d", m.etype, m.ndim); return false;
    }
    const int pnd = m.ndim == 2 ? 5 : 9;
    m.dstride = d->ndof;
    if (m.dstride != m.ndim && m.dstride != pnd) {
        set_error("ndof (%d) must be ndim (%d), or %d with PML nodes", m.dstride, m.ndim, pnd); return false;
    }
    m.ndof = m.ndim;
    if (m.nnode <= 0 || m.nelem <= 0 || m.ntotal <= 0 || m.nfree < 0 || m.nmat <= 0) {
        set_error("empty model (nnode=%d nelem=%d ntotal=%d nfree=%d nmat=%d)", m.nnode, m.nelem, m.ntotal, m.nfree, m.nmat);
        return false;
    }
    if (!d->coords || !d->totaldof || !d->freedof || !d->conn || !d->elem_mat || !d->mat_type || !d->mat_param) {
        set_error("model descriptor has a NULL array"); return false;
    }
    m.X.assign(d->coords, d->coords + (size_t)m.nnode * m.ndim);
    m.nndof.assign(m.nnode, m.dstride);
    if (d->node_ndof) {
        for (int n = 0; n < m.nnode; ++n) {
            const int k = d->node_ndof[n];
            if (k != m.ndim && k != pnd) { set_error("node %d has %d dofs (%d or %d expected)", n, k, m.ndim, pnd); return false; }
            if (k > m.dstride) { set_error("node %d has %d dofs, more than the stride %d", n, k, m.dstride); return false; }
            m.nndof[n] = k;
        }
    }
    m.tdof_all.assign((size_t)m.nnode * m.dstride, -1);
    m.fdof_all.assign((size_t)m.nnode * m.dstride, -1);
    m.tdof.resize((size_t)m.nnode * m.ndim);
    m.fdof.resize((size_t)m.nnode * m.ndim);
    for (int n = 0; n < m.nnode; ++n)
        for (int j = 0; j < m.nndof[n]; ++j) {
            const size_t i = (size_t)n * m.dstride + j;
            m.tdof_all[i] = d->totaldof[i];
            m.fdof_all[i] = d->freedof[i];
            if (j < m.ndim) { m.tdof[(size_t)n * m.ndim + j] = d->totaldof[i]; m.fdof[(size_t)n * m.ndim + j] = d->freedof[i]; }
        }
    m.conn.assign(d->conn, d->conn + (size_t)m.nelem * m.nen);
    m.epml.clear(); m.pml_par.clear();
    if (d->elem_pml) {
        bool any = false;
        for (int e = 0; e < m.nelem; ++e) any |= d->elem_pml[e] != 0;
        if (any) {
            if (!d->elem_pml_param) { set_error("PML elements without elem_pml_param"); return false; }
            m.epml.assign(m.nelem, 0);
            for (int e = 0; e < m.nelem; ++e) m.epml[e] = d->elem_pml[e] != 0;
            m.pml_par.assign(d->elem_pml_param, d->elem_pml_param + (size_t)m.nelem * (3 + 2 * m.ndim));
        }
    }
    m.emat.assign(d->elem_mat, d->elem_mat + m.nelem);
    m.thick.assign(m.nelem, 1.0);
    if (d->elem_thickness) m.thick.assign(d->elem_thickness, d->elem_thickness + m.nelem);
    m.mtype.assign(d->mat_type, d->mat_type + m.nmat);
    m.mpar.assign(d->mat_param, d->mat_param + (size_t)m.nmat * SVL_MAT_NPARAM);
    m.nodemass.clear();
    if (d->node_mass) m.nodemass.assign(d->node_mass, d->node_mass + m.ntotal);
    if (d->elem_rayleigh) {
        m.ray.assign(d->elem_rayleigh, d->elem_rayleigh + (size_t)2 * m.nelem);
        bool any = false;
        for (double v : m.ray) {
            if (!std::isfinite(v)) { set_error("non-finite Rayleigh coefficient"); return false; }
            any |= v != 0.0;
        }
        if (!any) m.ray.clear();
    }
    m.dp_dof.clear(); m.dp_eta.clear();
    if (d->ndashpot > 0) {
        if (!d->dashpot_dof || !d->dashpot_eta) { set_error("dashpot arrays are NULL"); return false; }
        m.dp_dof.assign(d->dashpot_dof, d->dashpot_dof + 2 * (size_t)d->ndashpot);
        m.dp_eta.assign(d->dashpot_eta, d->dashpot_eta + d->ndashpot);
        for (int32_t t : m.dp_dof) if (t < 0 || t >= m.ntotal) { set_error("dashpot dof %d out of range", t); return false; }
        for (double e : m.dp_eta) if (!(e >= 0.0) || !std::isfinite(e)) { set_error("dashpot coefficient must be finite and >= 0"); return false; }
    } else if (d->ndashpot < 0) { set_error("ndashpot < 0"); return false; }
    m.lumped = d->lumped;
    m.nconstraint = d->nconstraint;
    m.cslave.clear(); m.cptr.assign(1, 0); m.cmaster.clear(); m.cfactor.clear();
    if (m.nconstraint > 0) {
        if (!d->con_slave || !d->con_ptr || !d->con_master || !d->con_factor) { set_error("constraint arrays are NULL"); return false; }
        m.cslave.assign(d->con_slave, d->con_slave + m.nconstraint);
        m.cptr.assign(d->con_ptr, d->con_ptr + m.nconstraint + 1);
        if (m.cptr[0] != 0) { set_error("con_ptr[0] must be 0"); return false; }
        for (int c = 0; c < m.nconstraint; ++c)
            if (m.cptr[c + 1] < m.cptr[c]) { set_error("con_ptr is not monotone"); return false; }
        m.cmaster.assign(d->con_master, d->con_master + m.cptr.back());
        m.cfactor.assign(d->con_factor, d->con_factor + m.cptr.back());
        for (int c = 0; c < m.nconstraint; ++c)
            if (m.cslave[c] < 0 || m.cslave[c] >= m.ntotal) { set_error("constraint %d slave dof out of range", c); return false; }
        for (int32_t f : m.cmaster)
            if (f < 0 || f >= m.nfree) { set_error("constraint master dof %d out of range", f); return false; }
    }
    // index checks: every later device access is bounded by these
    for (int32_t n : m.conn) if (n < 0 || n >= m.nnode) { set_error("connectivity node %d out of range", n); return false; }
    for (int32_t k : m.emat) if (k < 0 || k >= m.nmat) { set_error("element material %d out of range", k); return false; }
    {
        std::vector<char> seen(m.ntotal, 0), fseen(std::max(m.nfree, 1), 0);
        for (int n = 0; n < m.nnode; ++n)
            for (int j = 0; j < m.nndof[n]; ++j) {
                const int32_t t = m.tdof_all[(size_t)n * m.dstride + j], f = m.fdof_all[(size_t)n * m.dstride + j];
                if (t < 0 || t >= m.ntotal) { set_error("total dof %d out of range", t); return false; }
                if (seen[t]) { set_error("total dof %d appears twice", t); return false; }
                seen[t] = 1;
                if (f >= m.nfree) { set_error("free dof %d out of range", f); return false; }
                if (f >= 0) { if (fseen[f]) { set_error("free dof %d appears twice", f); return false; } fseen[f] = 1; }
            }
    }
    if (m.has_pml()) {
        // PML elements take every dof of their nodes; PML thresholds and stretching
        for (int e = 0; e < m.nelem; ++e) {
            if (!m.epml[e]) continue;
            for (int a = 0; a < m.nen; ++a)
                if (m.nndof[m.conn[(size_t)e * m.nen + a]] != pnd) { set_error("PML element %d has a node without %d dofs", e, pnd); return false; }
            const double* p = &m.pml_par[(size_t)e * (3 + 2 * m.ndim)];
            if (!(p[1] > 0.0) || !(p[2] > 0.0 && p[2] <= 1.0)) { set_error("PML element %d: L > 0 and 0 < R <= 1 needed", e); return false; }
            const int mt = m.mtype[m.emat[e]];
            if (mt != SVL_MAT_ELASTIC2DPLANESTRAIN && mt != SVL_MAT_ELASTIC3DLINEAR) { set_error("PML element %d needs an elastic material", e); return false; }
        }
    } else {
        for (int n = 0; n < m.nnode; ++n)
            if (m.nndof[n] != m.ndim) { set_error("node %d has %d dofs but the model has no PML element", n, m.nndof[n]); return false; }
    }
    for (int k = 0; k < m.nmat; ++k) {
        int t = m.mtype[k];
        bool two = (t == SVL_MAT_ELASTIC2DPLANESTRAIN || t == SVL_MAT_PLASTICPLANESTRAINJ2);
        bool three = (t == SVL_MAT_ELASTIC3DLINEAR || t == SVL_MAT_PLASTIC3DJ2);
        if (!(two || three)) { set_error("unsupported material type %d", t); return false; }
        if ((m.ndim == 2) != two) { set_error("material %d (type %d) does not match ndim %d", k, t, m.ndim); return false; }
    }
    return true;
}

static void natural_derivs(int nd, const double* xi, double dN[8][3], double N[8]) {
    if (nd == 2) {
        static const double sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
        for (int a = 0; a < 4; ++a) {
            N[a] = 0.25 * (1.0 + sr[a] * xi[0]) * (1.0 + ss[a] * xi[1]);
            dN[a][0] = 0.25 * sr[a] * (1.0 + ss[a] * xi[1]);
            dN[a][1] = 0.25 * ss[a] * (1.0 + sr[a] * xi[0]);
            dN[a][2] = 0.0;
        }
    } else {
        static const double sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
        static const double ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
        static const double st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        for (int a = 0; a < 8; ++a) {
            const double fr = 1.0 + sr[a] * xi[0], fs = 1.0 + ss[a] * xi[1], ft = 1.0 + st[a] * xi[2];
            N[a] = 0.125 * fr * fs * ft;
            dN[a][0] = 0.125 * sr[a] * fs * ft;
            dN[a][1] = 0.125 * ss[a] * fr * ft;
            dN[a][2] = 0.125 * st[a] * fr * fs;
        }
    }
}

double gp_geometry(const HostModel& m, int e, int q, double dNx[8][3], double N[8]) {
    const int nd = m.ndim, nen = m.nen;
    double xi[3] = {(q & 1) ? kGaussAbscissa : -kGaussAbscissa,
                    (q & 2) ? kGaussAbscissa : -kGaussAbscissa,
                    (q & 4) ? kGaussAbscissa : -kGaussAbscissa};
    if (nd == 2) xi[2] = 0.0;
    double dN[8][3];
    natural_derivs(nd, xi, dN, N);
    // J_ij = d x_j / d r_i
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < nen; ++a) {
        const double* x = &m.X[(size_t)m.conn[(size_t)e * nen + a] * nd];
        for (int i = 0; i < nd; ++i)
            for (int j = 0; j < nd; ++j) J[i][j] += dN[a][i] * x[j];
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
    for (int a = 0; a < nen; ++a)
        for (int j = 0; j < nd; ++j) {
            double v = 0.0;
            for (int i = 0; i < nd; ++i) v += Ji[j][i] * dN[a][i];
            dNx[a][j] = v;
        }
    if (nd == 2)
        for (int a = 0; a < nen; ++a) dNx[a][2] = 0.0;
    return det;
}

void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)>& body) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>(hw, std::max<int64_t>(1, n / 4096));
    if (nt <= 1) { body(0, n); return; }
    std::vector<std::thread> th;
    for (int64_t i = 0; i < nt; ++i) th.emplace_back(body, n * i / nt, n * (i + 1) / nt);
    for (auto& t : th) t.join();
}

// Row-sum lumped mass of every element node, diag[(e*nen + a)*nd + j],
// computed once per host model into its cache.
static const std::vector<double>& lumped_element_ref(const HostModel& m) {
    const int nd = m.ndim, nen = m.nen, nc = nen * m.ndof;
    if (m.elem_lumped.size() == (size_t)m.nelem * nen * nd) return m.elem_lumped;
    std::vector<double>& diag = m.elem_lumped;
    diag.assign((size_t)m.nelem * nen * nd, 0.0);
    // The consistent mass of a displacement element is block diagonal in the
    // components, Me[(a,j)][(b,j)] = sum_q c_q N_a N_b for every j, so the
    // row-sum lumping (lin2DQuad4.cpp:272-282: the diagonal plus the row's
    // other entries in ascending column order; the zero entries change
    // nothing) is m_aa + sum_{b != a, ascending} m_ab, the same for every
    // component -- the same operations in the same order as on the full matrix.
    (void)nc;
    parallel_for(m.nelem, [&](int64_t e0, int64_t e1) {
        for (int64_t e = e0; e < e1; ++e) {
            double mab[8][8] = {};
            const double rho = m.param((int)e)[2];
            for (int q = 0; q < m.ngp; ++q) {
                double dNx[8][3], N[8];
                const double det = gp_geometry(m, (int)e, q, dNx, N);
                const double c = nd == 2 ? 1.0 * rho * m.thick[e] * std::fabs(det) : 1.0 * rho * std::fabs(det);
                for (int a = 0; a < nen; ++a)
                    for (int b = 0; b < nen; ++b) mab[a][b] += c * (N[a] * N[b]);
            }
            for (int a = 0; a < nen; ++a) {
                double d = mab[a][a];
                for (int b = 0; b < nen; ++b)
                    if (b != a) d += mab[a][b];
                for (int j = 0; j < nd; ++j) diag[((size_t)e * nen + a) * nd + j] = d;
            }
        }
    });
    return diag;
}

void element_lumped_masses(const HostModel& m, std::vector<double>& diag) { diag = lumped_element_ref(m); }

void lumped_mass_diag(const HostModel& m, double mtol, std::vector<double>& M) {
    const int nd = m.ndim, nen = m.nen;
    // element diagonals in parallel, assembled afterwards in element order
    const std::vector<double>& diag = lumped_element_ref(m);
    std::vector<double> Me_e(m.ntotal, 0.0);
    for (int e = 0; e < m.nelem; ++e)
        for (int a = 0; a < nen; ++a)
            for (int j = 0; j < nd; ++j) {
                const double v = diag[((size_t)e * nen + a) * nd + j];
                if (std::fabs(v) > mtol) Me_e[m.tdof[(size_t)m.conn[(size_t)e * nen + a] * m.ndof + j]] += v;
            }
    M.assign(m.ntotal, 0.0);
    for (int t = 0; t < m.ntotal; ++t) {
        double mn = 0.0;
        if (!m.nodemass.empty() && std::fabs(m.nodemass[t]) > mtol) mn = m.nodemass[t];
        M[t] = Me_e[t] + mn;
    }
}

void dashpot_tables(const HostModel& m, std::vector<int32_t>& ptr, std::vector<int32_t>& col,
                    std::vector<double>& eta) {
    ptr.assign(m.ntotal + 1, 0);
    col.clear(); eta.clear();
    const size_t n = m.dp_eta.size();
    for (size_t i = 0; i < n; ++i) { ptr[m.dp_dof[2 * i] + 1]++; ptr[m.dp_dof[2 * i + 1] + 1]++; }
    for (int t = 0; t < m.ntotal; ++t) ptr[t + 1] += ptr[t];
    col.resize(ptr.back()); eta.resize(ptr.back());
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (size_t i = 0; i < n; ++i) {
        const int32_t a = m.dp_dof[2 * i], b = m.dp_dof[2 * i + 1];
        col[fill[a]] = b; eta[fill[a]++] = m.dp_eta[i];
        col[fill[b]] = a; eta[fill[b]++] = m.dp_eta[i];
    }
}

void rayleigh_mass_diag(const HostModel& m, std::vector<double>& C) {
    const int nd = m.ndim, nen = m.nen;
    C.assign(m.ntotal, 0.0);
    if (m.ray.empty()) return;
    const std::vector<double>& diag = lumped_element_ref(m);
    for (int e = 0; e < m.nelem; ++e) {
        const double am = m.ray[2 * (size_t)e];
        if (am == 0.0) continue;
        for (int a = 0; a < nen; ++a)
            for (int j = 0; j < nd; ++j)
                C[m.tdof[(size_t)m.conn[(size_t)e * nen + a] * m.ndof + j]] += am * diag[((size_t)e * nen + a) * nd + j];
    }
}

int build_load_tables(const HostModel& m, const svl_load_desc* L, LoadTables& o) {
    o = LoadTables();
    o.ld_ptr.assign(m.ntotal + 1, 0);
    o.sm_ptr.assign(m.ntotal + 1, 0);
    if (!L) return SVL_OK;
    if (L->nseries > 0) {
        if (!L->series_ptr || !L->series_val) { set_error("series arrays are NULL"); return SVL_ERR_INVALID; }
        o.s_ptr.assign(L->series_ptr, L->series_ptr + L->nseries + 1);
        if (o.s_ptr[0] != 0) { set_error("series_ptr[0] must be 0"); return SVL_ERR_INVALID; }
        for (int s = 0; s < L->nseries; ++s)
            if (o.s_ptr[s + 1] < o.s_ptr[s]) { set_error("series_ptr is not monotone"); return SVL_ERR_INVALID; }
        o.s_val.assign(L->series_val, L->series_val + o.s_ptr.back());
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
    int st = csr(L->nforce, L->force_dof, L->force_series, L->force_coef, o.ld_ptr, o.ld_ser, o.ld_coef);
    if (st) return st;
    st = csr(L->nsupport, L->sm_dof, L->sm_series, L->sm_factor, o.sm_ptr, o.sm_ser, o.sm_fac);
    if (st) return st;
    o.has_sm = L->nsupport > 0;
    return SVL_OK;
}

void build_total_to_free(const HostModel& m, std::vector<int32_t>& ptr,
                         std::vector<int32_t>& col, std::vector<double>& val) {
    // rows of T as CSR: the identity entry of a free dof, then the masters of
    // a constrained one in constraint order; each row sorted by column (a
    // stable sort) with repeated columns summed
    const int nt = m.ntotal;
    std::vector<int64_t> start(nt + 1, 0);
    for (int n = 0; n < m.nnode; ++n)
        for (int j = 0; j < m.nndof[n]; ++j)
            if (m.fdof_all[(size_t)n * m.dstride + j] > -1) ++start[m.tdof_all[(size_t)n * m.dstride + j] + 1];
    for (int c = 0; c < m.nconstraint; ++c) start[m.cslave[c] + 1] += m.cptr[c + 1] - m.cptr[c];
    for (int t = 0; t < nt; ++t) start[t + 1] += start[t];
    std::vector<std::pair<int32_t, double>> ent((size_t)start[nt]);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int n = 0; n < m.nnode; ++n)
        for (int j = 0; j < m.nndof[n]; ++j) {
            const int32_t f = m.fdof_all[(size_t)n * m.dstride + j];
            if (f > -1) ent[(size_t)fill[m.tdof_all[(size_t)n * m.dstride + j]]++] = {f, 1.0};
        }
    for (int c = 0; c < m.nconstraint; ++c)
        for (int i = m.cptr[c]; i < m.cptr[c + 1]; ++i) ent[(size_t)fill[m.cslave[c]]++] = {m.cmaster[i], m.cfactor[i]};
    ptr.assign(nt + 1, 0);
    col.clear(); val.clear();
    col.reserve(ent.size()); val.reserve(ent.size());
    for (int t = 0; t < nt; ++t) {
        auto b = ent.begin() + start[t], e = ent.begin() + start[t + 1];
        if (e - b > 1)
            std::stable_sort(b, e, [](const std::pair<int32_t, double>& x, const std::pair<int32_t, double>& y) {
                return x.first < y.first;
            });
        for (auto it = b; it != e; ++it) {
            if ((int)col.size() > ptr[t] && col.back() == it->first) val.back() += it->second;
            else { col.push_back(it->first); val.push_back(it->second); }
        }
        ptr[t + 1] = (int32_t)col.size();
    }
}

// ---- explicit central difference with PML layers: host tables -------------
// Row-sum lumped N N blocks of the PML element matrices M, C, K, G
// (PML2DQuad4.cpp:233-470, PML3DHexa8.cpp:214-712: each block is a
// stretching combination s times rho N N on the displacement dofs and times
// -compliance N N on the stress dofs, so its row sum at node j is the Gauss
// sum of s N_j w |J|), the solid elements' lumped mass with the mass
// tolerance (and mass-proportional Rayleigh), the nodal masses, 1/(T^T d T)
// on the displacement free dofs and per PML node the inverse of
// Ms/dt^2 + Cs/2dt.  Element order throughout.
int explicit_pml_tables(const HostModel& m, double dt, double mtol, const LoadTables& lt, ExplicitPmlTables& out) {
    const int nd = m.ndim, nen = m.nen, pnd = m.pml_ndof(), ns = pnd - nd, npar = 3 + 2 * nd;
    const int nt = m.ntotal;
    std::vector<int8_t> sdof(nt, 0);
    std::vector<int32_t> snode_of(m.nnode, -1), sfirst;
    std::vector<char> pnode(m.nnode, 0);
    std::vector<int> sol, pml;
    for (int e = 0; e < m.nelem; ++e) ((m.has_pml() && m.epml[e]) ? pml : sol).push_back(e);
    for (int e : pml)
        for (int a = 0; a < nen; ++a) pnode[m.conn[(size_t)e * nen + a]] = 1;
    for (int n = 0; n < m.nnode; ++n) {
        if (!pnode[n]) continue;
        const int t0 = m.tdof_all[(size_t)n * m.dstride + nd];
        for (int j = 0; j < ns; ++j) {
            const int t = m.tdof_all[(size_t)n * m.dstride + nd + j];
            if (t != t0 + j) { set_error("explicit PML: the stress dofs of node %d are not consecutive", n); return SVL_ERR_UNSUPPORTED; }
            if (m.fdof_all[(size_t)n * m.dstride + nd + j] < 0) {
                set_error("explicit PML: node %d has a restrained or constrained stress dof", n); return SVL_ERR_UNSUPPORTED;
            }
            sdof[t] = 1;
        }
        snode_of[n] = (int32_t)sfirst.size();
        sfirst.push_back(t0);
    }
    for (int t = 0; t < nt; ++t)
        if (sdof[t] && lt.sm_ptr[t + 1] > lt.sm_ptr[t]) {
            set_error("explicit PML: support motion on a stress dof (total dof %d)", t); return SVL_ERR_UNSUPPORTED;
        }
    const int nsn = (int)sfirst.size();
    const size_t nb = (size_t)ns * ns;
    std::vector<double> Mu(nt, 0.0), Cu(nt, 0.0), Ku(nt, 0.0), Gu(nt, 0.0);
    std::vector<double> Bl[4];
    for (auto& v : Bl) v.assign((size_t)nsn * nb, 0.0);
    std::vector<int> sidx_of(m.nelem, -1), pidx_of(m.nelem, -1);
    for (size_t i = 0; i < sol.size(); ++i) sidx_of[sol[i]] = (int)i;
    for (size_t i = 0; i < pml.size(); ++i) pidx_of[pml[i]] = (int)i;
    const std::vector<double>& ml = lumped_element_ref(m);   // [(e nen + a) nd + j]
    // per PML element, matrix w and node j the Gauss sum g = sum_q s_w N_j w|J|
    // (every entry of the node's lumped blocks is g times a material constant),
    // in parallel; assembled below in element order
    std::vector<double> gs((size_t)pml.size() * 4 * nen, 0.0);
    parallel_for((int64_t)pml.size(), [&](int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) {
            const int e = pml[i];
            const double* pr = m.param(e);
            const double E = pr[0], nu = pr[1], rho = pr[2];
            const double mu = E / 2.0 / (1 + nu), lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
            const double* par = &m.pml_par[(size_t)e * npar];
            const double pm = par[0], L = par[1], R = par[2];
            const double Vp = std::sqrt((lambda + 2.0 * mu) / rho);
            const double a0 = (pm + 1.0) * (L / 10.0) / 2.0 / L * std::log(1.0 / R);
            const double b0 = (pm + 1.0) * Vp / 2.0 / L * std::log(1.0 / R);
            double* g = &gs[(size_t)i * 4 * nen];
            for (int q = 0; q < m.ngp; ++q) {
                double dNx[8][3], N[8];
                const double det = gp_geometry(m, e, q, dNx, N);
                const double f = gp_factor(m, e, det);
                double xg[3] = {0, 0, 0};
                for (int a = 0; a < nen; ++a)
                    for (int k = 0; k < nd; ++k) xg[k] += N[a] * m.X[(size_t)m.conn[(size_t)e * nen + a] * nd + k];
                double as[3] = {1, 1, 1}, bs[3] = {0, 0, 0};
                for (int k = 0; k < nd; ++k) {
                    const double r = std::pow((xg[k] - par[3 + k]) * par[3 + nd + k] / L, pm);
                    as[k] = 1.0 + a0 * r;
                    bs[k] = b0 * r;
                }
                double sc[4];
                if (nd == 2) {
                    sc[0] = as[0] * as[1]; sc[1] = as[0] * bs[1] + as[1] * bs[0]; sc[2] = bs[0] * bs[1]; sc[3] = 0.0;
                } else {
                    sc[0] = as[0] * as[1] * as[2];
                    sc[1] = as[0] * as[1] * bs[2] + as[0] * bs[1] * as[2] + bs[0] * as[1] * as[2];
                    sc[2] = as[0] * bs[1] * bs[2] + bs[0] * bs[1] * as[2] + bs[0] * as[1] * bs[2];
                    sc[3] = bs[0] * bs[1] * bs[2];
                }
                for (int w = 0; w < 4; ++w)
                    for (int j = 0; j < nen; ++j) g[w * nen + j] += sc[w] * (N[j] * f);
            }
        }
    });
    for (int e = 0; e < m.nelem; ++e) {
        if (sidx_of[e] >= 0) {
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e];
            for (int a = 0; a < nen; ++a)
                for (int j = 0; j < nd; ++j) {
                    const double v = ml[((size_t)e * nen + a) * nd + j];
                    const int t = m.tdof_all[(size_t)m.conn[(size_t)e * nen + a] * m.dstride + j];
                    if (std::fabs(v) > mtol) Mu[t] += v;
                    if (am != 0.0 && std::fabs(am * v) > 1e-12) Cu[t] += am * v;
                }
            continue;
        }
        const double* pr = m.param(e);
        const double E = pr[0], nu = pr[1], rho = pr[2];
        const double mu = E / 2.0 / (1 + nu), lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
        const double* g = &gs[(size_t)pidx_of[e] * 4 * nen];
        std::vector<double>* du[4] = {&Mu, &Cu, &Ku, &Gu};
        for (int w = 0; w < 4; ++w)
            for (int j = 0; j < nen; ++j) {
                const double gw = g[w * nen + j];
                if (gw == 0.0) continue;
                const int n = m.conn[(size_t)e * nen + j];
                for (int c = 0; c < nd; ++c) (*du[w])[m.tdof_all[(size_t)n * m.dstride + c]] += rho * gw;
                double* B = &Bl[w][(size_t)snode_of[n] * nb];
                if (nd == 2) {
                    const double k2 = (lambda + 2.0 * mu) / 4.0 / mu / (lambda + mu);
                    const double l2 = lambda / 4.0 / mu / (lambda + mu);
                    B[0 * 3 + 0] += -k2 * gw; B[1 * 3 + 1] += -k2 * gw;
                    B[0 * 3 + 1] += l2 * gw; B[1 * 3 + 0] += l2 * gw;
                    B[2 * 3 + 2] += -gw / mu;
                } else {
                    const double kap = (lambda + mu) / mu / (3.0 * lambda + 2.0 * mu);
                    const double lam = lambda / 2.0 / mu / (3.0 * lambda + 2.0 * mu);
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) B[r * 6 + c] += (r == c ? -kap : lam) * gw;
                    for (int r = 3; r < 6; ++r) B[r * 6 + r] += -gw / mu;
                }
            }
    }
    if (!m.nodemass.empty())
        for (int t = 0; t < nt; ++t) if (std::fabs(m.nodemass[t]) > mtol) Mu[t] += m.nodemass[t];
    std::vector<int32_t> Tp, Tc;
    std::vector<double> Tv;
    build_total_to_free(m, Tp, Tc, Tv);
    // T^T (Mu/dt^2 + Cu/2dt) T: diagonal when every constrained displacement
    // dof has one master (the EQUAL ties of mergeDomain)
    std::vector<double> kf(std::max(m.nfree, 1), 0.0), kinv(std::max(m.nfree, 1), 0.0);
    std::vector<char> sfree(std::max(m.nfree, 1), 0);
    for (int t = 0; t < nt; ++t) {
        if (sdof[t]) { for (int i = Tp[t]; i < Tp[t + 1]; ++i) sfree[Tc[i]] = 1; continue; }
        if (Tp[t + 1] - Tp[t] > 1) {
            set_error("explicit PML: total dof %d is constrained to more than one master (no diagonal solve)", t);
            return SVL_ERR_UNSUPPORTED;
        }
        const double d = 1.0 / dt / dt * Mu[t] + 1.0 / 2.0 / dt * Cu[t];
        for (int i = Tp[t]; i < Tp[t + 1]; ++i) kf[Tc[i]] += Tv[i] * d * Tv[i];
    }
    for (int f = 0; f < m.nfree; ++f) {
        if (sfree[f]) continue;
        if (!(kf[f] > 0.0)) { set_error("explicit PML: free displacement dof %d has no mass", f); return SVL_ERR_INVALID; }
        kinv[f] = 1.0 / kf[f];
    }
    std::vector<double> Dinv((size_t)nsn * nb, 0.0);
    for (int i = 0; i < nsn; ++i) {
        double A_[36], B[36];
        for (size_t k = 0; k < nb; ++k) { A_[k] = Bl[0][(size_t)i * nb + k] / dt / dt + Bl[1][(size_t)i * nb + k] / 2.0 / dt; B[k] = 0.0; }
        for (int r = 0; r < ns; ++r) B[r * ns + r] = 1.0;
        for (int c = 0; c < ns; ++c) {                   // Gauss-Jordan, partial pivoting
            int pv = c;
            for (int r = c + 1; r < ns; ++r) if (std::fabs(A_[r * ns + c]) > std::fabs(A_[pv * ns + c])) pv = r;
            if (!(std::fabs(A_[pv * ns + c]) > 0.0)) { set_error("explicit PML: singular stress block at PML node %d", i); return SVL_ERR_INVALID; }
            if (pv != c) for (int j = 0; j < ns; ++j) { std::swap(A_[pv * ns + j], A_[c * ns + j]); std::swap(B[pv * ns + j], B[c * ns + j]); }
            const double piv = A_[c * ns + c];
            for (int j = 0; j < ns; ++j) { A_[c * ns + j] /= piv; B[c * ns + j] /= piv; }
            for (int r = 0; r < ns; ++r) {
                if (r == c) continue;
                const double fr = A_[r * ns + c];
                if (fr == 0.0) continue;
                for (int j = 0; j < ns; ++j) { A_[r * ns + j] -= fr * A_[c * ns + j]; B[r * ns + j] -= fr * B[c * ns + j]; }
            }
        }
        for (size_t k = 0; k < nb; ++k) Dinv[(size_t)i * nb + k] = B[k];
    }
    out.sdof = std::move(sdof);
    out.sfirst = std::move(sfirst);
    out.snode_of = std::move(snode_of);
    out.Mu = std::move(Mu); out.Cu = std::move(Cu); out.Ku = std::move(Ku); out.Gu = std::move(Gu);
    out.Ms = std::move(Bl[0]); out.Cs = std::move(Bl[1]); out.Ks = std::move(Bl[2]); out.Gs = std::move(Bl[3]);
    out.Dinv = std::move(Dinv);
    out.kinv = std::move(kinv);
    out.ns = ns;
    return SVL_OK;
}

}  // namespace svl

using namespace svl;

extern "C" {

const char* svl_version(void) { return "svl_gb300 0.1.0 (sm_103a)"; }
const char* svl_last_error(void) { return g_err; }

/* ---- structured grid ---------------------------------------------------- */

static bool grid_check(const svl_grid_spec* s) {
    if (!s) { set_error("grid spec is NULL"); return false; }
    if (s->ndim != 2 && s->ndim != 3) { set_error("grid ndim must be 2 or 3"); return false; }
    for (int i = 0; i < s->ndim; ++i)
        if (s->ne[i] <= 0) { set_error("grid ne[%d] must be positive", i); return false; }
    double nn = 1.0;
    for (int i = 0; i < s->ndim; ++i) nn *= (s->ne[i] + 1.0);
    if (nn * s->ndim > 2.0e9) { set_error("grid too large for 32-bit dof numbers"); return false; }
    return true;
}

int svl_grid_sizes(const svl_grid_spec* s, int32_t* nnode, int32_t* nelem, int32_t* ntotal, int32_t* nfree, int32_t* ncon) {
    if (!grid_check(s)) return SVL_ERR_INVALID;
    const int nd = s->ndim;
    const int nx = s->ne[0], ny = s->ne[1], nz = nd == 3 ? s->ne[2] : 0;
    const int64_t nn = (int64_t)(nx + 1) * (ny + 1) * (nd == 3 ? nz + 1 : 1);
    const int64_t ne = (int64_t)nx * ny * (nd == 3 ? nz : 1);
    // count restrained / constrained dofs by building the masks
    int64_t nr = 0, nc = 0;
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n % (nx + 1));
        const int j = (int)((n / (nx + 1)) % (ny + 1));
        const int k = nd == 3 ? (int)(n / ((int64_t)(nx + 1) * (ny + 1))) : 0;
        int mask = 0;
        if (i == 0) mask |= s->fix_mask[0];
        if (i == nx) mask |= s->fix_mask[1];
        if (j == 0) mask |= s->fix_mask[2];
        if (j == ny) mask |= s->fix_mask[3];
        if (nd == 3 && k == 0) mask |= s->fix_mask[4];
        if (nd == 3 && k == nz) mask |= s->fix_mask[5];
        for (int d = 0; d < nd; ++d) {
            if (mask & (1 << d)) ++nr;
            else if (s->periodic_x && i == nx) ++nc;
        }
    }
    if (nnode) *nnode = (int32_t)nn;
    if (nelem) *nelem = (int32_t)ne;
    if (ntotal) *ntotal = (int32_t)(nn * nd);
    if (nfree) *nfree = (int32_t)(nn * nd - nr - nc);
    if (ncon) *ncon = (int32_t)nc;
    return SVL_OK;
}

int svl_grid_build(const svl_grid_spec* s, double* coords, int32_t* totaldof, int32_t* freedof,
                   int32_t* conn, int32_t* con_slave, int32_t* con_ptr, int32_t* con_master, double* con_factor) {
    if (!grid_check(s)) return SVL_ERR_INVALID;
    if (!coords || !totaldof || !freedof || !conn) { set_error("grid output array is NULL"); return SVL_ERR_INVALID; }
    const int nd = s->ndim;
    const int nx = s->ne[0], ny = s->ne[1], nz = nd == 3 ? s->ne[2] : 0;
    const int64_t nn = (int64_t)(nx + 1) * (ny + 1) * (nd == 3 ? nz + 1 : 1);
    const double hx = s->h[0], hy = s->h[1], hz = nd == 3 ? s->h[2] : 0.0;
    // Builder.py: coords = P0 + i*DX + j*DY + k*DZ, node tags x-fastest
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n % (nx + 1));
        const int j = (int)((n / (nx + 1)) % (ny + 1));
        const int k = nd == 3 ? (int)(n / ((int64_t)(nx + 1) * (ny + 1))) : 0;
        coords[n * nd + 0] = s->origin[0] + i * hx;
        coords[n * nd + 1] = s->origin[1] + j * hy;
        if (nd == 3) coords[n * nd + 2] = s->origin[2] + k * hz;
    }
    // Restraints mark freedof = -1, periodic x-max dofs get constraint tags
    // -2, -3, ... in ascending node order (dof-minor); PlainScheme then
    // numbers total dofs consecutively and free dofs over the unmarked ones
    // (Numberer.py:185-233).
    int32_t ncount = 0, tcount = 0, fcount = 0;
    std::vector<int64_t> slave_nodes; std::vector<int> slave_dofs;
    for (int64_t n = 0; n < nn; ++n) {
        const int i = (int)(n % (nx + 1));
        const int j = (int)((n / (nx + 1)) % (ny + 1));
        const int k = nd == 3 ? (int)(n / ((int64_t)(nx + 1) * (ny + 1))) : 0;
        int mask = 0;
        if (i == 0) mask |= s->fix_mask[0];
        if (i == nx) mask |= s->fix_mask[1];
        if (j == 0) mask |= s->fix_mask[2];
        if (j == ny) mask |= s->fix_mask[3];
        if (nd == 3 && k == 0) mask |= s->fix_mask[4];
        if (nd == 3 && k == nz) mask |= s->fix_mask[5];
        for (int d = 0; d < nd; ++d) {
            totaldof[n * nd + d] = tcount++;
            if (mask & (1 << d)) freedof[n * nd + d] = -1;
            else if (s->periodic_x && i == nx) {
                freedof[n * nd + d] = -2 - ncount;
                slave_nodes.push_back(n); slave_dofs.push_back(d);
                ++ncount;
            } else freedof[n * nd + d] = fcount++;
        }
    }
    if (ncount > 0) {
        if (!con_slave || !con_ptr || !con_master || !con_factor) { set_error("constraint output arrays are NULL"); return SVL_ERR_INVALID; }
        con_ptr[0] = 0;
        for (int c = 0; c < ncount; ++c) {
            const int64_t n = slave_nodes[c];
            const int d = slave_dofs[c];
            const int64_t master = n - nx;   // same row, i = 0
            con_slave[c] = totaldof[n * nd + d];
            con_master[c] = freedof[master * nd + d];
            con_factor[c] = 1.0;
            con_ptr[c + 1] = c + 1;
            if (con_master[c] < 0) { set_error("periodic master dof of node %lld is not free", (long long)master); return SVL_ERR_INVALID; }
        }
    }
    // connectivity (Builder.py:167-183 for Hexa8; Quad4 analogous)
    int64_t e = 0;
    if (nd == 2) {
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i, ++e) {
                const int32_t n1 = j * (nx + 1) + i;
                conn[e * 4 + 0] = n1;
                conn[e * 4 + 1] = n1 + 1;
                conn[e * 4 + 2] = n1 + 1 + (nx + 1);
                conn[e * 4 + 3] = n1 + (nx + 1);
            }
    } else {
        const int64_t layer = (int64_t)(nx + 1) * (ny + 1);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i, ++e) {
                    const int64_t n1 = layer * k + (int64_t)j * (nx + 1) + i;
                    conn[e * 8 + 0] = (int32_t)n1;
                    conn[e * 8 + 1] = (int32_t)(n1 + 1);
                    conn[e * 8 + 2] = (int32_t)(n1 + 1 + (nx + 1));
                    conn[e * 8 + 3] = (int32_t)(n1 + (nx + 1));
                    conn[e * 8 + 4] = (int32_t)(n1 + layer);
                    conn[e * 8 + 5] = (int32_t)(n1 + layer + 1);
                    conn[e * 8 + 6] = (int32_t)(n1 + layer + 1 + (nx + 1));
                    conn[e * 8 + 7] = (int32_t)(n1 + layer + (nx + 1));
                }
    }
    return SVL_OK;
}

int svl_element_body_force(const svl_model_desc* d, int32_t elem, const double* q, double* fe) {
    HostModel m;
    if (!model_from_desc(d, m)) return SVL_ERR_INVALID;
    if (elem < 0 || elem >= m.nelem || !q || !fe) { set_error("bad element index or NULL array"); return SVL_ERR_INVALID; }
    const int nd = m.ndim, nen = m.nen;
    for (int i = 0; i < nen * nd; ++i) fe[i] = 0.0;
    const double rho = m.param(elem)[2];
    for (int g = 0; g < m.ngp; ++g) {
        double dNx[8][3], N[8];
        const double det = gp_geometry(m, elem, g, dNx, N);
        const double c = nd == 2 ? 1.0 * rho * m.thick[elem] * std::fabs(det) : 1.0 * rho * std::fabs(det);
        for (int a = 0; a < nen; ++a)
            for (int j = 0; j < nd; ++j) fe[a * nd + j] += c * (N[a] * q[j]);
    }
    return SVL_OK;
}

int svl_lumped_mass(const svl_model_desc* d, double mtol, double* mass_total) {
    HostModel m;
    if (!model_from_desc(d, m)) return SVL_ERR_INVALID;
    if (!mass_total) { set_error("output is NULL"); return SVL_ERR_INVALID; }
    std::vector<double> M;
    lumped_mass_diag(m, mtol, M);
    std::memcpy(mass_total, M.data(), sizeof(double) * M.size());
    return SVL_OK;
}

}  // extern "C"
