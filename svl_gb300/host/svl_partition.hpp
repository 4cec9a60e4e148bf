// Partition-file reader for C++ hosts: the pre-processor's per-process JSON
// (`<run dir>/Partition/<name>.<combo>.<rank>.json`, PP/Core/SeismoVLAB.py
// createPartitions) mapped onto svl_model_desc / svl_load_desc, as the
// run-process parses it (RP/12-Utilities/Driver.hpp UpdateMesh,
// UpdateMaterials, UpdateLoads, UpdateSupportMotion, UpdateConstraints,
// 392-1722, and the simulation block, 1760-1840).  A C++ maintainer replaces
// the Mesh built by Driver.hpp:1981-2045 with
//
//   svl::gpu::Partition part = svl::gpu::load_partition(path);
//   svl_model_desc md = part.model();
//   svl_load_desc  ld = part.loads();
//
// and hands md / ld to the integrators of svl_integrators.hpp.  The arrays are
// owned by the Partition; the descriptors point into it and live as long as it
// does.  Covered (as the library's Python reader): lin2DQuad4 / lin3DHexa8
// with PML2DQuad4 / PML3DHexa8 layers (5 / 9-dof nodes); Elastic2DPlaneStrain,
// Elastic3DLinear, PlasticPlaneStrainJ2, Plastic3DJ2; restraints; EQUAL-type
// constraints; nodal masses; Free / Rayleigh dampings; ZeroLength1D elements
// with a Viscous1DLinear material (Lysmer dashpots); point loads (concentrated
// and body), element body loads and domain-reduction loads; constant and
// time-series functions; support motions; node and element recorders.  Anything else
// throws svl::gpu::Error with SVL_ERR_UNSUPPORTED naming it.
#pragma once

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "svl_integrators.hpp"

namespace svl {
namespace gpu {

// ---- a small JSON reader (objects, arrays, strings, numbers, literals) ----
class Json {
public:
    enum Kind { Null, Bool, Number, String, Array, Object };
    Kind kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;
    std::vector<std::string> keys;     // object keys in file order

    static Json parse(const std::string& text) {
        size_t i = 0;
        Json j = value(text, i);
        skip(text, i);
        if (i != text.size()) fail(text, i, "trailing characters");
        return j;
    }
    bool has(const std::string& k) const { return kind == Object && obj.count(k) != 0; }
    const Json& at(const std::string& k) const {
        auto it = obj.find(k);
        if (kind != Object || it == obj.end()) throw Error(SVL_ERR_INVALID, "partition file: missing key \"" + k + "\"");
        return it->second;
    }
    double number() const {
        if (kind == Number) return num;
        if (kind == String) return std::strtod(str.c_str(), nullptr);      // numbers written as strings
        throw Error(SVL_ERR_INVALID, "partition file: a number was expected");
    }
    double number(const std::string& k, double dflt) const { return has(k) ? at(k).number() : dflt; }
    std::string text() const {
        if (kind == String) return str;
        if (kind == Number) {
            if (num == std::floor(num) && std::fabs(num) < 1e15) return std::to_string((long long)num);
            std::ostringstream s;
            s.precision(17);
            s << num;
            return s.str();
        }
        throw Error(SVL_ERR_INVALID, "partition file: a string was expected");
    }
    std::string text(const std::string& k, const std::string& dflt) const { return has(k) ? at(k).text() : dflt; }
    const std::vector<Json>& list() const {
        if (kind != Array) throw Error(SVL_ERR_INVALID, "partition file: a list was expected");
        return arr;
    }

private:
    [[noreturn]] static void fail(const std::string&, size_t i, const char* what) {
        throw Error(SVL_ERR_INVALID, std::string("partition file: JSON ") + what + " at offset " + std::to_string(i));
    }
    static void skip(const std::string& t, size_t& i) {
        while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
    }
    static std::string string_at(const std::string& t, size_t& i) {
        std::string out;
        ++i;                                                   // opening quote
        while (i < t.size() && t[i] != '"') {
            char c = t[i++];
            if (c == '\\') {
                if (i >= t.size()) fail(t, i, "bad escape");
                const char e = t[i++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (i + 4 > t.size()) fail(t, i, "bad escape");
                        const unsigned cp = (unsigned)std::strtoul(t.substr(i, 4).c_str(), nullptr, 16);
                        i += 4;
                        if (cp < 0x80) out += (char)cp;                        // names and paths are ASCII
                        else out += '?';
                        break;
                    }
                    default: out += e;                                  // \" \\ \/
                }
            } else {
                out += c;
            }
        }
        if (i >= t.size()) fail(t, i, "unterminated string");
        ++i;
        return out;
    }
    static Json value(const std::string& t, size_t& i) {
        skip(t, i);
        if (i >= t.size()) fail(t, i, "unexpected end");
        Json j;
        const char c = t[i];
        if (c == '{') {
            j.kind = Object;
            ++i;
            skip(t, i);
            if (i < t.size() && t[i] == '}') { ++i; return j; }
            for (;;) {
                skip(t, i);
                if (i >= t.size() || t[i] != '"') fail(t, i, "object key expected");
                std::string k = string_at(t, i);
                skip(t, i);
                if (i >= t.size() || t[i] != ':') fail(t, i, "':' expected");
                ++i;
                if (!j.obj.count(k)) j.keys.push_back(k);
                j.obj[k] = value(t, i);
                skip(t, i);
                if (i < t.size() && t[i] == ',') { ++i; continue; }
                if (i < t.size() && t[i] == '}') { ++i; return j; }
                fail(t, i, "',' or '}' expected");
            }
        }
        if (c == '[') {
            j.kind = Array;
            ++i;
            skip(t, i);
            if (i < t.size() && t[i] == ']') { ++i; return j; }
            for (;;) {
                j.arr.push_back(value(t, i));
                skip(t, i);
                if (i < t.size() && t[i] == ',') { ++i; continue; }
                if (i < t.size() && t[i] == ']') { ++i; return j; }
                fail(t, i, "',' or ']' expected");
            }
        }
        if (c == '"') {
            j.kind = String;
            j.str = string_at(t, i);
            return j;
        }
        if (t.compare(i, 4, "true") == 0) { j.kind = Bool; j.b = true; i += 4; return j; }
        if (t.compare(i, 5, "false") == 0) { j.kind = Bool; i += 5; return j; }
        if (t.compare(i, 4, "null") == 0) { i += 4; return j; }
        const char* s = t.c_str() + i;
        char* end = nullptr;
        j.num = std::strtod(s, &end);
        if (end == s) fail(t, i, "value expected");
        j.kind = Number;
        i += (size_t)(end - s);
        return j;
    }
};

inline std::string upper(std::string s) {
    for (char& c : s) c = (char)std::toupper((unsigned char)c);
    return s;
}

inline std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(SVL_ERR_INVALID, "cannot open " + path);
    std::ostringstream s;
    s << f.rdbuf();
    return s.str();
}

// Time-series file: the number of values, then the values (Driver.hpp:1514-1527).
inline std::vector<double> read_series(const std::string& path) {
    std::istringstream s(read_file(path));
    double n = 0;
    if (!(s >> n)) throw Error(SVL_ERR_INVALID, path + ": empty time series");
    std::vector<double> v((size_t)n);
    for (double& x : v)
        if (!(s >> x)) throw Error(SVL_ERR_INVALID, path + ": fewer values than announced");
    return v;
}

// Keys of a JSON object that are integer tags, in ascending numeric order
// (the run-process keeps nodes, elements and loads in std::map order).
inline std::vector<int> sorted_tags(const Json& o) {
    std::vector<int> t;
    if (o.kind != Json::Object) return t;
    for (const auto& kv : o.obj) t.push_back(std::atoi(kv.first.c_str()));
    std::sort(t.begin(), t.end());
    return t;
}

struct NodeRecorder {
    std::string name = "NODE";         // NODE or ELEMENT
    std::string file, response;        // NODE: DISP, VEL, ACCEL, REACTION; ELEMENT: STRESS, STRAIN, INTERNALFORCE, STRAINRATE
    std::vector<int> ids;              // node or element tags
    int precision = 8;
    int nsamp = 1;
};

class Partition {
public:
    // model arrays (svl_model_desc)
    int ndim = 0, nnode = 0, stride = 0, ntotal = 0, nfree = 0, elem_type = 0, nelem = 0, nmat = 0;
    bool lumped = false;
    std::vector<double> coords, mat_param, thickness, node_mass, rayleigh, pml_param, dashpot_eta, con_factor;
    std::vector<int32_t> totaldof, freedof, node_ndof, conn, elem_mat, mat_type, elem_pml, dashpot_dof, con_slave,
        con_ptr, con_master;
    // load arrays (svl_load_desc)
    std::vector<int32_t> series_ptr{0}, force_dof, force_series, sm_dof, sm_series, drm_elem, drm_node_row, drm_node_ext;
    std::vector<double> series_val, force_coef, sm_factor, drm_factor, drm_motion;
    int drm_nt = 0;
    // simulation block
    std::string integrator, algorithm = "LINEAR", solver, combo_folder;
    double dt = 0, ftol = 1e-12, mtol = 1e-12, ktol = 1e-12, solver_tol = 1e-12, cnvgtol = 1e-6;
    int nt = 0, nstep = 50, cnvgtest = 4;
    std::vector<int> node_tags, elem_tags;
    std::vector<NodeRecorder> recorders;

    bool has_pml() const { return std::any_of(elem_pml.begin(), elem_pml.end(), [](int32_t v) { return v != 0; }); }

    svl_model_desc model() const {
        svl_model_desc d{};
        d.ndim = ndim;
        d.nnode = nnode;
        d.ndof = stride;
        d.coords = coords.data();
        d.totaldof = totaldof.data();
        d.freedof = freedof.data();
        d.ntotal = ntotal;
        d.nfree = nfree;
        d.nconstraint = (int32_t)con_slave.size();
        d.con_slave = con_slave.empty() ? nullptr : con_slave.data();
        d.con_ptr = con_slave.empty() ? nullptr : con_ptr.data();
        d.con_master = con_slave.empty() ? nullptr : con_master.data();
        d.con_factor = con_slave.empty() ? nullptr : con_factor.data();
        d.elem_type = elem_type;
        d.nelem = nelem;
        d.conn = conn.data();
        d.elem_mat = elem_mat.data();
        d.elem_thickness = thickness.empty() ? nullptr : thickness.data();
        d.nmat = nmat;
        d.mat_type = mat_type.data();
        d.mat_param = mat_param.data();
        d.lumped = lumped ? 1 : 0;
        d.node_mass = node_mass.empty() ? nullptr : node_mass.data();
        d.elem_rayleigh = rayleigh.empty() ? nullptr : rayleigh.data();
        const bool pml = has_pml();
        d.node_ndof = stride != ndim ? node_ndof.data() : nullptr;
        d.elem_pml = pml ? elem_pml.data() : nullptr;
        d.elem_pml_param = pml ? pml_param.data() : nullptr;
        d.ndashpot = (int32_t)dashpot_eta.size();
        d.dashpot_dof = dashpot_eta.empty() ? nullptr : dashpot_dof.data();
        d.dashpot_eta = dashpot_eta.empty() ? nullptr : dashpot_eta.data();
        return d;
    }

    svl_load_desc loads() const {
        svl_load_desc d{};
        d.nseries = (int32_t)series_ptr.size() - 1;
        d.series_ptr = series_ptr.data();
        d.series_val = series_val.empty() ? nullptr : series_val.data();
        d.nforce = (int32_t)force_dof.size();
        d.force_dof = force_dof.data();
        d.force_series = force_series.data();
        d.force_coef = force_coef.data();
        d.nsupport = (int32_t)sm_dof.size();
        d.sm_dof = sm_dof.data();
        d.sm_series = sm_series.data();
        d.sm_factor = sm_factor.data();
        d.ndrm = (int32_t)drm_elem.size();
        if (d.ndrm) {
            d.drm_elem = drm_elem.data();
            d.drm_factor = drm_factor.data();
            d.drm_nt = drm_nt;
            d.drm_node_row = drm_node_row.data();
            d.drm_node_ext = drm_node_ext.data();
            d.drm_motion = drm_motion.data();
        }
        return d;
    }

    int add_series(std::vector<double> v) {
        series_val.insert(series_val.end(), v.begin(), v.end());
        series_ptr.push_back((int32_t)series_val.size());
        return (int)series_ptr.size() - 2;
    }
};

namespace detail {

struct MatSpec {
    int type;
    std::vector<const char*> keys;
};

inline const std::map<std::string, MatSpec>& materials() {
    static const std::map<std::string, MatSpec> m = {
        {"ELASTIC2DPLANESTRAIN", {SVL_MAT_ELASTIC2DPLANESTRAIN, {"E", "nu", "rho"}}},
        {"ELASTIC3DLINEAR", {SVL_MAT_ELASTIC3DLINEAR, {"E", "nu", "rho"}}},
        {"PLASTICPLANESTRAINJ2", {SVL_MAT_PLASTICPLANESTRAINJ2, {"K", "G", "rho", "h", "beta", "Sy"}}},
        {"PLASTIC3DJ2", {SVL_MAT_PLASTIC3DJ2, {"K", "G", "rho", "h", "beta", "Sy"}}},
    };
    return m;
}

inline std::string join(const std::string& dir, const std::string& f) {
    if (!f.empty() && f[0] == '/') return f;
    if (dir.empty()) return f;
    return dir + "/" + f;
}

[[noreturn]] inline void unsupported(const std::string& what) { throw Error(SVL_ERR_UNSUPPORTED, what); }

}  // namespace detail

// Parses one partition file.  Time-series and free-field files are looked up
// relative to `run_dir` (default: the folder that holds the Partition folder,
// the run-process's working directory).
inline Partition load_partition(const std::string& path, std::string run_dir = "") {
    using detail::unsupported;
    const Json d = Json::parse(read_file(path));
    if (run_dir.empty()) {
        std::string dir = path.substr(0, path.find_last_of('/') == std::string::npos ? 0 : path.find_last_of('/'));
        const size_t cut = dir.find_last_of('/');
        const std::string last = cut == std::string::npos ? dir : dir.substr(cut + 1);
        run_dir = last == "Partition" ? (cut == std::string::npos ? std::string(".") : dir.substr(0, cut)) : dir;
    }
    Partition P;
    const Json& g = d.at("Global");
    P.ndim = (int)g.at("ndim").number();
    const int ndim = P.ndim, pnd = ndim == 2 ? 5 : 9;
    // nodes in ascending tag order (the run-process's std::map order)
    const Json& N = d.at("Nodes");
    P.node_tags = sorted_tags(N);
    P.nnode = (int)P.node_tags.size();
    std::map<int, int> npos;
    for (int i = 0; i < P.nnode; ++i) npos[P.node_tags[i]] = i;
    P.node_ndof.resize(P.nnode);
    for (int i = 0; i < P.nnode; ++i) {
        const int nd = (int)N.at(std::to_string(P.node_tags[i])).at("ndof").number();
        if (nd != ndim && nd != pnd)
            unsupported("nodes with " + std::to_string(nd) + " dofs: " + std::to_string(ndim) + "-dof displacement nodes and " +
                        std::to_string(pnd) + "-dof PML nodes are covered");
        P.node_ndof[i] = nd;
        P.stride = std::max(P.stride, nd);
    }
    P.coords.resize((size_t)P.nnode * ndim);
    P.totaldof.assign((size_t)P.nnode * P.stride, -1);
    P.freedof.assign((size_t)P.nnode * P.stride, -1);
    for (int i = 0; i < P.nnode; ++i) {
        const Json& n = N.at(std::to_string(P.node_tags[i]));
        const auto& xc = n.at("coords").list();
        for (int c = 0; c < ndim; ++c) P.coords[(size_t)i * ndim + c] = xc.at(c).number();
        const auto& td = n.at("totaldof").list();
        const auto& fd = n.at("freedof").list();
        for (int c = 0; c < P.node_ndof[i]; ++c) {
            P.totaldof[(size_t)i * P.stride + c] = (int32_t)td.at(c).number();
            P.freedof[(size_t)i * P.stride + c] = (int32_t)fd.at(c).number();
        }
    }
    auto tdof = [&](int node, int c) { return P.totaldof[(size_t)node * P.stride + c]; };
    // materials (Viscous1DLinear only as a ZeroLength1D dashpot, Driver.hpp:602-607)
    std::map<int, double> viscous;
    std::vector<int> mtags;
    const Json empty;
    const Json& M = d.has("Materials") ? d.at("Materials") : empty;
    for (int t : sorted_tags(M)) {
        const Json& mt = M.at(std::to_string(t));
        if (upper(mt.at("name").text()) == "VISCOUS1DLINEAR") viscous[t] = mt.at("attributes").number("eta", 0.0);
        else mtags.push_back(t);
    }
    std::map<int, int> mpos;
    P.nmat = (int)mtags.size();
    P.mat_type.resize(P.nmat);
    P.mat_param.assign((size_t)P.nmat * SVL_MAT_NPARAM, 0.0);
    for (int i = 0; i < P.nmat; ++i) {
        const Json& mt = M.at(std::to_string(mtags[i]));
        const std::string name = upper(mt.at("name").text());
        auto it = detail::materials().find(name);
        if (it == detail::materials().end()) unsupported("material " + mt.at("name").text() + " (tag " + std::to_string(mtags[i]) + ") is not covered");
        P.mat_type[i] = it->second.type;
        for (size_t k = 0; k < it->second.keys.size(); ++k)
            P.mat_param[(size_t)i * SVL_MAT_NPARAM + k] = mt.at("attributes").at(it->second.keys[k]).number();
        mpos[mtags[i]] = i;
    }
    // elements in ascending tag order; ZeroLength1D elements with a viscous
    // material become dashpots on their direction `dir` (ZeroLength1D.cpp:210-228)
    const Json& E = d.at("Elements");
    std::vector<int> solid_tags;
    for (int t : sorted_tags(E)) {
        const Json& e = E.at(std::to_string(t));
        if (upper(e.at("name").text()) != "ZEROLENGTH1D") { solid_tags.push_back(t); continue; }
        const int mt = (int)e.at("attributes").at("material").number();
        if (!viscous.count(mt)) unsupported("ZeroLength1D element " + std::to_string(t) + ": only a Viscous1DLinear material (a dashpot) is covered");
        const int j = (int)e.at("attributes").at("dir").number();
        if (j < 0 || j >= ndim) unsupported("ZeroLength1D element " + std::to_string(t) + ": dir out of range");
        const auto& c = e.at("conn").list();
        P.dashpot_dof.push_back(tdof(npos.at((int)c.at(0).number()), j));
        P.dashpot_dof.push_back(tdof(npos.at((int)c.at(1).number()), j));
        P.dashpot_eta.push_back(viscous[mt]);
    }
    P.elem_tags = solid_tags;
    P.nelem = (int)solid_tags.size();
    std::set<std::string> solid;
    for (int t : solid_tags) {
        std::string n = upper(E.at(std::to_string(t)).at("name").text());
        if (n == "PML2DQUAD4") n = "LIN2DQUAD4";
        if (n == "PML3DHEXA8") n = "LIN3DHEXA8";
        solid.insert(n);
    }
    if (solid.size() != 1 || (*solid.begin() != "LIN2DQUAD4" && *solid.begin() != "LIN3DHEXA8"))
        unsupported("element classes: one of LIN2DQUAD4, LIN3DHEXA8 per model (with its PML class) is covered");
    const bool quad = *solid.begin() == "LIN2DQUAD4";
    if ((quad ? 2 : 3) != ndim) unsupported("element dimension does not match Global.ndim");
    P.elem_type = quad ? SVL_ELEM_LIN2DQUAD4 : SVL_ELEM_LIN3DHEXA8;
    const int nen = quad ? 4 : 8, npar = 3 + 2 * ndim;
    P.conn.resize((size_t)P.nelem * nen);
    P.elem_mat.resize(P.nelem);
    P.elem_pml.assign(P.nelem, 0);
    P.pml_param.assign((size_t)P.nelem * npar, 0.0);
    if (ndim == 2) P.thickness.resize(P.nelem);
    std::map<int, int> epos;
    for (int i = 0; i < P.nelem; ++i) {
        const Json& e = E.at(std::to_string(solid_tags[i]));
        epos[solid_tags[i]] = i;
        const auto& c = e.at("conn").list();
        for (int a = 0; a < nen; ++a) P.conn[(size_t)i * nen + a] = npos.at((int)c.at(a).number());
        const Json& at = e.at("attributes");
        P.elem_mat[i] = mpos.at((int)at.at("material").number());
        if (ndim == 2) P.thickness[i] = at.number("th", 1.0);
        const std::string name = upper(e.at("name").text());
        if (name == "PML2DQUAD4" || name == "PML3DHEXA8") {
            // PML parameters (Driver.hpp:1203-1220, 1288-1306): n, L, R, x0, npml
            P.elem_pml[i] = 1;
            double* pp = &P.pml_param[(size_t)i * npar];
            pp[0] = at.at("n").number();
            pp[1] = at.at("L").number();
            pp[2] = at.at("R").number();
            for (int c2 = 0; c2 < ndim; ++c2) {
                pp[3 + c2] = at.at("x0").list().at(c2).number();
                pp[3 + ndim + c2] = at.at("npml").list().at(c2).number();
            }
        }
    }
    // dampings in ascending tag order, each over its element list
    // (Driver.hpp:1365-1405); a later tag overrides an earlier one
    std::vector<double> ray((size_t)P.nelem * 2, 0.0);
    bool any_ray = false;
    const Json& D = d.has("Dampings") ? d.at("Dampings") : empty;
    for (int t : sorted_tags(D)) {
        const Json& dm = D.at(std::to_string(t));
        const std::string name = upper(dm.at("name").text());
        const Json& at = dm.has("attributes") ? dm.at("attributes") : empty;
        double am = 0.0, ak = 0.0;
        if (name == "RAYLEIGH") { am = at.number("am", 0.0); ak = at.number("ak", 0.0); }
        else if (name != "FREE") unsupported("damping " + dm.at("name").text() + " (tag " + std::to_string(t) + ") is not covered");
        if (at.has("list"))
            for (const Json& e : at.at("list").list()) {
                auto it = epos.find((int)e.number());
                if (it == epos.end()) continue;
                ray[(size_t)it->second * 2] = am;
                ray[(size_t)it->second * 2 + 1] = ak;
            }
    }
    for (double v : ray) any_ray = any_ray || v != 0.0;
    if (any_ray) P.rayleigh = ray;
    // nodal masses (Node::GetMass), also the weights of body point loads
    P.ntotal = (int)g.at("ntotal").number();
    P.nfree = (int)g.at("nfree").number();
    std::map<int, std::vector<double>> nmass;
    const Json& MS = d.has("Masses") ? d.at("Masses") : empty;
    if (MS.kind == Json::Object && !MS.obj.empty()) {
        P.node_mass.assign(P.ntotal, 0.0);
        for (const auto& kv : MS.obj) {
            const int i = npos.at(std::atoi(kv.first.c_str()));
            std::vector<double> m;
            for (const Json& v : kv.second.at("mass").list()) m.push_back(v.number());
            for (size_t k = 0; k < m.size(); ++k) P.node_mass[tdof(i, (int)k)] += m[k];
            nmass[i] = m;
        }
    }
    // constraints: slave total dof <- sum factor * master free dof, descending tags
    const Json& CS = d.has("Constraints") ? d.at("Constraints") : empty;
    std::vector<int> ctags = sorted_tags(CS);
    std::reverse(ctags.begin(), ctags.end());
    if (!ctags.empty()) {
        P.con_ptr.assign(1, 0);
        for (int t : ctags) {
            const Json& c = CS.at(std::to_string(t));
            P.con_slave.push_back((int32_t)c.at("stag").number());
            const auto& mt = c.at("mtag").list();
            const auto& fc = c.at("factor").list();
            for (size_t k = 0; k < mt.size(); ++k) {
                P.con_master.push_back((int32_t)mt[k].number());
                P.con_factor.push_back(fc.at(k).number());
            }
            P.con_ptr.push_back((int32_t)P.con_master.size());
        }
    }
    P.lumped = upper(g.text("massform", "CONSISTENT")) == "LUMPED";
    int ntot = 0, nfr = 0;
    for (int i = 0; i < P.nnode; ++i)
        for (int c = 0; c < P.node_ndof[i]; ++c) {
            ntot = std::max(ntot, tdof(i, c) + 1);
            nfr = std::max(nfr, P.freedof[(size_t)i * P.stride + c] + 1);
        }
    if (ntot != P.ntotal || nfr != P.nfree) throw Error(SVL_ERR_INVALID, "Global ntotal/nfree do not match the nodes");
    // simulation block
    const Json& sim = d.at("Simulations");
    const Json& sat = sim.at("attributes");
    const Json& integ = sat.at("integrator");
    P.integrator = upper(integ.at("name").text());
    P.dt = integ.at("dt").number();
    P.ftol = integ.number("ftol", 1e-12);
    P.mtol = integ.number("mtol", 1e-12);
    P.ktol = integ.number("ktol", 1e-12);
    if (upper(sat.at("analysis").at("name").text()) != "DYNAMIC") unsupported("analysis " + sat.at("analysis").at("name").text() + " is not covered");
    P.nt = (int)sat.at("analysis").at("nt").number();
    if (sat.has("algorithm")) {
        const Json& al = sat.at("algorithm");
        P.algorithm = upper(al.text("name", "LINEAR"));
        P.nstep = (int)al.number("nstep", 50);
        P.cnvgtol = al.number("cnvgtol", 1e-6);
        P.cnvgtest = (int)al.number("cnvgtest", 4);
    }
    if (sat.has("solver")) {
        P.solver = upper(sat.at("solver").text("name", ""));
        P.solver_tol = P.solver == "PETSC" ? sat.at("solver").number("tol", 1e-12) : 1e-12;
    }
    const Json& combo = d.at("Combinations").at(sim.at("combo").text());
    P.combo_folder = combo.at("attributes").text("folder", combo.at("name").text());
    const svl_model_desc md = P.model();
    // loads of the combination (Assembler::ComputeExternalForceVector,
    // Assembler.cpp:291-489): every load is assembled by assignment into its
    // own vector, Fext(dof) = Fn (point loads) or Fn Mn (body point loads, Mn
    // the node's Masses entries; nodes without one get nothing), then factor *
    // Fext is added; across loads the entries add, within one load a node
    // listed twice counts once
    const auto& lt = combo.at("attributes").at("load").list();
    const auto& lf = combo.at("attributes").at("factor").list();
    std::map<int, std::pair<int, int>> drm_nodes;            // node position -> (row block, exterior)
    std::vector<double> drm_blocks;
    for (size_t li = 0; li < lt.size(); ++li) {
        const std::string ltag = lt[li].text();
        const double fac = lf.at(li).number();
        const Json& ld = d.at("Loads").at(ltag);
        const Json& la = ld.at("attributes");
        const std::string lname = upper(ld.at("name").text()), kind = upper(la.at("type").text()), fun = upper(la.text("name", ""));
        if (lname == "ELEMENTLOAD" && kind == "GENERALWAVE") {
            // domain reduction: per node of the elements a file `nt nFields cond`
            // then u, v, a per direction per row (Driver.hpp:1669-1722)
            std::set<int> seen;                              // a later load's file replaces an earlier one's
            for (const Json& et : la.at("list").list()) {
                const int e = epos.at((int)et.number());
                P.drm_elem.push_back(e);
                P.drm_factor.push_back(fac);
                for (const Json& nt : E.at(et.text()).at("conn").list()) {
                    const int ntag = (int)nt.number(), n = npos.at(ntag);
                    if (!seen.insert(n).second) continue;
                    std::string f = la.at("file").text();
                    for (size_t dollar = f.find('$'); dollar != std::string::npos; dollar = f.find('$'))
                        f.replace(dollar, 1, std::to_string(ntag));
                    std::istringstream s(read_file(detail::join(run_dir, f)));
                    double rows = 0, nf = 0, cond = 0;
                    s >> rows >> nf >> cond;
                    if ((int)nf != 3 * ndim) throw Error(SVL_ERR_INVALID, f + ": u, v, a per direction expected on every row");
                    if (P.drm_nt == 0) P.drm_nt = (int)rows;
                    if ((int)rows != P.drm_nt) throw Error(SVL_ERR_INVALID, "every DRM node needs the same number of rows");
                    const size_t base = drm_blocks.size();
                    drm_blocks.resize(base + (size_t)rows * (size_t)nf);
                    for (size_t k = 0; k < (size_t)rows * (size_t)nf; ++k)
                        if (!(s >> drm_blocks[base + k])) throw Error(SVL_ERR_INVALID, f + ": fewer values than announced");
                    // (block, exterior flag); blocks are put in node order below
                    drm_nodes[n] = {(int)(base / ((size_t)rows * (size_t)nf)), cond != 0.0 ? 1 : 0};
                }
            }
            continue;
        }
        std::vector<double> series;
        if (fun == "TIMESERIES") series = read_series(detail::join(run_dir, la.at("file").text()));
        else if (fun == "CONSTANT") series.assign(std::max(P.nt, 1), la.at("mag").number());   // every step
        else unsupported("load function " + la.text("name", "?") + " is not covered");
        const int s = P.add_series(series);
        std::vector<double> dir;
        for (const Json& v : la.at("dir").list()) dir.push_back(v.number());
        std::vector<int> nodes;
        if (la.has("list"))
            for (const Json& v : la.at("list").list()) {
                const int t = (int)v.number();
                if (std::find(nodes.begin(), nodes.end(), t) == nodes.end()) nodes.push_back(t);
            }
        if (lname == "POINTLOAD" && kind == "CONCENTRATED") {
            for (int t : nodes) {
                const int i = npos.at(t);
                for (int j = 0; j < P.stride && j < (int)dir.size(); ++j)
                    if (dir[j] != 0.0) {
                        P.force_dof.push_back(tdof(i, j));
                        P.force_series.push_back(s);
                        P.force_coef.push_back(fac * dir[j]);
                    }
            }
        } else if (lname == "POINTLOAD" && kind == "BODY") {
            for (int t : nodes) {
                const int i = npos.at(t);
                auto it = nmass.find(i);
                if (it == nmass.end()) continue;
                for (size_t j = 0; j < dir.size() && j < it->second.size(); ++j) {
                    P.force_dof.push_back(tdof(i, (int)j));
                    P.force_series.push_back(s);
                    P.force_coef.push_back(fac * dir[j] * it->second[j]);
                }
            }
        } else if (lname == "ELEMENTLOAD" && kind == "BODY") {
            // rho * integral of H^T dir per element (Assembler.cpp:439-459)
            std::vector<double> fe((size_t)nen * ndim), q(dir);
            q.resize(std::max<size_t>(q.size(), (size_t)ndim), 0.0);
            for (const Json& et : la.at("list").list()) {
                const int e = epos.at((int)et.number());
                check(svl_element_body_force(&md, e, q.data(), fe.data()));
                for (int a = 0; a < nen; ++a)
                    for (int j = 0; j < ndim; ++j) {
                        const double v = fe[(size_t)a * ndim + j];
                        if (v == 0.0) continue;
                        P.force_dof.push_back(tdof(P.conn[(size_t)e * nen + a], j));
                        P.force_series.push_back(s);
                        P.force_coef.push_back(fac * v);
                    }
            }
        } else {
            unsupported("load " + ld.at("name").text() + "/" + la.at("type").text() + " (tag " + ltag + ") is not covered");
        }
    }
    if (!P.drm_elem.empty()) {
        // motion blocks in node order
        P.drm_node_row.assign(P.nnode, -1);
        P.drm_node_ext.assign(P.nnode, 0);
        const size_t blk = (size_t)P.drm_nt * 3 * ndim;
        int row = 0;
        for (const auto& kv : drm_nodes) {
            P.drm_node_row[kv.first] = row++;
            P.drm_node_ext[kv.first] = kv.second.second;
            const double* src = &drm_blocks[(size_t)kv.second.first * blk];
            P.drm_motion.insert(P.drm_motion.end(), src, src + blk);
        }
    }
    // support motions (Assembler.cpp:493-532, Node.cpp:228-247)
    const Json& SP = d.has("Supports") ? d.at("Supports") : empty;
    if (SP.kind == Json::Object)
        for (const std::string& key : SP.keys) {                        // file order
            const int i = npos.at(std::atoi(key.c_str()));
            const Json& sp = SP.at(key);
            const std::string type = upper(sp.at("type").text());
            const auto& dofs = sp.at("dof").list();
            for (size_t n = 0; n < dofs.size(); ++n) {
                std::vector<double> series;
                if (type == "TIMESERIES") series = read_series(detail::join(run_dir, sp.at("file").list().at(n).text()));
                else if (type == "CONSTANT") series.assign(1, sp.at("value").list().at(n).number());
                else unsupported("support motion " + sp.at("type").text() + " is not covered");
                P.sm_dof.push_back(tdof(i, (int)dofs[n].number()));
                P.sm_series.push_back(P.add_series(series));
                P.sm_factor.push_back(1.0);
            }
        }
    // node and element recorders (Recorder.cpp:73-166, 239-323)
    const Json& RC = d.has("Recorders") ? d.at("Recorders") : empty;
    for (int t : sorted_tags(RC)) {
        const Json& r = RC.at(std::to_string(t));
        NodeRecorder nr;
        nr.name = upper(r.at("name").text());
        nr.file = r.at("file").text();
        nr.response = upper(r.at("resp").text());
        if (nr.name == "NODE") {
            if (nr.response != "DISP" && nr.response != "VEL" && nr.response != "ACCEL" && nr.response != "REACTION")
                unsupported("node recorder response " + r.at("resp").text() + " is not covered");
        } else if (nr.name == "ELEMENT") {
            if (nr.response != "STRESS" && nr.response != "STRAIN" && nr.response != "INTERNALFORCE" && nr.response != "STRAINRATE")
                unsupported("element recorder response " + r.at("resp").text() + " is not covered");
            for (const Json& v : r.at("list").list()) {
                auto it = epos.find((int)v.number());
                if (it == epos.end() || P.elem_pml[it->second]) unsupported("element recorder " + nr.file + ": element " + v.text() + " is not a solid element of this model");
            }
        } else {
            unsupported("recorder " + r.at("name").text() + " is not covered (NODE, ELEMENT)");
        }
        for (const Json& v : r.at("list").list()) nr.ids.push_back((int)v.number());
        nr.precision = (int)r.number("ndps", 8);
        nr.nsamp = (int)r.number("nsamp", 1);
        P.recorders.push_back(nr);
    }
    return P;
}

}  // namespace gpu
}  // namespace svl
