"""Reader for SeismoVLAB partition files and writer for its node recorders.

A partition file is what the SVL pre-processor writes for one process
(`<run dir>/Partition/<name>.<combo>.<rank>.json`, PP/Core/SeismoVLAB.py
createPartitions) and what the run-process parses (RP/12-Utilities/Driver.hpp
UpdateMesh / UpdateMaterials / UpdateLoads / UpdateSupportMotion /
UpdateConstraints, 392-1700, and the simulation block 1760-1840).  This module
maps it onto the library's model and load descriptors so an unmodified
pre-processed model runs on the GPU integrators, and writes node recorder
output in the run-process's text format (RP/12-Utilities/Recorder.cpp:73-106
header, 239-268 rows).

Covered: lin2DQuad4 / lin3DHexa8 elements with PML2DQuad4 / PML3DHexa8
layers (5 / 9 dofs at their nodes); Elastic2DPlaneStrain, Elastic3DLinear,
PlasticPlaneStrainJ2, Plastic3DJ2 materials; restraints; EQUAL-type
constraints; nodal masses; Rayleigh dampings; ZeroLength1D elements with a
Viscous1DLinear material (Lysmer dashpots); domain-reduction (DRM) element
loads with per-node free-field files; point loads and element body
loads (constant or time series); support motions (constant or time series);
node recorders of displacement, velocity, acceleration or reaction; element
recorders of stress, strain, internal force or strain rate; the integrators
CentralDifference, Newmark and ExtendedNewmark under the names the run-process
accepts (Driver.hpp:1808-1822).  Anything else raises PartitionError naming it.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional

import numpy as np

from . import _capi as capi
from .model import Loads, Model

_ELEM = {"LIN2DQUAD4": (2, 4, capi.SVL_ELEM_LIN2DQUAD4), "LIN3DHEXA8": (3, 8, capi.SVL_ELEM_LIN3DHEXA8)}
_PML = {"PML2DQUAD4": "LIN2DQUAD4", "PML3DHEXA8": "LIN3DHEXA8"}
_MAT = {
    "ELASTIC2DPLANESTRAIN": (capi.SVL_MAT_ELASTIC2DPLANESTRAIN, ("E", "nu", "rho")),
    "ELASTIC3DLINEAR": (capi.SVL_MAT_ELASTIC3DLINEAR, ("E", "nu", "rho")),
    "PLASTICPLANESTRAINJ2": (capi.SVL_MAT_PLASTICPLANESTRAINJ2, ("K", "G", "rho", "h", "beta", "Sy")),
    "PLASTIC3DJ2": (capi.SVL_MAT_PLASTIC3DJ2, ("K", "G", "rho", "h", "beta", "Sy")),
}


class PartitionError(ValueError):
    """The partition file uses something this path does not cover."""


def read_series(path: Path) -> np.ndarray:
    """Time-series file: first token the number of values, then the values
    (Driver.hpp:1514-1527)."""
    tok = path.read_text().split()
    n = int(float(tok[0]))
    vals = np.array([float(t) for t in tok[1:1 + n]], dtype=np.float64)
    if vals.size != n:
        raise PartitionError("%s: expected %d values, found %d" % (path, n, vals.size))
    return vals


def read_drm_motion(root: Path, pattern: str, elems: list, npos: dict, ndim: int) -> dict:
    """Free-field motion of every node of the DRM elements: the file named by
    `pattern` with "$" replaced by the node tag holds `nt nFields cond` and
    then nt rows of u, v, a per direction; cond 1 marks an exterior node
    (Driver.hpp:1689-1719)."""
    out = {}
    for e in elems:
        for ntag in e["conn"]:
            ntag = int(ntag)
            if npos[ntag] in out:
                continue
            path = Path(pattern.replace("$", str(ntag)))
            if not path.is_absolute():
                path = root / path
            tok = path.read_text().split()
            nt, nf, cond = int(float(tok[0])), int(float(tok[1])), int(float(tok[2]))
            if nf != 3 * ndim:
                raise PartitionError("%s: %d fields per row, %d expected (u, v, a)" % (path, nf, 3 * ndim))
            vals = np.array([float(x) for x in tok[3:3 + nt * nf]]).reshape(nt, nf)
            out[npos[ntag]] = (vals, bool(cond))
    return out


@dataclass
class Recorder:
    name: str
    file: str
    response: str
    ids: List[int]
    precision: int
    nsamp: int = 1


@dataclass
class Partition:
    model: Model
    loads: Loads
    integrator: str
    dt: float
    nt: int
    ftol: float
    mtol: float
    ktol: float
    algorithm: dict
    solver: dict
    combo_folder: str
    node_tags: np.ndarray
    elem_tags: np.ndarray
    recorders: List[Recorder] = field(default_factory=list)
    root: Optional[Path] = None

    def make_integrator(self, pcg_tol: Optional[float] = None):
        """The GPU integrator the simulation block asks for: CENTRALDIFFERENCE
        (on a model with PML layers the library's explicit PML scheme on the
        PML-capable handle), NEWMARK (NewmarkBeta; on a model with PML layers the PML-capable
        handle in NewmarkBeta mode) or EXTENDEDNEWMARK (ExtendedNewmarkBeta),
        with the algorithm LINEAR or NEWTON (`cnvgtol` 1e-6, `nstep` 50,
        `cnvgtest` 4 by default, Driver.hpp:1786-1822); an iterative solver's
        `tol` is the solve tolerance, a direct solver gets 1e-12."""
        from .integrators import CentralDifference, ExtendedNewmarkBeta, NewmarkBeta
        algo = str(self.algorithm.get("name", "LINEAR")).upper()
        if algo not in ("LINEAR", "NEWTON"):
            raise PartitionError("algorithm %s is not covered (LINEAR, NEWTON)" % algo)
        if self.integrator == "CENTRALDIFFERENCE":
            if algo != "LINEAR":
                raise PartitionError("CENTRALDIFFERENCE is covered with the LINEAR algorithm")
            return CentralDifference(self.model, self.loads, self.dt, ftol=self.ftol, mtol=self.mtol)
        if self.integrator in ("NEWMARK", "EXTENDEDNEWMARK"):
            tol = pcg_tol if pcg_tol is not None else (float(self.solver.get("tol", 1e-12))
                                                       if self.solver.get("name", "").upper() == "PETSC" else 1e-12)
            kw = dict(algorithm=algo.lower(), maxit=int(self.algorithm.get("nstep", 50)),
                      cnvgtol=float(self.algorithm.get("cnvgtol", 1e-6)),
                      cnvgtest=int(self.algorithm.get("cnvgtest", 4)))
            if self.integrator == "EXTENDEDNEWMARK":
                return ExtendedNewmarkBeta(self.model, self.loads, self.dt, tol=tol, ftol=self.ftol, mtol=self.mtol,
                                           **kw)
            return NewmarkBeta(self.model, self.loads, self.dt, pcg_tol=tol, ftol=self.ftol, mtol=self.mtol, **kw)
        raise PartitionError("integrator %s is not covered (the run-process names CENTRALDIFFERENCE, NEWMARK, "
                             "EXTENDEDNEWMARK)" % self.integrator)

    def run(self, write_recorders: bool = True, solution_dir: Optional[Path] = None):
        """The run-process's dynamic loop (DynamicAnalysis.cpp:25-64): steps
        k = 1 .. nt-1 and every node recorder written after each step.  Returns
        the displacement history [nt-1][ntotal]."""
        h = self.make_integrator()
        erecs = [r for r in self.recorders if r.name == "ELEMENT"]
        if erecs and not hasattr(h, "element_response"):
            h.close()
            raise PartitionError("ELEMENT recorders are covered for CENTRALDIFFERENCE and NEWMARK on models without "
                                 "PML layers")
        need_r = any(r.response == "REACTION" for r in self.recorders)
        if need_r and self.integrator == "CENTRALDIFFERENCE" and self.model.elem_pml is not None \
                and np.any(self.model.elem_pml):
            h.close()
            raise PartitionError("REACTION recorders are not covered for CENTRALDIFFERENCE on models with PML layers "
                                 "(the explicit PML scheme's stress dofs live at the half steps)")
        h.Initialize()
        nsteps = self.nt - 1
        need_va = any(r.response in ("VEL", "ACCEL") for r in self.recorders)
        R = None
        epos = {int(t): i for i, t in enumerate(self.elem_tags)}
        EH = {id(r): [] for r in erecs}                  # per element recorder: one row per step
        if need_va or need_r or erecs:
            U = np.zeros((nsteps, self.model.ntotal))
            V = np.zeros_like(U) if need_va else None
            A = np.zeros_like(U) if need_va else None
            R = np.zeros_like(U) if need_r else None
            for s in range(nsteps):
                if h.ComputeNewStep(s + 1):
                    raise RuntimeError("A PROBLEM WAS ENCOUNTERED at step %d: %s"
                                       % (s + 1, capi.lib().svl_last_error().decode()))
                U[s] = h.GetDisplacements()
                if need_va:
                    V[s], A[s] = h.GetVelocities(), h.GetAccelerations()
                if need_r:                     # DynamicAnalysis::UpdateDomain (DynamicAnalysis.cpp:128-150)
                    R[s] = h.ComputeReactionForce(s + 1)
                for r in erecs:                # Recorder::WriteElementResponse after every step
                    EH[id(r)].append(h.element_response(r.response, [epos[t] for t in r.ids]).reshape(-1))
        else:
            U = h.run(1, nsteps, history=True)
            V = A = None
        h.close()
        if write_recorders and self.recorders:
            out = Path(solution_dir) if solution_dir else (self.root / "Solution" / self.combo_folder)
            out.mkdir(parents=True, exist_ok=True)
            for r in self.recorders:
                if r.name == "ELEMENT":
                    write_element_recorder(out / r.file, self, r, np.array(EH[id(r)]))
                    continue
                hist = {"DISP": U, "VEL": V, "ACCEL": A, "REACTION": R}[r.response]
                write_node_recorder(out / r.file, self, r, hist)
        return U


def write_node_recorder(path: Path, part: Partition, rec: Recorder, hist: np.ndarray):
    """Node recorder in the run-process's format: `n_nodes n_dofs ntotal nt`,
    one `tag ndof totaldofs...` line per node, then one line per step with every
    recorded dof in scientific notation with `precision` digits, each value
    followed by a space (Recorder.cpp:73-106, 239-268)."""
    m = part.model
    pos = {int(t): i for i, t in enumerate(part.node_tags)}
    idx = [pos[t] for t in rec.ids]
    nnd = m.dof_mask().sum(axis=1)
    fmt = "%." + str(int(rec.precision)) + "e "
    dofs = [m.totaldof[i, :nnd[i]] for i in idx]
    cols = np.concatenate(dofs) if idx else np.zeros(0, np.int64)
    with open(path, "w") as f:
        f.write("%d %d %d %d\n" % (len(idx), cols.size, m.ntotal, part.nt))
        for t, d in zip(rec.ids, dofs):
            f.write("%d %d %s\n" % (t, d.size, " ".join(str(int(x)) for x in d)))
        for row in hist[:, cols]:
            f.write("".join(fmt % v for v in row) + "\n")


def write_element_recorder(path: Path, part: Partition, rec: Recorder, rows: np.ndarray):
    """Element recorder in the run-process's format (Recorder.cpp:107-166 header,
    272-323 rows): `n_elements ntotal nt`, then per element `tag ndof totaldofs...`
    (INTERNALFORCE) or `tag n_gauss_points n_components` (STRESS, STRAIN,
    STRAINRATE), then one line per step with the elements' values (Gauss points
    row by row) in scientific notation, each followed by a space."""
    m = part.model
    epos = {int(t): i for i, t in enumerate(part.elem_tags)}
    ngp = 4 if m.ndim == 2 else 8
    ncomp = 3 if m.ndim == 2 else 6
    fmt = "%." + str(int(rec.precision)) + "e "
    with open(path, "w") as f:
        f.write("%d %d %d\n" % (len(rec.ids), m.ntotal, part.nt))
        for t in rec.ids:
            if rec.response == "INTERNALFORCE":
                nodes = m.conn[epos[t]]
                dofs = [int(x) for n in nodes for x in m.totaldof[n, :m.dof_mask()[n].sum()]]
                f.write("%d %d %s\n" % (t, m.ndim * m.conn.shape[1], " ".join(str(x) for x in dofs)))
            else:
                f.write("%d %d %d\n" % (t, ngp, ncomp))
        for row in rows:
            f.write("".join(fmt % v for v in row) + "\n")


def load_partition(path, run_dir=None) -> Partition:
    """Parses one partition file.  Time-series files are looked up relative to
    `run_dir` (default: the directory that holds the Partition folder, the
    run-process's working directory)."""
    path = Path(path)
    d = json.loads(path.read_text())
    root = Path(run_dir) if run_dir else (path.parent.parent if path.parent.name == "Partition" else path.parent)
    g = d["Global"]
    ndim = int(g["ndim"])
    # nodes in ascending tag order (the run-process's std::map order)
    ntags = sorted(int(t) for t in d["Nodes"])
    nodes = [d["Nodes"][str(t)] for t in ntags]
    pnd = 5 if ndim == 2 else 9
    nnd = np.array([int(n["ndof"]) for n in nodes], dtype=np.int32)
    if not np.all((nnd == ndim) | (nnd == pnd)):
        raise PartitionError("nodes with %s dofs: %d-dof displacement nodes and %d-dof PML nodes are covered"
                             % (sorted(set(nnd.tolist())), ndim, pnd))
    stride = int(nnd.max())
    coords = np.array([n["coords"] for n in nodes], dtype=np.float64).reshape(len(nodes), ndim)
    totaldof = -np.ones((len(nodes), stride), np.int32)
    freedof = -np.ones((len(nodes), stride), np.int32)
    for i, n in enumerate(nodes):
        totaldof[i, :nnd[i]] = n["totaldof"]
        freedof[i, :nnd[i]] = n["freedof"]
    npos = {t: i for i, t in enumerate(ntags)}
    # materials (Viscous1DLinear, Driver.hpp:602-607, only as a ZeroLength1D dashpot)
    viscous = {int(t): float(mt["attributes"].get("eta", 0.0)) for t, mt in d.get("Materials", {}).items()
               if mt["name"].upper() == "VISCOUS1DLINEAR"}
    mtags = sorted(int(t) for t in d.get("Materials", {}) if int(t) not in viscous)
    mpos = {t: i for i, t in enumerate(mtags)}
    mat_type = np.zeros(len(mtags), np.int32)
    mat_param = np.zeros((len(mtags), capi.SVL_MAT_NPARAM))
    for i, t in enumerate(mtags):
        mat = d["Materials"][str(t)]
        name = mat["name"].upper()
        if name not in _MAT:
            raise PartitionError("material %s (tag %d) is not covered" % (mat["name"], t))
        mat_type[i], keys = _MAT[name]
        mat_param[i, :len(keys)] = [float(mat["attributes"][k]) for k in keys]
    # elements in ascending tag order; ZeroLength1D elements with a viscous
    # material become dashpots on their direction `dir` (ZeroLength1D.cpp:210-228)
    dash_dof, dash_eta = [], []
    for t in sorted(int(x) for x in d["Elements"]):
        e = d["Elements"][str(t)]
        if e["name"].upper() != "ZEROLENGTH1D":
            continue
        mt = int(e["attributes"]["material"])
        if mt not in viscous:
            raise PartitionError("ZeroLength1D element %d: only a Viscous1DLinear material (a dashpot) is covered" % t)
        j = int(e["attributes"]["dir"])
        a, b = (npos[int(c)] for c in e["conn"])
        if not (0 <= j < ndim):
            raise PartitionError("ZeroLength1D element %d: dir %d out of range" % (t, j))
        dash_dof.append((int(totaldof[a, j]), int(totaldof[b, j])))
        dash_eta.append(viscous[mt])
    etags = sorted(int(t) for t in d["Elements"] if d["Elements"][t]["name"].upper() != "ZEROLENGTH1D")
    els = [d["Elements"][str(t)] for t in etags]
    names = {e["name"].upper() for e in els}
    solid = {_PML.get(n, n) for n in names}
    if len(solid) != 1 or next(iter(solid)) not in _ELEM:
        raise PartitionError("element classes %s: one of %s per model (with its PML class) is covered"
                             % (sorted(names), sorted(_ELEM)))
    edim, nen, etype = _ELEM[next(iter(solid))]
    if edim != ndim:
        raise PartitionError("element dimension does not match Global.ndim")
    # PML elements (Driver.hpp:1203-1220, 1288-1306): n, L, R, x0, npml
    epml = np.array([1 if e["name"].upper() in _PML else 0 for e in els], dtype=np.int32)
    pml_param = np.zeros((len(els), 3 + 2 * ndim))
    for i, e in enumerate(els):
        if epml[i]:
            a = e["attributes"]
            pml_param[i] = [float(a["n"]), float(a["L"]), float(a["R"])] + [float(v) for v in a["x0"][:ndim]] \
                + [float(v) for v in a["npml"][:ndim]]
    conn = np.array([[npos[int(c)] for c in e["conn"]] for e in els], dtype=np.int32).reshape(len(els), nen)
    elem_mat = np.array([mpos[int(e["attributes"]["material"])] for e in els], dtype=np.int32)
    thick = np.array([float(e["attributes"].get("th", 1.0)) for e in els]) if ndim == 2 else None
    # dampings in ascending tag order, each assigned to its element list
    # (Driver.hpp:1365-1405); a later tag overrides an earlier one
    epos = {t: i for i, t in enumerate(etags)}
    ray = np.zeros((len(etags), 2))
    for t in sorted(int(x) for x in d.get("Dampings", {})):
        dm = d["Dampings"][str(t)]
        name = dm["name"].upper()
        at = dm.get("attributes", {})
        if name == "FREE":
            par = (0.0, 0.0)
        elif name == "RAYLEIGH":
            par = (float(at.get("am", 0.0)), float(at.get("ak", 0.0)))
        else:
            raise PartitionError("damping %s (tag %d) is not covered" % (dm["name"], t))
        for e in at.get("list", []):
            if int(e) in epos:
                ray[epos[int(e)]] = par
    # nodal masses
    node_mass = None
    nmass = {}                                   # node position -> its mass entries (Node::GetMass)
    if d.get("Masses"):
        node_mass = np.zeros(int(g["ntotal"]))
        for t, ms in d["Masses"].items():
            i = npos[int(t)]
            nmass[i] = [float(v) for v in ms["mass"]]
            for k, v in enumerate(ms["mass"]):
                node_mass[totaldof[i, k]] += float(v)
    # constraints: slave total dof <- sum factor * master free dof
    con = None
    if d.get("Constraints"):
        ctags = sorted((int(t) for t in d["Constraints"]), reverse=True)
        cs, cp, cm, cf = [], [0], [], []
        for t in ctags:
            c = d["Constraints"][str(t)]
            cs.append(int(c["stag"]))
            cm += [int(x) for x in c["mtag"]]
            cf += [float(x) for x in c["factor"]]
            cp.append(len(cm))
        con = (np.array(cs, np.int32), np.array(cp, np.int32), np.array(cm, np.int32), np.array(cf))
    model = Model(ndim=ndim, coords=coords, totaldof=totaldof, freedof=freedof, conn=conn, elem_type=etype,
                  elem_mat=elem_mat, mat_type=mat_type, mat_param=mat_param,
                  lumped=str(g.get("massform", "CONSISTENT")).upper() == "LUMPED",
                  thickness=thick, node_mass=node_mass, rayleigh=ray if np.any(ray) else None,
                  node_ndof=nnd if stride != ndim else None, elem_pml=epml if epml.any() else None,
                  pml_param=pml_param if epml.any() else None,
                  dashpot_dof=np.array(dash_dof, np.int32).reshape(-1, 2) if dash_dof else None,
                  dashpot_eta=np.array(dash_eta) if dash_eta else None)
    if con is not None:
        model.con_slave, model.con_ptr, model.con_master, model.con_factor = con
    if model.ntotal != int(g["ntotal"]) or model.nfree != int(g["nfree"]):
        raise PartitionError("Global ntotal/nfree do not match the nodes")
    # simulation block
    sim = d["Simulations"]
    at = sim["attributes"]
    integ = at["integrator"]
    nt = int(at["analysis"]["nt"])
    if at["analysis"]["name"].upper() != "DYNAMIC":
        raise PartitionError("analysis %s is not covered" % at["analysis"]["name"])
    combo = d["Combinations"][str(sim["combo"])]
    loads = Loads()
    for ltag, fac in zip(combo["attributes"]["load"], combo["attributes"]["factor"]):
        ld = d["Loads"][str(ltag)]
        la = ld["attributes"]
        kind, fun = la["type"].upper(), la["name"].upper()
        if ld["name"].upper() == "ELEMENTLOAD" and kind == "GENERALWAVE":
            loads.add_drm(model, [epos[int(e)] for e in la["list"]],
                          read_drm_motion(root, la["file"], [e for e in (d["Elements"][str(t)] for t in la["list"])],
                                          npos, ndim), factor=float(fac))
            continue
        if fun == "TIMESERIES":
            series = read_series(root / la["file"])
        elif fun == "CONSTANT":
            series = np.full(nt, float(la["mag"]))          # GetLoadVector() of a constant load: every step
        else:
            raise PartitionError("load function %s is not covered" % la["name"])
        s = loads.add_series(series)
        direction = [float(x) for x in la["dir"]]
        # Assembler::ComputeExternalForceVector (Assembler.cpp:291-489) assembles
        # every load into its own zeroed vector by assignment, Fext(dof) = Fn(i)
        # (point loads) or Fn(i) * Mn(i) (body point loads, Mn the node's mass
        # entries; nodes without a Masses entry get nothing), then adds
        # factor * Fext: across loads the entries add, within one load a node
        # listed twice counts once
        nodes = list(dict.fromkeys(int(t) for t in la.get("list", [])))
        if ld["name"].upper() == "POINTLOAD" and kind == "CONCENTRATED":
            for ntag in nodes:
                loads.add_point_load(model, npos[int(ntag)], direction, s, factor=float(fac))
        elif ld["name"].upper() == "POINTLOAD" and kind == "BODY":
            for ntag in nodes:
                i = npos[int(ntag)]
                if i not in nmass:
                    continue
                mn = nmass[i]
                for j, v in enumerate(direction[:len(mn)]):
                    loads.force_dof.append(int(model.totaldof[i, j]))
                    loads.force_series.append(s)
                    loads.force_coef.append(float(fac) * v * mn[j])
        elif ld["name"].upper() == "ELEMENTLOAD" and kind == "BODY":
            loads.add_body_load(model, [epos[int(e)] for e in la["list"]], direction, s, factor=float(fac))
        else:
            raise PartitionError("load %s/%s (tag %s) is not covered" % (ld["name"], la["type"], ltag))
    for ntag, sp in d.get("Supports", {}).items():
        i = npos[int(ntag)]
        for n, dof in enumerate(sp["dof"]):
            if sp["type"].upper() == "TIMESERIES":
                series = read_series(root / sp["file"][n])
            elif sp["type"].upper() == "CONSTANT":
                series = np.array([float(sp["value"][n])])
            else:
                raise PartitionError("support motion %s is not covered" % sp["type"])
            loads.add_support_motion(model, i, int(dof), loads.add_series(series))
    recs = []
    for rtag in sorted(d.get("Recorders", {}), key=int):
        r = d["Recorders"][rtag]
        rname, resp = r["name"].upper(), r["resp"].upper()
        if rname == "NODE":
            if resp not in ("DISP", "VEL", "ACCEL", "REACTION"):
                raise PartitionError("node recorder response %s is not covered" % r["resp"])
        elif rname == "ELEMENT":
            if resp not in ("STRAIN", "STRESS", "INTERNALFORCE", "STRAINRATE"):
                raise PartitionError("element recorder response %s is not covered" % r["resp"])
            for t in r["list"]:
                if int(t) not in epos or epml[epos[int(t)]]:
                    raise PartitionError("element recorder %s: element %s is not a solid element of this model"
                                         % (r["file"], t))
        else:
            raise PartitionError("recorder %s is not covered (NODE, ELEMENT)" % r["name"])
        recs.append(Recorder(name=rname, file=r["file"], response=resp, ids=[int(x) for x in r["list"]],
                             precision=int(r.get("ndps", 8)), nsamp=int(r.get("nsamp", 1))))
    return Partition(model=model, loads=loads, integrator=integ["name"].upper(), dt=float(integ["dt"]), nt=nt,
                     ftol=float(integ.get("ftol", 1e-12)), mtol=float(integ.get("mtol", 1e-12)),
                     ktol=float(integ.get("ktol", 1e-12)), algorithm=at.get("algorithm", {}),
                     solver=at.get("solver", {}), combo_folder=combo["attributes"].get("folder", combo["name"]),
                     node_tags=np.array(ntags), elem_tags=np.array(etags), recorders=recs, root=root)
