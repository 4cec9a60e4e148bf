"""Host-side model and load containers (the arrays behind svl_model_desc /
svl_load_desc) and the structured-grid builder.

A `Model` holds one pre-processed SVL partition: nodes in ascending tag
order, elements in ascending tag order, PlainScheme total/free dof numbers
(PP/Core/Numberer.py:185-233) and the material table.  Ensembles of
independent instances are one `Model` whose instances are disjoint node and
element blocks (`Model.concat`), so one launch steps them all.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _capi as capi
from ._capi import as_f64, as_i32, check, lib, ptr


@dataclass
class Model:
    ndim: int
    coords: np.ndarray            # [nnode, ndim]
    totaldof: np.ndarray          # [nnode, ndof]
    freedof: np.ndarray           # [nnode, ndof]
    conn: np.ndarray              # [nelem, nen] node positions
    elem_type: int
    elem_mat: np.ndarray          # [nelem]
    mat_type: np.ndarray          # [nmat]
    mat_param: np.ndarray         # [nmat, 8]
    thickness: Optional[np.ndarray] = None
    con_slave: Optional[np.ndarray] = None
    con_ptr: Optional[np.ndarray] = None
    con_master: Optional[np.ndarray] = None
    con_factor: Optional[np.ndarray] = None
    lumped: bool = True
    node_mass: Optional[np.ndarray] = None
    rayleigh: Optional[np.ndarray] = None  # [nelem, 2] (am, ak) or None
    node_ndof: Optional[np.ndarray] = None  # [nnode] dofs of each node (PML nodes 5 / 9), None: all ndof
    elem_pml: Optional[np.ndarray] = None   # [nelem] 1 for PML2DQuad4 / PML3DHexa8 elements
    pml_param: Optional[np.ndarray] = None  # [nelem, 3 + 2 ndim] n, L, R, x0, npml
    dashpot_dof: Optional[np.ndarray] = None  # [n, 2] total dofs of Lysmer dashpots (ZeroLength1D)
    dashpot_eta: Optional[np.ndarray] = None  # [n] damping coefficients
    grid_shape: Optional[tuple] = None   # (nx, ny[, nz]) when built by grid()
    _keep: list = field(default_factory=list, repr=False)

    @property
    def nnode(self):
        return int(self.coords.shape[0])

    @property
    def nelem(self):
        return int(self.conn.shape[0])

    @property
    def ndof(self):
        return int(self.totaldof.shape[1])

    def dof_mask(self) -> np.ndarray:
        """[nnode, ndof] True where the node has that dof."""
        if self.node_ndof is None:
            return np.ones(self.totaldof.shape, bool)
        return np.arange(self.totaldof.shape[1])[None, :] < np.asarray(self.node_ndof)[:, None]

    @property
    def ntotal(self):
        return int(self.dof_mask().sum())

    @property
    def nfree(self):
        return int(((self.freedof >= 0) & self.dof_mask()).sum())

    @property
    def nconstraint(self):
        return 0 if self.con_slave is None else int(self.con_slave.size)

    def desc(self) -> capi.ModelDesc:
        arrs = dict(
            coords=as_f64(self.coords), totaldof=as_i32(self.totaldof), freedof=as_i32(self.freedof),
            conn=as_i32(self.conn), elem_mat=as_i32(self.elem_mat), mat_type=as_i32(self.mat_type),
            mat_param=as_f64(self.mat_param),
            thickness=None if self.thickness is None else as_f64(self.thickness),
            con_slave=None if self.con_slave is None else as_i32(self.con_slave),
            con_ptr=None if self.con_ptr is None else as_i32(self.con_ptr),
            con_master=None if self.con_master is None else as_i32(self.con_master),
            con_factor=None if self.con_factor is None else as_f64(self.con_factor),
            node_mass=None if self.node_mass is None else as_f64(self.node_mass),
            rayleigh=None if self.rayleigh is None else as_f64(self.rayleigh),
            node_ndof=None if self.node_ndof is None else as_i32(self.node_ndof),
            elem_pml=None if self.elem_pml is None else as_i32(self.elem_pml),
            pml_param=None if self.pml_param is None else as_f64(self.pml_param),
            dashpot_dof=None if self.dashpot_dof is None else as_i32(self.dashpot_dof),
            dashpot_eta=None if self.dashpot_eta is None else as_f64(self.dashpot_eta),
        )
        self._keep = list(arrs.values())
        d = capi.ModelDesc()
        d.ndim = self.ndim
        d.nnode = self.nnode
        d.ndof = self.ndof
        d.coords = ptr(arrs["coords"], C.c_double)
        d.totaldof = ptr(arrs["totaldof"], C.c_int32)
        d.freedof = ptr(arrs["freedof"], C.c_int32)
        d.ntotal = self.ntotal
        d.nfree = self.nfree
        d.nconstraint = self.nconstraint
        d.con_slave = ptr(arrs["con_slave"], C.c_int32)
        d.con_ptr = ptr(arrs["con_ptr"], C.c_int32)
        d.con_master = ptr(arrs["con_master"], C.c_int32)
        d.con_factor = ptr(arrs["con_factor"], C.c_double)
        d.elem_type = self.elem_type
        d.nelem = self.nelem
        d.conn = ptr(arrs["conn"], C.c_int32)
        d.elem_mat = ptr(arrs["elem_mat"], C.c_int32)
        d.elem_thickness = ptr(arrs["thickness"], C.c_double)
        d.nmat = int(self.mat_type.size)
        d.mat_type = ptr(arrs["mat_type"], C.c_int32)
        d.mat_param = ptr(arrs["mat_param"], C.c_double)
        d.lumped = 1 if self.lumped else 0
        d.node_mass = ptr(arrs["node_mass"], C.c_double)
        d.elem_rayleigh = ptr(arrs["rayleigh"], C.c_double)
        d.node_ndof = ptr(arrs["node_ndof"], C.c_int32)
        d.elem_pml = ptr(arrs["elem_pml"], C.c_int32)
        d.elem_pml_param = ptr(arrs["pml_param"], C.c_double)
        d.ndashpot = 0 if self.dashpot_eta is None else int(np.asarray(self.dashpot_eta).size)
        d.dashpot_dof = ptr(arrs["dashpot_dof"], C.c_int32)
        d.dashpot_eta = ptr(arrs["dashpot_eta"], C.c_double)
        return d

    # ------------------------------------------------------------------
    @staticmethod
    def grid(ndim: int, ne: Sequence[int], h: Sequence[float], origin=(0.0, 0.0, 0.0),
             fix_mask=(0, 0, 0, 0, 0, 0), periodic_x: bool = False,
             mat_type=None, mat_param=None, elem_mat=None) -> "Model":
        """Structured Q4/H8 grid numbered like makeDomainArea/Volume +
        PlainScheme, generated by the library (svl_grid_build)."""
        L = lib()
        spec = capi.GridSpec()
        spec.ndim = ndim
        for i in range(3):
            spec.ne[i] = int(ne[i]) if i < ndim else 0
            spec.h[i] = float(h[i]) if i < ndim else 0.0
            spec.origin[i] = float(origin[i]) if i < len(origin) else 0.0
        for i in range(6):
            spec.fix_mask[i] = int(fix_mask[i])
        spec.periodic_x = 1 if periodic_x else 0
        nn, ne_, nt, nf, nc = (C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32())
        check(L.svl_grid_sizes(C.byref(spec), C.byref(nn), C.byref(ne_), C.byref(nt), C.byref(nf), C.byref(nc)))
        nen = 4 if ndim == 2 else 8
        coords = np.zeros((nn.value, ndim))
        tdof = np.zeros((nn.value, ndim), np.int32)
        fdof = np.zeros((nn.value, ndim), np.int32)
        conn = np.zeros((ne_.value, nen), np.int32)
        ncon = nc.value
        cs = np.zeros(max(ncon, 1), np.int32)
        cp = np.zeros(ncon + 1, np.int32)
        cm = np.zeros(max(ncon, 1), np.int32)
        cf = np.zeros(max(ncon, 1))
        check(L.svl_grid_build(C.byref(spec), ptr(coords, C.c_double), ptr(tdof, C.c_int32), ptr(fdof, C.c_int32),
                               ptr(conn, C.c_int32), ptr(cs, C.c_int32), ptr(cp, C.c_int32), ptr(cm, C.c_int32),
                               ptr(cf, C.c_double)))
        if mat_type is None:
            mat_type = np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN if ndim == 2 else capi.SVL_MAT_ELASTIC3DLINEAR], np.int32)
            mat_param = np.array([[2.0e8, 0.25, 2000.0, 0, 0, 0, 0, 0]])
        if elem_mat is None:
            elem_mat = np.zeros(ne_.value, np.int32)
        m = Model(ndim=ndim, coords=coords, totaldof=tdof, freedof=fdof, conn=conn,
                  elem_type=capi.SVL_ELEM_LIN2DQUAD4 if ndim == 2 else capi.SVL_ELEM_LIN3DHEXA8,
                  elem_mat=as_i32(elem_mat), mat_type=as_i32(mat_type), mat_param=as_f64(np.atleast_2d(mat_param)),
                  grid_shape=tuple(int(x) for x in ne[:ndim]))
        if ncon > 0:
            m.con_slave, m.con_ptr, m.con_master, m.con_factor = cs[:ncon], cp, cm[:ncon], cf[:ncon]
        return m

    @staticmethod
    def concat(models: List["Model"]) -> "Model":
        """Disjoint union of models with the same element type (ensembles).
        Node, dof and element numbers are offset block by block, so instance
        i keeps its own PlainScheme order inside its block."""
        assert models and all(m.elem_type == models[0].elem_type for m in models)
        nd = models[0].ndim
        coords, tdof, fdof, conn, emat, mtyp, mpar = [], [], [], [], [], [], []
        cs, cm, cf, cnt = [], [], [], []
        thick = []
        noff = toff = foff = moff = 0
        any_thick = any(m.thickness is not None for m in models)
        for m in models:
            coords.append(m.coords)
            tdof.append(m.totaldof + toff)
            fd = m.freedof.copy()
            fd[fd >= 0] += foff
            fdof.append(fd)
            conn.append(m.conn + noff)
            emat.append(m.elem_mat + moff)
            mtyp.append(m.mat_type)
            mpar.append(m.mat_param)
            if any_thick:
                thick.append(m.thickness if m.thickness is not None else np.ones(m.nelem))
            if m.nconstraint:
                cs.append(m.con_slave + toff)
                cm.append(m.con_master + foff)
                cf.append(m.con_factor)
                cnt.append(np.diff(m.con_ptr))
            noff += m.nnode
            toff += m.ntotal
            foff += m.nfree
            moff += int(m.mat_type.size)
        out = Model(ndim=nd, coords=np.concatenate(coords), totaldof=np.concatenate(tdof).astype(np.int32),
                    freedof=np.concatenate(fdof).astype(np.int32), conn=np.concatenate(conn).astype(np.int32),
                    elem_type=models[0].elem_type, elem_mat=np.concatenate(emat).astype(np.int32),
                    mat_type=np.concatenate(mtyp).astype(np.int32), mat_param=np.concatenate(mpar),
                    thickness=np.concatenate(thick) if any_thick else None)
        if cs:
            out.con_slave = np.concatenate(cs).astype(np.int32)
            out.con_master = np.concatenate(cm).astype(np.int32)
            out.con_factor = np.concatenate(cf)
            out.con_ptr = np.concatenate([[0], np.cumsum(np.concatenate(cnt))]).astype(np.int32)
        return out

    def body_force(self, elem: int, q: Sequence[float]) -> np.ndarray:
        """rho * int(H^T q) over element `elem` (unit amplitude)."""
        nen = self.conn.shape[1]
        fe = np.zeros(nen * self.ndim)
        qa = as_f64(np.asarray(q, dtype=float))
        d = self.desc()
        check(lib().svl_element_body_force(C.byref(d), int(elem), ptr(qa, C.c_double), ptr(fe, C.c_double)))
        return fe

    def lumped_mass(self, mtol: float = 1e-12) -> np.ndarray:
        M = np.zeros(self.ntotal)
        d = self.desc()
        check(lib().svl_lumped_mass(C.byref(d), float(mtol), ptr(M, C.c_double)))
        return M


@dataclass
class Loads:
    """Time series plus force and support-motion entries (svl_load_desc)."""
    series: List[np.ndarray] = field(default_factory=list)
    force_dof: List[int] = field(default_factory=list)
    force_series: List[int] = field(default_factory=list)
    force_coef: List[float] = field(default_factory=list)
    sm_dof: List[int] = field(default_factory=list)
    sm_series: List[int] = field(default_factory=list)
    sm_factor: List[float] = field(default_factory=list)
    # domain-reduction (DRM) entries: element positions with their load factor,
    # and per node the free-field motion [nt, 3 ndim] (u, v, a) and the exterior flag
    drm_elem: List[int] = field(default_factory=list)
    drm_factor: List[float] = field(default_factory=list)
    drm_motion: dict = field(default_factory=dict)      # node position -> (ndarray [nt, 3 ndim], exterior flag)
    _nnode: int = field(default=0, repr=False)
    _keep: list = field(default_factory=list, repr=False)

    def add_drm(self, model: Model, elems: Sequence[int], motion: dict, factor: float = 1.0):
        """ELEMENTLOAD "GENERALWAVE": the elements of the DRM layer and, for every
        node of theirs, (free-field motion [nt, 3 ndim] as in the node file,
        exterior flag).  Exterior motions are negated inside, as the
        run-process does when it reads the files (Driver.hpp:1700-1719)."""
        self._nnode = model.nnode
        for e in elems:
            self.drm_elem.append(int(e))
            self.drm_factor.append(float(factor))
        for n, (sig, ext) in motion.items():
            self.drm_motion[int(n)] = (np.ascontiguousarray(sig, dtype=np.float64), 1 if ext else 0)

    def add_series(self, values) -> int:
        self.series.append(as_f64(values))
        return len(self.series) - 1

    def add_point_load(self, model: Model, node: int, direction: Sequence[float], series: int, factor: float = 1.0):
        """PointLoad on one node (Assembler.cpp:334-350): coef = factor * dir."""
        for j, v in enumerate(direction):
            if v != 0.0:
                self.force_dof.append(int(model.totaldof[node, j]))
                self.force_series.append(series)
                self.force_coef.append(factor * float(v))

    def add_body_load(self, model: Model, elems: Sequence[int], direction: Sequence[float], series: int,
                      factor: float = 1.0, element_force=None):
        """Element body load (Assembler.cpp:439-459) resolved to dof entries.
        element_force(e, direction) -> nodal vector of one element (default
        Model.body_force, the library's svl_element_body_force)."""
        nen = model.conn.shape[1]
        for e in elems:
            fe = (element_force or model.body_force)(int(e), direction)
            for a in range(nen):
                for j in range(model.ndim):
                    v = fe[a * model.ndim + j]
                    if v != 0.0:
                        self.force_dof.append(int(model.totaldof[model.conn[e, a], j]))
                        self.force_series.append(series)
                        self.force_coef.append(factor * v)

    def add_support_motion(self, model: Model, node: int, dof: int, series: int, factor: float = 1.0):
        self.sm_dof.append(int(model.totaldof[node, dof]))
        self.sm_series.append(series)
        self.sm_factor.append(float(factor))

    def external_force(self, ntotal: int, k: int) -> np.ndarray:
        """Fext(k) on total dofs from the force entries (point, body-point and
        element body loads already resolved to dofs): sum of coef * series[k],
        a series read past its end giving 0 (Assembler::ComputeExternalForceVector,
        Assembler.cpp:291-489).  Domain-reduction forces are computed on the
        device inside the step and are not covered here."""
        if self.drm_elem:
            raise ValueError("external_force: domain-reduction loads are not covered on the host")
        f = np.zeros(int(ntotal))
        for dof, s_, c in zip(self.force_dof, self.force_series, self.force_coef):
            ser = self.series[s_]
            if 0 <= k < ser.size:
                f[dof] += c * ser[k]
        return f

    @staticmethod
    def concat(parts: List["Loads"], models: List[Model]) -> "Loads":
        out = Loads()
        toff = 0
        for L, m in zip(parts, models):
            soff = len(out.series)
            out.series += L.series
            out.force_dof += [d + toff for d in L.force_dof]
            out.force_series += [s + soff for s in L.force_series]
            out.force_coef += L.force_coef
            out.sm_dof += [d + toff for d in L.sm_dof]
            out.sm_series += [s + soff for s in L.sm_series]
            out.sm_factor += L.sm_factor
            toff += m.ntotal
        return out

    def desc(self) -> capi.LoadDesc:
        sptr = np.zeros(len(self.series) + 1, np.int32)
        sptr[1:] = np.cumsum([s.size for s in self.series]) if self.series else []
        sval = np.concatenate(self.series) if self.series else np.zeros(1)
        arrs = [as_i32(sptr), as_f64(sval), as_i32(self.force_dof or [0]), as_i32(self.force_series or [0]),
                as_f64(self.force_coef or [0.0]), as_i32(self.sm_dof or [0]), as_i32(self.sm_series or [0]),
                as_f64(self.sm_factor or [0.0])]
        self._keep = arrs
        d = capi.LoadDesc()
        d.nseries = len(self.series)
        d.series_ptr = ptr(arrs[0], C.c_int32)
        d.series_val = ptr(arrs[1], C.c_double)
        d.nforce = len(self.force_dof)
        d.force_dof = ptr(arrs[2], C.c_int32)
        d.force_series = ptr(arrs[3], C.c_int32)
        d.force_coef = ptr(arrs[4], C.c_double)
        d.nsupport = len(self.sm_dof)
        d.sm_dof = ptr(arrs[5], C.c_int32)
        d.sm_series = ptr(arrs[6], C.c_int32)
        d.sm_factor = ptr(arrs[7], C.c_double)
        d.ndrm = len(self.drm_elem)
        if self.drm_elem:
            nnode = self._nnode
            rows = -np.ones(nnode, np.int32)
            ext = np.zeros(nnode, np.int32)
            nts = {sig.shape[0] for sig, _ in self.drm_motion.values()}
            if len(nts) != 1:
                raise ValueError("every DRM node needs the same number of rows")
            nt = nts.pop()
            blocks = []
            for i, n in enumerate(sorted(self.drm_motion)):
                sig, e = self.drm_motion[n]
                rows[n] = i
                ext[n] = e
                blocks.append(sig)
            extra = [as_i32(self.drm_elem), as_f64(self.drm_factor), rows, ext, as_f64(np.concatenate(blocks, axis=0))]
            self._keep += extra
            d.drm_elem = ptr(extra[0], C.c_int32)
            d.drm_factor = ptr(extra[1], C.c_double)
            d.drm_nt = int(nt)
            d.drm_node_row = ptr(extra[2], C.c_int32)
            d.drm_node_ext = ptr(extra[3], C.c_int32)
            d.drm_motion = ptr(extra[4], C.c_double)
        return d


def ricker(nt: int, dt: float, f0: float, t0: Optional[float] = None, amp: float = 1.0) -> np.ndarray:
    """Ricker wavelet Ap (1 - 2 beta) exp(-beta), beta = (pi f0 (t - t0))^2
    (the 'VEL' form of PP/Core/PlaneWave.py:222-223), sampled at k*dt."""
    if t0 is None:
        t0 = 1.2 / f0
    t = np.arange(nt) * dt
    beta = (np.pi * f0 * (t - t0)) ** 2
    return amp * (1.0 - 2.0 * beta) * np.exp(-beta)


def elastic_params(ndim: int, E: float, nu: float, rho: float) -> np.ndarray:
    return np.array([E, nu, rho, 0, 0, 0, 0, 0], dtype=float)


def j2_params(K: float, G: float, rho: float, H: float, beta: float, sigma_y: float) -> np.ndarray:
    return np.array([K, G, rho, H, beta, sigma_y, 0, 0], dtype=float)
