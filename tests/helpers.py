"""Shared model builders for the tests (small, seeded)."""
from __future__ import annotations

import numpy as np

from svl_gb300 import _capi as capi
from svl_gb300.model import Loads, Model, elastic_params, j2_params, ricker


def rel_l2(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def q4_box(nx=20, ny=10, h=1.0, E=2.0e8, nu=0.25, rho=2000.0, amp=1.0e6, f0=5.0, dt=None, nt=400):
    """Config-1 style plane-strain box: fixed bottom, x-roller sides, vertical
    Ricker point load at the top-centre node."""
    m = Model.grid(2, (nx, ny), (h, h), fix_mask=(1, 1, 3, 0, 0, 0),
                   mat_type=np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN], np.int32),
                   mat_param=elastic_params(2, E, nu, rho)[None, :])
    G = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    vp = np.sqrt((lam + 2 * G) / rho)
    if dt is None:
        dt = 0.5 * h / vp
    L = Loads()
    s = L.add_series(ricker(nt + 1, dt, f0, amp=amp))
    top_centre = ny * (nx + 1) + nx // 2
    L.add_point_load(m, top_centre, (0.0, -1.0), s)
    return m, L, dt


def h8_box(nx=6, ny=5, nz=4, h=2.0, seed=0, amp=1.0e7, f0=3.0, nt=300, heterogeneous=True):
    """Config-2 style box (no PML): fixed bottom, rollers on the sides, a
    per-element random Vs field and a pair of opposite body loads."""
    rng = np.random.default_rng(seed)
    ne = nx * ny * nz
    rho, nu = 2100.0, 0.3
    vs = 400.0 * np.exp(0.198 * rng.standard_normal(ne) - 0.5 * 0.198 ** 2) if heterogeneous else np.full(ne, 400.0)
    G = rho * vs ** 2
    E = 2 * G * (1 + nu)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2] = E, nu, rho
    m = Model.grid(3, (nx, ny, nz), (h, h, h), fix_mask=(1, 1, 2, 2, 7, 0),
                   mat_type=np.full(ne, capi.SVL_MAT_ELASTIC3DLINEAR, np.int32), mat_param=mp,
                   elem_mat=np.arange(ne, dtype=np.int32))
    vp = np.sqrt(E.max() * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho)
    dt = 0.5 * h / vp
    L = Loads()
    s = L.add_series(ricker(nt + 1, dt, f0, amp=1.0))
    c = (nz // 2) * nx * ny + (ny // 2) * nx + nx // 2
    L.add_body_load(m, [c], (amp, 0.0, 0.0), s)
    c2 = c + nx if c + nx < ne else c - 1
    L.add_body_load(m, [c2], (-amp, 0.0, 0.0), s)
    return m, L, dt


def q4_j2_columns(ncol=3, width=4, heights=(6, 9, 12), h=0.5, seed=1, nt=300, pga=3.0):
    """Config-3 style ensemble: J2 plane-strain soil columns with periodic
    sides and a base support motion, one instance per column."""
    rng = np.random.default_rng(seed)
    models, loads = [], []
    dts = []
    for c in range(ncol):
        ny = heights[c % len(heights)]
        vs = rng.uniform(150, 500)
        rho, nu = 2000.0, 0.3
        G = rho * vs ** 2
        K = 2 * G * (1 + nu) / (3 * (1 - 2 * nu))
        su = rng.uniform(30e3, 120e3)
        m = Model.grid(2, (width, ny), (h, h), fix_mask=(0, 0, 3, 0, 0, 0), periodic_x=True,
                       mat_type=np.array([capi.SVL_MAT_PLASTICPLANESTRAINJ2], np.int32),
                       mat_param=j2_params(K, G, rho, 0.02 * G, 1.0, np.sqrt(3.0) * su)[None, :])
        vp = np.sqrt((K + 4 * G / 3) / rho)
        dts.append(0.5 * h / vp)
        models.append(m)
    dt = min(dts)
    for c, m in enumerate(models):
        L = Loads()
        t = np.arange(nt + 1) * dt
        f1, f2 = rng.uniform(1, 4), rng.uniform(5, 12)
        disp = pga / (2 * np.pi * f1) ** 2 * (np.sin(2 * np.pi * f1 * t) * np.exp(-t * 2.0)
                                              + 0.3 * np.sin(2 * np.pi * f2 * t)) * (1 - np.exp(-(t / 0.02) ** 2))
        s = L.add_series(disp)
        for i in range(width + 1):
            L.add_support_motion(m, i, 0, s)
        loads.append(L)
    return Model.concat(models), Loads.concat(loads, models), dt


def pml_box(ndim=2, ni=(6, 4), npml=2, h=1.0, E=2.0e8, nu=0.25, rho=2000.0, nt=80, amp=1.0e6, f0=8.0,
            dt_factor=2.0, R=1.0e-6, mexp=2.0, lumped=True):
    """Elastic box with PML layers on the lateral sides and the bottom
    (PML2DQuad4 / PML3DHexa8 with 5 / 9 dofs at their nodes), the outer PML
    boundary fixed in displacement, a Ricker point load at the top centre.
    Geometry and connectivity from the grid generator; dofs numbered node by
    node with each node's own count (PlainScheme order)."""
    pnd = 5 if ndim == 2 else 9
    ne = [ni[0] + 2 * npml, ni[1] + npml] if ndim == 2 else [ni[0] + 2 * npml, ni[1] + 2 * npml, ni[2] + npml]
    mt = capi.SVL_MAT_ELASTIC2DPLANESTRAIN if ndim == 2 else capi.SVL_MAT_ELASTIC3DLINEAR
    g = Model.grid(ndim, ne, (h,) * ndim, mat_type=np.array([mt], np.int32),
                   mat_param=elastic_params(ndim, E, nu, rho)[None, :])
    nel = g.nelem
    # element grid indices (generator order: x fastest)
    idx = np.stack(np.unravel_index(np.arange(nel), ne[::-1])[::-1], axis=1)
    vert = ndim - 1
    lo = [npml * h] * ndim
    hi = [(npml + ni[d]) * h for d in range(ndim)]
    par = np.zeros((nel, 3 + 2 * ndim))
    epml = np.zeros(nel, np.int32)
    for e in range(nel):
        n = np.zeros(ndim)
        x0 = np.zeros(ndim)
        for d in range(ndim):
            i = idx[e, d]
            if i < npml:
                n[d], x0[d] = -1.0, lo[d]
            elif d != vert and i >= ne[d] - npml:
                n[d], x0[d] = 1.0, hi[d]
        if np.any(n != 0):
            epml[e] = 1
            par[e] = np.concatenate([[mexp, npml * h, R], x0, n])
    pnode = np.zeros(g.nnode, bool)
    pnode[g.conn[epml == 1].ravel()] = True
    ndof_n = np.where(pnode, pnd, ndim).astype(np.int32)
    tdof = -np.ones((g.nnode, pnd), np.int32)
    fdof = -np.ones((g.nnode, pnd), np.int32)
    X = g.coords
    outer = np.zeros(g.nnode, bool)
    for d in range(ndim):
        outer |= np.isclose(X[:, d], 0.0) if d == vert else (np.isclose(X[:, d], 0.0) | np.isclose(X[:, d], ne[d] * h))
    t = f = 0
    for nd_ in range(g.nnode):
        for j in range(ndof_n[nd_]):
            tdof[nd_, j] = t
            t += 1
            if not (outer[nd_] and j < ndim):
                fdof[nd_, j] = f
                f += 1
    m = Model(ndim=ndim, coords=X, totaldof=tdof, freedof=fdof, conn=g.conn, elem_type=g.elem_type,
              elem_mat=g.elem_mat, mat_type=g.mat_type, mat_param=g.mat_param, lumped=lumped,
              node_ndof=ndof_n, elem_pml=epml, pml_param=par)
    G = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    vp = np.sqrt((lam + 2 * G) / rho)
    dt = dt_factor * h / vp
    L = Loads()
    s = L.add_series(ricker(nt + 1, dt, f0, amp=amp))
    top = np.flatnonzero(np.isclose(X[:, vert], ne[vert] * h))
    c = top[np.argmin(np.sum((X[top, :vert] - np.array(hi[:vert]) / 2 - np.array(lo[:vert]) / 2) ** 2, axis=1))]
    L.add_point_load(m, int(c), tuple([0.0] * vert + [-1.0]), s)
    return m, L, dt


def pml_j2_box(ndim=2, ni=(10, 6), npml=2, nj2=3, su=15e3, **kw):
    """pml_box whose solid elements in the top `nj2` element layers carry a
    J2 material with the same elastic moduli (H = 0.02 G, beta = 0.5, pure
    shear yield su): plastic layers over an elastic half-space with PML."""
    m, L, dt = pml_box(ndim, ni, npml=npml, **kw)
    E, nu, rho = m.mat_param[0, :3]
    G = E / (2 * (1 + nu))
    K = E / (3 * (1 - 2 * nu))
    mt = capi.SVL_MAT_PLASTICPLANESTRAINJ2 if ndim == 2 else capi.SVL_MAT_PLASTIC3DJ2
    m.mat_type = np.array([m.mat_type[0], mt], np.int32)
    m.mat_param = np.vstack([m.mat_param[0], j2_params(K, G, rho, 0.02 * G, 0.5, np.sqrt(3.0) * su)])
    vert = ndim - 1
    X = m.coords
    h = kw.get("h", 1.0)
    ytop = X[:, vert].max()
    emat = np.array(m.elem_mat, np.int32)
    for e in range(m.nelem):
        if not m.elem_pml[e] and X[m.conn[e], vert].min() >= ytop - nj2 * h - 1e-9:
            emat[e] = 1
    m.elem_mat = emat
    return m, L, dt


def lysmer_box(nx=12, ny=6, h=1.0, E=2.0e8, nu=0.25, rho=2000.0, nt=200, amp=1.0e6, f0=8.0, dt_factor=0.5):
    """Plane-strain box whose sides and bottom are free but held by Lysmer
    dashpots (ZeroLength1D + Viscous1DLinear) to anchor nodes that are fixed:
    normal dashpots rho Vp h and tangential rho Vs h per boundary node (half on
    corner-adjacent edges is not attempted; the test needs only the operator)."""
    m = Model.grid(2, (nx, ny), (h, h), mat_type=np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN], np.int32),
                   mat_param=elastic_params(2, E, nu, rho)[None, :])
    G = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    vp, vs = np.sqrt((lam + 2 * G) / rho), np.sqrt(G / rho)
    X = m.coords
    bnodes = [n for n in range(m.nnode) if np.isclose(X[n, 1], 0) or np.isclose(X[n, 0], 0) or np.isclose(X[n, 0], nx * h)]
    nn0 = m.nnode
    na = len(bnodes)
    coords = np.vstack([X, X[bnodes]])
    tdof = np.vstack([m.totaldof, (m.ntotal + np.arange(2 * na)).reshape(na, 2)]).astype(np.int32)
    fdof = np.vstack([m.freedof, -np.ones((na, 2), np.int32)]).astype(np.int32)
    dof, eta = [], []
    for i, n in enumerate(bnodes):
        a = nn0 + i
        bottom = np.isclose(X[n, 1], 0)
        for j in range(2):
            normal = (j == 1) if bottom else (j == 0)
            dof.append((int(m.totaldof[n, j]), int(tdof[a, j])))
            eta.append(rho * (vp if normal else vs) * h)
    m2 = Model(ndim=2, coords=coords, totaldof=tdof, freedof=fdof, conn=m.conn, elem_type=m.elem_type,
               elem_mat=m.elem_mat, mat_type=m.mat_type, mat_param=m.mat_param, lumped=True,
               dashpot_dof=np.array(dof, np.int32), dashpot_eta=np.array(eta))
    dt = dt_factor * h / vp
    L = Loads()
    s = L.add_series(ricker(nt + 1, dt, f0, amp=amp))
    top = ny * (nx + 1) + nx // 2
    L.add_point_load(m2, top, (0.0, -1.0), s)
    return m2, L, dt


def drm_box(nx=12, ny=8, h=1.0, E=2.0e8, nu=0.25, rho=2000.0, nt=120, dt_factor=0.5, f0=6.0, seed=0):
    """Plane-strain box with a one-element domain-reduction layer: the ring of
    elements one element in from the sides and bottom; its inner nodes are the
    boundary nodes, its outer nodes the exterior ones.  The free field is a
    vertically travelling SV pulse u_x = g(t - y/Vs) (with v, a by finite
    differences of the same expression), seeded amplitude."""
    m = Model.grid(2, (nx, ny), (h, h), fix_mask=(1, 1, 3, 0, 0, 0),
                   mat_type=np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN], np.int32),
                   mat_param=elastic_params(2, E, nu, rho)[None, :])
    G = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    vp, vs = np.sqrt((lam + 2 * G) / rho), np.sqrt(G / rho)
    dt = dt_factor * h / vp
    X = m.coords
    xmin, xmax, ymin = h, (nx - 1) * h, h
    inner = lambda p: (p[0] >= xmin - 1e-9) and (p[0] <= xmax + 1e-9) and (p[1] >= ymin - 1e-9)  # noqa: E731
    elems = []
    for e in range(m.nelem):
        c = X[m.conn[e]]
        ins = [inner(p) for p in c]
        if any(ins) and not all(ins):
            elems.append(e)
    nodes = sorted(set(int(n) for e in elems for n in m.conn[e]))
    amp = 1e-3 * (1.0 + np.random.default_rng(seed).random())
    t = np.arange(nt + 2) * dt
    def g(tau):
        a = (np.pi * f0 * (tau - 1.2 / f0)) ** 2
        return amp * (1 - 2 * a) * np.exp(-a)
    motion = {}
    for n in nodes:
        y = X[n, 1]
        u = g(t - (ny * h - y) / vs)
        v = np.gradient(u, dt)
        a = np.gradient(v, dt)
        sig = np.zeros((nt + 2, 6))
        sig[:, 0], sig[:, 2], sig[:, 4] = u, v, a
        motion[n] = (sig, not inner(X[n]))
    L = Loads()
    L.add_drm(m, elems, motion, factor=1.0)
    return m, L, dt, elems, motion
