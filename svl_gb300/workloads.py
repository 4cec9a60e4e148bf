"""Seeded synthetic models with the shapes and value distributions of the
benchmark configurations (no reference data is used):

* config1: 200 x 100 lin2DQuad4 plane-strain box, h = 1 m, rho = 2000,
  Vs = 200, nu = 0.25, fixed bottom, x-roller sides, vertical Ricker
  (f0 = 5 Hz) point load at the top-centre node, dt = 0.5 h / Vp.
* config2: 128 x 128 x 64 lin3DHexa8 box, h = 2 m, Vs log-normal (mean 400,
  COV 0.2, exponential correlation 20 m), nu = 0.3, rho = 2100,
  double-couple-like body force (four element groups) with a Ricker
  f0 = 3 Hz, dt = 0.5 h / max Vp.  config2_pml: the configuration as
  specified, whose outer 10 element layers on the four sides and the bottom
  are PML3DHexa8 (9 dofs at their nodes, the pre-processor's reference points
  and normals, the outer PML boundary fixed in displacement); config2: the
  same box with a fixed bottom and roller sides instead of the PML band.
* config3: an ensemble of 2D plane-strain soil columns, 10 lin2DQuad4
  elements wide, heights uniform in [50, 400] elements of 0.5 m (seeded),
  PlasticPlaneStrainJ2 (G = rho Vs^2 with Vs uniform in [150, 500] m/s,
  su uniform in [30, 120] kPa, Sy = sqrt(3) su, H = 0.02 G, beta = 1,
  rho = 2000, nu = 0.3), periodic side nodes (EQUAL constraints), fixed base
  driven by a horizontal support motion: band-limited (0.1-20 Hz) white-noise
  acceleration scaled to a PGA uniform in [0.1, 0.5] g, integrated twice in
  the frequency domain.  dt = min(5e-4, 0.5 h / max Vp): 5e-4 s exceeds the
  explicit limit of the stiffest columns, so the stable step is used.
* config4: 64 x 64 x 64 lin3DHexa8 box, h = 1 m, seeded piecewise-layered
  shear modulus (layer contrast up to 100x) times 10% log-normal noise per
  element, nu = 0.3, rho = 2000, Newmark average acceleration at
  dt = 10 x the explicit limit h / max Vp, the same double-couple Ricker
  source (f0 = 3 Hz); fixed bottom, rollers on the sides.
* config5: lin3DHexa8 grid (h = 2 m) whose top layers are Plastic3DJ2 (su
  40-150 kPa by depth) over an elastic base; the half-space below is
  represented by Lysmer dashpots on the base nodes (the SPD alternative to a
  PML half-space for PCG), the incident band-limited plane wave (0.1-10 Hz,
  PGA 0.3 g) by the Lysmer input force; Newmark-Newton.
"""
from __future__ import annotations

import numpy as np

from . import _capi as capi
from .model import Loads, Model, ricker


def lognormal_field(shape, h, mean, cov, corr_len, seed):
    """Log-normal field with exponential correlation, by spectral synthesis
    of a Gaussian field on the element grid (periodic embedding on a grid
    padded by one correlation length)."""
    rng = np.random.default_rng(seed)
    pad = [int(s + np.ceil(corr_len / h)) for s in shape]
    white = rng.standard_normal(pad)
    ks = np.meshgrid(*[np.fft.fftfreq(n, d=h) * 2 * np.pi for n in pad], indexing="ij")
    k2 = sum(k * k for k in ks)
    d = len(shape)
    # spectral density of exp(-r/l) in d dimensions ~ (1 + k^2 l^2)^(-(d+1)/2)
    psd = (1.0 + k2 * corr_len ** 2) ** (-(d + 1) / 2.0)
    g = np.real(np.fft.ifftn(np.fft.fftn(white) * np.sqrt(psd)))
    g = g[tuple(slice(0, s) for s in shape)]
    g = (g - g.mean()) / g.std()
    sigma = np.sqrt(np.log(1.0 + cov ** 2))
    mu = np.log(mean) - 0.5 * sigma ** 2
    return np.exp(mu + sigma * g)


def config1(nx=200, ny=100, nt=2001, amp=1.0e6):
    h, rho, vs, nu = 1.0, 2000.0, 200.0, 0.25
    G = rho * vs ** 2
    E = 2 * G * (1 + nu)
    m = Model.grid(2, (nx, ny), (h, h), fix_mask=(1, 1, 3, 0, 0, 0),
                   mat_type=np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN], np.int32),
                   mat_param=np.array([[E, nu, rho, 0, 0, 0, 0, 0]]))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    vp = np.sqrt((lam + 2 * G) / rho)
    dt = 0.5 * h / vp
    L = Loads()
    s = L.add_series(ricker(nt, dt, 5.0, amp=amp))
    L.add_point_load(m, ny * (nx + 1) + nx // 2, (0.0, -1.0), s)
    return m, L, dt


def config2(nx=128, ny=128, nz=64, nt=4001, seed=0, amp=1.0e3):
    h, rho, nu = 2.0, 2100.0, 0.3
    vs = lognormal_field((nx, ny, nz), h, 400.0, 0.2, 20.0, seed)
    # element order: x fastest, then y, then z (Builder.py:167-183)
    vs_e = np.transpose(vs, (2, 1, 0)).reshape(-1)
    ne = nx * ny * nz
    G = rho * vs_e ** 2
    E = 2 * G * (1 + nu)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2] = E, nu, rho
    m = Model.grid(3, (nx, ny, nz), (h, h, h), fix_mask=(1, 1, 2, 2, 7, 0),
                   mat_type=np.full(ne, capi.SVL_MAT_ELASTIC3DLINEAR, np.int32), mat_param=mp,
                   elem_mat=np.arange(ne, dtype=np.int32))
    vp_max = np.sqrt(E.max() * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho)
    dt = 0.5 * h / vp_max
    L = Loads()
    s = L.add_series(ricker(nt, dt, 3.0, amp=1.0))
    cx, cy, cz = nx // 2, ny // 2, nz // 2

    def eid(i, j, k):
        return (k * ny + j) * nx + i
    # double couple: +x on the element above, -x below; +y right, -y left
    L.add_body_load(m, [eid(cx, cy + 1, cz)], (amp, 0.0, 0.0), s)
    L.add_body_load(m, [eid(cx, cy - 1, cz)], (-amp, 0.0, 0.0), s)
    L.add_body_load(m, [eid(cx + 1, cy, cz)], (0.0, amp, 0.0), s)
    L.add_body_load(m, [eid(cx - 1, cy, cz)], (0.0, -amp, 0.0), s)
    return m, L, dt


def layered_stiffness(nz, n_layers, contrast, seed):
    """Per-element-layer shear modulus factor: n_layers seeded layers of
    random thickness, log-uniform factors in [1, contrast] (the softest and
    stiffest layers pinned to 1 and `contrast`)."""
    rng = np.random.default_rng(seed)
    cuts = np.sort(rng.choice(np.arange(1, nz), size=n_layers - 1, replace=False))
    f = np.exp(rng.uniform(0.0, np.log(contrast), n_layers))
    f[np.argmin(f)], f[np.argmax(f)] = 1.0, contrast
    layer = np.searchsorted(cuts, np.arange(nz), side="right")
    return f[layer]


def config4(nx=64, ny=64, nz=64, nt=501, seed=0, amp=1.0e3, contrast=100.0, n_layers=6):
    h, rho, nu, vs_soft = 1.0, 2000.0, 0.3, 100.0
    rng = np.random.default_rng(seed + 1)
    ne = nx * ny * nz
    fz = layered_stiffness(nz, n_layers, contrast, seed)          # [nz]
    noise = np.exp(0.1 * rng.standard_normal(ne) - 0.5 * 0.1 ** 2)
    k = np.arange(ne) // (nx * ny)                                   # element layer (x fastest)
    G = rho * vs_soft ** 2 * fz[k] * noise
    E = 2 * G * (1 + nu)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2] = E, nu, rho
    m = Model.grid(3, (nx, ny, nz), (h, h, h), fix_mask=(1, 1, 2, 2, 7, 0),
                   mat_type=np.full(ne, capi.SVL_MAT_ELASTIC3DLINEAR, np.int32), mat_param=mp,
                   elem_mat=np.arange(ne, dtype=np.int32))
    vp_max = np.sqrt(E.max() * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho)
    dt = 10.0 * h / vp_max
    L = Loads()
    s = L.add_series(ricker(nt, dt, 3.0, amp=1.0))
    cx, cy, cz = nx // 2, ny // 2, nz // 2

    def eid(i, j, kk):
        return (kk * ny + j) * nx + i
    L.add_body_load(m, [eid(cx, cy + 1, cz)], (amp, 0.0, 0.0), s)
    L.add_body_load(m, [eid(cx, cy - 1, cz)], (-amp, 0.0, 0.0), s)
    L.add_body_load(m, [eid(cx + 1, cy, cz)], (0.0, amp, 0.0), s)
    L.add_body_load(m, [eid(cx - 1, cy, cz)], (0.0, -amp, 0.0), s)
    return m, L, dt


def base_motion(nt, dt, f_lo, f_hi, pga, rng):
    """Displacement whose second derivative is band-limited white noise with
    peak |acceleration| = pga (spectral double integration, no drift)."""
    n = int(2 ** np.ceil(np.log2(max(nt, 2))))
    w = rng.standard_normal(n)
    W = np.fft.rfft(w)
    f = np.fft.rfftfreq(n, dt)
    band = (f >= f_lo) & (f <= f_hi)
    W[~band] = 0.0
    acc = np.fft.irfft(W, n)[:nt]
    acc *= pga / max(np.abs(acc).max(), 1e-300)
    Wa = np.fft.rfft(np.concatenate([acc, np.zeros(n - nt)]))
    om = 2 * np.pi * f
    D = np.zeros_like(Wa)
    D[band] = -Wa[band] / om[band] ** 2
    return np.fft.irfft(D, n)[:nt]


def config3(ncol=256, seed=0, nt=None, width=10, h=0.5, duration=20.0, hmin=50, hmax=400):
    """Returns (model, loads, dt, info) of the whole ensemble as one model
    (columns concatenated; instances never interact)."""
    from .model import j2_params
    rng = np.random.default_rng(seed)
    rho, nu = 2000.0, 0.3
    heights = rng.integers(hmin, hmax + 1, ncol)
    vs = rng.uniform(150.0, 500.0, ncol)
    su = rng.uniform(30e3, 120e3, ncol)
    pga = rng.uniform(0.1, 0.5, ncol) * 9.81
    vp = vs * np.sqrt(2 * (1 - nu) / (1 - 2 * nu))
    dt = min(5e-4, 0.5 * h / vp.max())
    if nt is None:
        nt = int(round(duration / dt)) + 1
    models = []
    for c in range(ncol):
        G = rho * vs[c] ** 2
        K = 2 * G * (1 + nu) / (3 * (1 - 2 * nu))
        m = Model.grid(2, (width, int(heights[c])), (h, h), fix_mask=(0, 0, 3, 0, 0, 0), periodic_x=True,
                       mat_type=np.array([capi.SVL_MAT_PLASTICPLANESTRAINJ2], np.int32),
                       mat_param=j2_params(K, G, rho, 0.02 * G, 1.0, np.sqrt(3.0) * su[c])[None, :])
        models.append(m)
    loads = []
    for c, m in enumerate(models):
        L = Loads()
        s = L.add_series(base_motion(nt, dt, 0.1, 20.0, pga[c], rng))
        for i in range(width + 1):
            L.add_support_motion(m, i, 0, s)
        loads.append(L)
    info = {"columns": ncol, "elements": int(sum(x.nelem for x in models)), "dt": dt, "nt": nt,
            "heights": [int(heights.min()), int(heights.max())]}
    return Model.concat(models), Loads.concat(loads, models), dt, info


def config5(nx=128, ny=128, nz=64, n_j2=16, nt=301, seed=0, h=2.0, pga=0.3 * 9.81):
    """Nonlinear implicit model: lin3DHexa8 grid, the top `n_j2` element
    layers Plastic3DJ2 (su uniform in [40, 150] kPa by depth, seeded; H =
    0.02 G, beta = 1), elastic below; Vs 300 m/s (J2 layers 200 m/s), nu = 0.3,
    rho = 2000.  The half-space below is represented by Lysmer dashpots on the
    base nodes (rho Vs A tangential, rho Vp A normal, A the node's base area)
    tied to fixed anchor nodes, which keeps the effective stiffness SPD; the
    incident plane wave (band-limited 0.1-10 Hz, PGA `pga`) enters as the
    Lysmer input force 2 rho Vs A v_in(t) in x on the base nodes.  Sides:
    rollers.  dt = 0.5 h / Vp of the elastic layers."""
    from .model import j2_params
    rng = np.random.default_rng(seed + 5)
    rho, nu = 2000.0, 0.3
    vs_el, vs_j2 = 300.0, 200.0
    ne = nx * ny * nz
    k = np.arange(ne) // (nx * ny)                     # element layer, 0 at the base
    j2 = k >= nz - n_j2
    mp = np.zeros((ne, 8))
    mt = np.where(j2, capi.SVL_MAT_PLASTIC3DJ2, capi.SVL_MAT_ELASTIC3DLINEAR).astype(np.int32)
    G_el, G_j2 = rho * vs_el ** 2, rho * vs_j2 ** 2
    E_el = 2 * G_el * (1 + nu)
    K_j2 = 2 * G_j2 * (1 + nu) / (3 * (1 - 2 * nu))
    su_layer = np.sort(rng.uniform(40e3, 150e3, n_j2))[::-1]          # stiffer with depth
    for e in np.flatnonzero(~j2):
        mp[e, :3] = (E_el, nu, rho)
    for e in np.flatnonzero(j2):
        layer = nz - 1 - k[e]
        mp[e] = j2_params(K_j2, G_j2, rho, 0.02 * G_j2, 1.0, np.sqrt(3.0) * su_layer[layer])
    g = Model.grid(3, (nx, ny, nz), (h, h, h), fix_mask=(1, 1, 2, 2, 0, 0),
                   mat_type=mt, mat_param=mp, elem_mat=np.arange(ne, dtype=np.int32))
    vp = vs_el * np.sqrt(2 * (1 - nu) / (1 - 2 * nu))
    dt = 0.5 * h / vp
    X = g.coords
    base = np.flatnonzero(np.isclose(X[:, 2], 0.0))
    nb = base.size
    nn0 = g.nnode
    coords = np.vstack([X, X[base]])
    tdof = np.vstack([g.totaldof, (g.ntotal + np.arange(3 * nb)).reshape(nb, 3)]).astype(np.int32)
    fdof = np.vstack([g.freedof, -np.ones((nb, 3), np.int32)]).astype(np.int32)
    ix = np.rint(X[base, 0] / h).astype(int)
    iy = np.rint(X[base, 1] / h).astype(int)
    area = h * h * np.where((ix == 0) | (ix == nx), 0.5, 1.0) * np.where((iy == 0) | (iy == ny), 0.5, 1.0)
    dof, eta = [], []
    for i, n in enumerate(base):
        for j in range(3):
            dof.append((int(g.totaldof[n, j]), int(tdof[nn0 + i, j])))
            eta.append(rho * (vp if j == 2 else vs_el) * area[i])
    m = Model(ndim=3, coords=coords, totaldof=tdof, freedof=fdof, conn=g.conn, elem_type=g.elem_type,
              elem_mat=g.elem_mat, mat_type=g.mat_type, mat_param=g.mat_param, lumped=True,
              dashpot_dof=np.array(dof, np.int32), dashpot_eta=np.array(eta))
    # the record is synthesised over 20 s (frequency resolution for the 0.1-10 Hz
    # band) and the first nt + 2 samples are used
    disp = base_motion(max(nt + 2, int(20.0 / dt)), dt, 0.1, 10.0, pga, rng)[:nt + 2]
    v_in = np.gradient(disp, dt)
    L = Loads()
    s = L.add_series(v_in)
    for i, n in enumerate(base):
        if g.freedof[n, 0] >= 0:
            L.force_dof.append(int(g.totaldof[n, 0]))
            L.force_series.append(s)
            L.force_coef.append(2.0 * rho * vs_el * area[i])
    return m, L, dt


def config5_pml(nx=128, ny=128, nz=64, npml=10, n_j2=16, nt=301, seed=0, h=2.0, pga=0.3 * 9.81, pml_m=2.0,
                pml_R=1.0e-6):
    """Nonlinear implicit model with a PML half-space: lin3DHexa8 grid of
    nx x ny x nz elements whose outer `npml` element layers on the four sides
    and the bottom are PML3DHexa8 (9 dofs at their nodes; n = pml_m, L = npml h,
    R = pml_R; the outer PML boundary fixed in displacement); the top `n_j2`
    layers of the solid region Plastic3DJ2 (su uniform in [40, 150] kPa by
    depth, seeded; H = 0.02 G, beta = 1), elastic below (Vs 300 m/s, J2
    layers 200 m/s, nu = 0.3, rho = 2000).  The band-limited plane wave
    (0.1-10 Hz, PGA `pga`) enters as the x force 2 rho Vs A v_in(t) on the
    solid nodes of the plane two elements above the bottom PML (an up-going
    plane-wave source; the down-going half leaves through the bottom PML).
    Dofs numbered node by node with each node's own count (PlainScheme
    order).  dt = 0.5 h / Vp of the elastic layers."""
    from .model import j2_params
    rng = np.random.default_rng(seed + 55)
    rho, nu = 2000.0, 0.3
    vs_el, vs_j2 = 300.0, 200.0
    ne = nx * ny * nz
    e = np.arange(ne)
    ix, iy, iz = e % nx, (e // nx) % ny, e // (nx * ny)
    # PML normal and reference point per element
    nvec = np.zeros((ne, 3))
    x0 = np.zeros((ne, 3))
    lo, hi = npml * h, np.array([nx - npml, ny - npml]) * h
    for d, i, n in ((0, ix, nx), (1, iy, ny)):
        m_lo, m_hi = i < npml, i >= n - npml
        nvec[m_lo, d], x0[m_lo, d] = -1.0, lo
        nvec[m_hi, d], x0[m_hi, d] = 1.0, hi[d]
    m_bot = iz < npml
    nvec[m_bot, 2], x0[m_bot, 2] = -1.0, lo
    epml = np.any(nvec != 0.0, axis=1).astype(np.int32)
    par = np.zeros((ne, 9))
    par[:, 0], par[:, 1], par[:, 2] = pml_m, npml * h, pml_R
    par[:, 3:6], par[:, 6:9] = x0, nvec
    par[epml == 0] = 0.0
    # materials: J2 in the top n_j2 layers of the solid region, elastic elsewhere
    j2 = (iz >= nz - n_j2) & (epml == 0)
    mt = np.where(j2, capi.SVL_MAT_PLASTIC3DJ2, capi.SVL_MAT_ELASTIC3DLINEAR).astype(np.int32)
    G_el, G_j2 = rho * vs_el ** 2, rho * vs_j2 ** 2
    E_el = 2 * G_el * (1 + nu)
    K_j2 = 2 * G_j2 * (1 + nu) / (3 * (1 - 2 * nu))
    su_layer = np.sort(rng.uniform(40e3, 150e3, n_j2))[::-1]
    mp = np.zeros((ne, 8))
    mp[~j2, 0], mp[~j2, 1], mp[~j2, 2] = E_el, nu, rho
    layer = nz - 1 - iz[j2]
    H = 0.02 * G_j2
    mp[j2] = np.stack([np.full(layer.size, K_j2), np.full(layer.size, G_j2), np.full(layer.size, rho),
                       np.full(layer.size, H), np.ones(layer.size), np.sqrt(3.0) * su_layer[layer],
                       np.zeros(layer.size), np.zeros(layer.size)], axis=1)
    g = Model.grid(3, (nx, ny, nz), (h, h, h), mat_type=mt, mat_param=mp, elem_mat=np.arange(ne, dtype=np.int32))
    # dofs: 9 at the nodes of PML elements, 3 elsewhere, node by node
    nn = g.nnode
    pnode = np.zeros(nn, bool)
    pnode[g.conn[epml == 1].ravel()] = True
    ndof_n = np.where(pnode, 9, 3).astype(np.int32)
    X = g.coords
    outer = (np.isclose(X[:, 0], 0.0) | np.isclose(X[:, 0], nx * h) | np.isclose(X[:, 1], 0.0)
             | np.isclose(X[:, 1], ny * h) | np.isclose(X[:, 2], 0.0))
    j = np.arange(9)[None, :]
    has = j < ndof_n[:, None]
    off = np.concatenate([[0], np.cumsum(ndof_n)[:-1]]).astype(np.int64)
    tdof = np.where(has, off[:, None] + j, -1).astype(np.int32)
    free = has & ~(outer[:, None] & (j < 3))
    fdof = np.full((nn, 9), -1, np.int64)
    fdof[free] = np.arange(int(free.sum()))          # row-major = node by node
    m = Model(ndim=3, coords=X, totaldof=tdof, freedof=fdof.astype(np.int32), conn=g.conn, elem_type=g.elem_type,
              elem_mat=g.elem_mat, mat_type=g.mat_type, mat_param=g.mat_param, lumped=True,
              node_ndof=ndof_n, elem_pml=epml, pml_param=par)
    vp = vs_el * np.sqrt(2 * (1 - nu) / (1 - 2 * nu))
    dt = 0.5 * h / vp
    disp = base_motion(max(nt + 2, int(20.0 / dt)), dt, 0.1, 10.0, pga, rng)[:nt + 2]
    v_in = np.gradient(disp, dt)
    L = Loads()
    s = L.add_series(v_in)
    zs = (npml + 2) * h
    src = np.flatnonzero(np.isclose(X[:, 2], zs) & ~pnode)
    for n in src:
        L.force_dof.append(int(tdof[n, 0]))
        L.force_series.append(s)
        L.force_coef.append(2.0 * rho * vs_el * h * h)
    return m, L, dt


def grid_nodes_conn(ne, h):
    """Node coordinates (x fastest) and lin3DHexa8 connectivity of an
    nx x ny x nz box (PP/Method/Builder.py makeDomainVolume: nodes x-fastest,
    element nodes n1..n8 as Builder.py:167-183), in numpy."""
    nx, ny, nz = ne
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    X = np.stack([i.transpose(2, 1, 0).ravel() * h, j.transpose(2, 1, 0).ravel() * h,
                  k.transpose(2, 1, 0).ravel() * h], axis=1).astype(np.float64)
    ei, ej, ek = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ei, ej, ek = (a.transpose(2, 1, 0).ravel() for a in (ei, ej, ek))
    layer = (nx + 1) * (ny + 1)
    n1 = layer * ek + ej * (nx + 1) + ei
    conn = np.stack([n1, n1 + 1, n1 + 1 + (nx + 1), n1 + (nx + 1),
                     n1 + layer, n1 + layer + 1, n1 + layer + 1 + (nx + 1), n1 + layer + (nx + 1)], axis=1)
    return X, conn.astype(np.int32)


def pml_attributes(ne, h, npml):
    """PML3DHexa8 parameters of the outer `npml` element layers on the four
    sides and the bottom of an nx x ny x nz box, as the pre-processor's
    setPMLattributes writes them (PP/Method/Builder.py:804-901): the
    reference point x0 is the corner, edge or face point of the inner box the
    element lies beyond, and the normal npml the unit vector towards the
    element (1/sqrt(2), 1/sqrt(3) components at edges and corners).  Returns
    the PML flag [nelem] and the parameter rows [nelem, 9] = m (set by the
    caller), L, R (set by the caller), x0[3], npml[3]."""
    nx, ny, nz = ne
    e = np.arange(nx * ny * nz)
    ix, iy, iz = e % nx, (e // nx) % ny, e // (nx * ny)
    side = np.zeros((e.size, 3), np.int64)          # -1 below / 0 inside / +1 above, per direction
    side[ix < npml, 0] = -1
    side[ix >= nx - npml, 0] = 1
    side[iy < npml, 1] = -1
    side[iy >= ny - npml, 1] = 1
    side[iz < npml, 2] = -1
    epml = np.any(side != 0, axis=1).astype(np.int32)
    lo = np.array([npml * h, npml * h, npml * h])
    hi = np.array([(nx - npml) * h, (ny - npml) * h, np.inf])
    ctr = np.array([nx * h / 2.0, ny * h / 2.0, (nz * h + npml * h) / 2.0])
    par = np.zeros((e.size, 9))
    cnt = np.sum(side != 0, axis=1)
    for d in range(3):
        x0 = np.where(side[:, d] < 0, lo[d], np.where(side[:, d] > 0, hi[d], ctr[d]))
        par[:, 3 + d] = x0
        par[:, 6 + d] = np.where(cnt > 0, side[:, d] / np.sqrt(np.maximum(cnt, 1)), 0.0)
    par[epml == 0] = 0.0
    return epml, par


def config2_pml(nx=128, ny=128, nz=64, npml=10, nt=4001, seed=0, amp=1.0e3, pml_m=2.0, pml_R=1.0e-6,
                element_force=None):
    """Config 2 as specified: the config2 box and source with its outer `npml`
    element layers on the four sides and the bottom PML3DHexa8 (m = pml_m,
    L = npml h, R = pml_R; the log-normal Vs field everywhere), 9 dofs at the
    nodes of PML elements and 3 elsewhere (node-by-node PlainScheme order),
    the outer PML boundary fixed in displacement, the top free.  Built in
    numpy; element_force(model, e, direction) is the element body-force
    routine (default the library's svl_element_body_force)."""
    h, rho, nu = 2.0, 2100.0, 0.3
    vs = lognormal_field((nx, ny, nz), h, 400.0, 0.2, 20.0, seed)
    vs_e = np.transpose(vs, (2, 1, 0)).reshape(-1)
    ne = nx * ny * nz
    G = rho * vs_e ** 2
    E = 2 * G * (1 + nu)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2] = E, nu, rho
    X, conn = grid_nodes_conn((nx, ny, nz), h)
    epml, par = pml_attributes((nx, ny, nz), h, npml)
    par[epml == 1, 0], par[epml == 1, 1], par[epml == 1, 2] = pml_m, npml * h, pml_R
    nn = X.shape[0]
    pnode = np.zeros(nn, bool)
    pnode[conn[epml == 1].ravel()] = True
    ndof_n = np.where(pnode, 9, 3).astype(np.int32)
    outer = (np.isclose(X[:, 0], 0.0) | np.isclose(X[:, 0], nx * h) | np.isclose(X[:, 1], 0.0)
             | np.isclose(X[:, 1], ny * h) | np.isclose(X[:, 2], 0.0))
    j = np.arange(9)[None, :]
    has = j < ndof_n[:, None]
    off = np.concatenate([[0], np.cumsum(ndof_n)[:-1]]).astype(np.int64)
    tdof = np.where(has, off[:, None] + j, -1).astype(np.int32)
    free = has & ~(outer[:, None] & (j < 3))
    fdof = np.full((nn, 9), -1, np.int64)
    fdof[free] = np.arange(int(free.sum()))
    m = Model(ndim=3, coords=X, totaldof=tdof, freedof=fdof.astype(np.int32), conn=conn,
              elem_type=capi.SVL_ELEM_LIN3DHEXA8, elem_mat=np.arange(ne, dtype=np.int32),
              mat_type=np.full(ne, capi.SVL_MAT_ELASTIC3DLINEAR, np.int32), mat_param=mp, lumped=True,
              node_ndof=ndof_n, elem_pml=epml, pml_param=par, grid_shape=(nx, ny, nz))
    vp_max = np.sqrt(E.max() * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho)
    dt = 0.5 * h / vp_max
    L = Loads()
    s = L.add_series(ricker(nt, dt, 3.0, amp=1.0))
    cx, cy, cz = nx // 2, ny // 2, (nz + npml) // 2

    def eid(i, j, k):
        return (k * ny + j) * nx + i
    for e, d in ((eid(cx, cy + 1, cz), (amp, 0.0, 0.0)), (eid(cx, cy - 1, cz), (-amp, 0.0, 0.0)),
                 (eid(cx + 1, cy, cz), (0.0, amp, 0.0)), (eid(cx - 1, cy, cz), (0.0, -amp, 0.0))):
        L.add_body_load(m, [e], d, s,
                        element_force=None if element_force is None else (lambda e2, q, m_=m: element_force(m_, e2, q)))
    return m, L, dt
