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
