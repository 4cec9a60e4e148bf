"""Central difference with a non-diagonal K = M/dt^2 + C/2dt in the oracle
(CDGen: a consistent mass, massform Consistent, or stiffness-proportional
Rayleigh damping; CentralDifference.cpp:64-151, factorised once like
SimplicialLDLT) against a dense numpy restatement of the same recurrences
built from the oracle's element matrices."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import h8_box, q4_box, rel_l2


def _dense_cd(m, L, dt, n):
    nt = m.ntotal
    M, C, K = (np.zeros((nt, nt)) for _ in range(3))
    ray = m.rayleigh if m.rayleigh is not None else np.zeros((m.nelem, 2))
    for e in range(m.nelem):
        Ke, Ml, Mc = O.element_matrices(m, e)
        Me = Ml if m.lumped else Mc
        d = m.totaldof[m.conn[e]].reshape(-1)
        K[np.ix_(d, d)] += Ke
        M[np.ix_(d, d)] += Me
        C[np.ix_(d, d)] += ray[e, 0] * Me + ray[e, 1] * Ke
    free = np.full(nt, -1)
    free[m.totaldof.reshape(-1)] = m.freedof.reshape(-1)
    idx = np.flatnonzero(free >= 0)
    fr = idx[np.argsort(free[idx])]
    Keff = (M / dt ** 2 + C / (2 * dt))[np.ix_(fr, fr)]
    U, Up = np.zeros(nt), np.zeros(nt)
    H = []
    for k in range(1, n + 1):
        f = np.zeros(nt)
        for dof, s_, c in zip(L.force_dof, L.force_series, L.force_coef):
            ser = L.series[s_]
            if 0 <= k < ser.size:
                f[dof] += c * ser[k]
        F = f - K @ U + (M / dt ** 2 - C / (2 * dt)) @ (U - Up)
        du = np.zeros(nt)
        du[fr] = np.linalg.solve(Keff, F[fr])
        Up, U = U, U + du
        H.append(U.copy())
    return np.array(H)


@pytest.mark.parametrize("case", ["q4_consistent", "h8_consistent", "q4_lumped_ak", "q4_consistent_rayleigh"])
def test_cd_general_matches_dense(case):
    if case.startswith("q4"):
        m, L, dt = q4_box(8, 5, nt=80)
    else:
        m, L, dt = h8_box(3, 3, 2, nt=80)
    if "consistent" in case:
        m.lumped = False
        dt *= 0.5                                 # the consistent mass lowers the stable step
    if "ak" in case or "rayleigh" in case:
        m.rayleigh = np.tile([2.0, 2.0e-4], (m.nelem, 1))
    n = 60
    hist, *_ = O.cd_run(m, L, dt, n)
    hd = _dense_cd(m, L, dt, n)
    assert np.abs(hd).max() > 0
    assert rel_l2(hist, hd) <= 1e-10


def _column(ny=12, width=4, h=0.5, nt=200):
    """Elastic plane-strain soil column, periodic sides (EQUAL constraints),
    base shaken horizontally (support motion), consistent mass."""
    from svl_gb300 import _capi as capi
    from svl_gb300.model import Loads, Model, elastic_params
    rho, vs, nu = 2000.0, 250.0, 0.3
    G = rho * vs ** 2
    E = 2 * G * (1 + nu)
    m = Model.grid(2, (width, ny), (h, h), fix_mask=(0, 0, 3, 0, 0, 0), periodic_x=True,
                   mat_type=np.array([capi.SVL_MAT_ELASTIC2DPLANESTRAIN], np.int32),
                   mat_param=elastic_params(2, E, nu, rho)[None, :])
    m.lumped = False
    m.rayleigh = np.tile([0.5, 2.0e-4], (m.nelem, 1))
    vp = np.sqrt(E * (1 - nu) / ((1 + nu) * (1 - 2 * nu)) / rho)
    dt = 0.2 * h / vp
    L = Loads()
    t = np.arange(nt + 1) * dt
    disp = 1e-3 * np.sin(2 * np.pi * 8.0 * t) * (1 - np.exp(-(t / 0.01) ** 2))
    s = L.add_series(disp)
    for i in range(width + 1):
        L.add_support_motion(m, i, 0, s)
    return m, L, dt


def _dense_cd_general(m, L, dt, n):
    """T^T K T du = T^T R - T^T K SM(k); dU = T du + SM(k); the element
    strain of the next step from U + T du (CentralDifference.cpp:124-231)."""
    nt = m.ntotal
    M, C, K = (np.zeros((nt, nt)) for _ in range(3))
    for e in range(m.nelem):
        Ke, Ml, Mc = O.element_matrices(m, e)
        Me = Ml if m.lumped else Mc
        d = m.totaldof[m.conn[e]].reshape(-1)
        K[np.ix_(d, d)] += Ke
        M[np.ix_(d, d)] += Me
        C[np.ix_(d, d)] += m.rayleigh[e, 0] * Me + m.rayleigh[e, 1] * Ke
    T = np.zeros((nt, m.nfree))
    for t_, f in zip(m.totaldof.reshape(-1), m.freedof.reshape(-1)):
        if f >= 0:
            T[t_, f] = 1.0
    for c in range(m.con_slave.size):
        for i in range(m.con_ptr[c], m.con_ptr[c + 1]):
            T[m.con_slave[c], m.con_master[i]] += m.con_factor[i]
    Keff = M / dt ** 2 + C / (2 * dt)
    A = T.T @ Keff @ T

    def g(s, k):
        ser = L.series[s]
        return ser[k] if 0 <= k < ser.size else ser[0]

    U, Up, Us = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    H = []
    for k in range(1, n + 1):
        sm = np.zeros(nt)
        for dof, s_, fac in zip(L.sm_dof, L.sm_series, L.sm_factor):
            sm[dof] += fac * (g(s_, k) - g(s_, k - 1))
        R = -K @ Us + (M / dt ** 2 - C / (2 * dt)) @ (U - Up)
        du = np.linalg.solve(A, T.T @ R - T.T @ (Keff @ sm))
        dut = T @ du
        Us = U + dut
        Up, U = U, U + dut + sm
        H.append(U.copy())
    return np.array(H)


def test_cd_general_constraints_support_motion_matches_dense():
    """The non-diagonal central difference with EQUAL constraints (periodic
    column) and a base support motion, consistent mass and Rayleigh (am, ak),
    against the dense restatement with T and SM."""
    m, L, dt = _column()
    assert m.con_slave is not None and len(L.sm_dof) > 0
    n = 150
    hist, *_ = O.cd_run(m, L, dt, n)
    hd = _dense_cd_general(m, L, dt, n)
    assert np.abs(hd).max() > 0
    assert rel_l2(hist, hd) <= 1e-10
