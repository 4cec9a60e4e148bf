"""Rayleigh damping in the oracle, pinned against a dense textbook restatement.

The oracle assembles C = sum_e (am_e M_e + ak_e K0_e) (lin2DQuad4.cpp:322-372,
Driver.hpp:1375-1400) into the Newmark effective force and stiffness
(NewmarkBeta.cpp:215, 231) and, for mass-proportional damping, into the
central-difference diagonal (CentralDifference.cpp:70, 217).  The checks here
integrate the same equations with dense numpy matrices built from the
oracle's element matrices; the undamped runs fix the load-step convention.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import h8_box, q4_box, rel_l2


def _fext(L, ntotal, k):
    f = np.zeros(ntotal)
    for d, s, c in zip(L.force_dof, L.force_series, L.force_coef):
        ser = L.series[s]
        if 0 <= k < ser.size:
            f[d] += c * ser[k]
    return f


def _assemble(m, ray):
    nt = m.ntotal
    K = np.zeros((nt, nt))
    M = np.zeros((nt, nt))
    Cm = np.zeros((nt, nt))
    nd = m.ndim
    for e in range(m.nelem):
        Ke, Ml, _ = O.element_matrices(m, e)
        dofs = m.totaldof[m.conn[e]].reshape(-1)
        K[np.ix_(dofs, dofs)] += Ke
        M[np.ix_(dofs, dofs)] += Ml
        Cm[np.ix_(dofs, dofs)] += ray[e, 0] * Ml + ray[e, 1] * Ke
    free = np.full(nt, -1)
    fd = m.freedof.reshape(-1)
    td = m.totaldof.reshape(-1)
    free[td] = fd
    idx = np.flatnonzero(free >= 0)
    order = idx[np.argsort(free[idx])]
    return K, M, Cm, order


def _newmark_dense(m, L, dt, nsteps, ray):
    K, M, C, fr = _assemble(m, ray)
    nt = m.ntotal
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    Keff = (K + 4.0 / dt ** 2 * M + 2.0 / dt * C)[np.ix_(fr, fr)]
    hist = np.zeros((nsteps, nt))
    for i in range(nsteps):
        k = 1 + i
        F = _fext(L, nt, k) - K @ U + M @ (4.0 / dt * V + A) + C @ V
        du = np.zeros(nt)
        du[fr] = np.linalg.solve(Keff, F[fr])
        An = 4.0 / dt ** 2 * du - 4.0 / dt * V - A
        V = 2.0 / dt * du - V
        A = An
        U = U + du
        hist[i] = U
    return hist


def _cd_dense(m, L, dt, nsteps, am):
    _, M, _, fr = _assemble(m, np.zeros((m.nelem, 2)))
    Md = np.diag(M).copy()
    Cd = np.zeros(m.ntotal)
    for e in range(m.nelem):
        _, Ml, _ = O.element_matrices(m, e)
        dofs = m.totaldof[m.conn[e]].reshape(-1)
        Cd[dofs] += am[e] * np.diag(Ml)
    K, *_ = _assemble(m, np.zeros((m.nelem, 2)))
    nt = m.ntotal
    U, Up = np.zeros(nt), np.zeros(nt)
    hist = np.zeros((nsteps, nt))
    for i in range(nsteps):
        k = 1 + i
        R = _fext(L, nt, k) - K @ U + (Md / dt ** 2 - Cd / (2 * dt)) * (U - Up)
        du = np.zeros(nt)
        du[fr] = R[fr] / (Md / dt ** 2 + Cd / (2 * dt))[fr]
        Up = U
        U = U + du
        hist[i] = U
    return hist


def _ray(m, am, ak, seed=0):
    rng = np.random.default_rng(seed)
    r = np.zeros((m.nelem, 2))
    r[:, 0] = am * (0.5 + rng.random(m.nelem))
    r[:, 1] = ak * (0.5 + rng.random(m.nelem))
    return r


@pytest.mark.parametrize("builder", ["q4", "h8"])
def test_newmark_rayleigh_matches_dense_restatement(builder):
    if builder == "q4":
        m, L, dt = q4_box(8, 5, nt=60)
    else:
        m, L, dt = h8_box(3, 3, 2, nt=60)
    dt = 4 * dt
    # undamped: fixes the load-index convention of the restatement
    h0, _ = O.newmark_run(m, L, dt, 40)
    assert rel_l2(_newmark_dense(m, L, dt, 40, np.zeros((m.nelem, 2))), h0) <= 1e-9
    m.rayleigh = _ray(m, 3.0, 2.0e-3)
    h1, _ = O.newmark_run(m, L, dt, 40)
    hd = _newmark_dense(m, L, dt, 40, m.rayleigh)
    assert rel_l2(hd, h1) <= 1e-9
    assert rel_l2(h1, h0) > 1e-2                  # the damping changes the response
    assert np.linalg.norm(h1[-10:]) < np.linalg.norm(h0[-10:])


def test_central_difference_mass_proportional_damping():
    m, L, dt = q4_box(10, 6, nt=200)
    am = 8.0 * (0.5 + np.random.default_rng(1).random(m.nelem))
    h0, *_ = O.cd_run(m, L, dt, 200)
    m.rayleigh = np.stack([am, np.zeros(m.nelem)], axis=1)
    h1, *_ = O.cd_run(m, L, dt, 200)
    hd = _cd_dense(m, L, dt, 200, am)
    assert rel_l2(hd, h1) <= 1e-10
    assert rel_l2(h1, h0) > 1e-3


def test_central_difference_stiffness_proportional_damping_damps():
    """With ak > 0 the oracle takes the factorised K = M/dt^2 + C/2dt path
    (CentralDifference.cpp:64-151); the damped free vibration decays faster
    than the undamped one."""
    m, L, dt = q4_box(4, 3, nt=120)
    h0, *_ = O.cd_run(m, L, dt, 100)
    m.rayleigh = np.tile([0.0, 5e-3], (m.nelem, 1))
    h1, *_ = O.cd_run(m, L, dt, 100)
    assert np.all(np.isfinite(h1)) and np.abs(h1).max() > 0
    assert np.abs(h1[-30:]).max() < np.abs(h0[-30:]).max()


def _dashpot_matrix(m):
    C = np.zeros((m.ntotal, m.ntotal))
    for (a, b), e in zip(m.dashpot_dof, m.dashpot_eta):
        C[a, a] += e; C[b, b] += e; C[a, b] -= e; C[b, a] -= e
    return C


def test_lysmer_dashpots_newmark_and_central_difference():
    """ZeroLength1D dashpots (C_e = eta [1 -1; -1 1]) held to fixed anchors:
    Newmark against the dense restatement, CD against its diagonal form."""
    from tests.helpers import lysmer_box
    m, L, dt = lysmer_box(10, 5, nt=200)
    K, M, Cr, fr = _assemble(m, np.zeros((m.nelem, 2)))
    C = _dashpot_matrix(m)
    # Newmark
    nt = m.ntotal
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    dtn = 4 * dt
    Keff = (K + 4.0 / dtn ** 2 * M + 2.0 / dtn * C)[np.ix_(fr, fr)]
    hd = np.zeros((60, nt))
    for i in range(60):
        F = _fext(L, nt, 1 + i) - K @ U + M @ (4.0 / dtn * V + A) + C @ V
        du = np.zeros(nt)
        du[fr] = np.linalg.solve(Keff, F[fr])
        An = 4.0 / dtn ** 2 * du - 4.0 / dtn * V - A
        V = 2.0 / dtn * du - V
        A = An
        U = U + du
        hd[i] = U
    h1, _ = O.newmark_run(m, L, dtn, 60)
    assert rel_l2(h1, hd) <= 1e-9
    m0 = dict(dashpot_dof=m.dashpot_dof, dashpot_eta=m.dashpot_eta)
    m.dashpot_dof = m.dashpot_eta = None
    h0, _ = O.newmark_run(m, L, dtn, 60)
    assert rel_l2(h1, h0) > 1e-3
    m.dashpot_dof, m.dashpot_eta = m0["dashpot_dof"], m0["dashpot_eta"]
    # central difference: M/dt^2 + C/2dt is diagonal on the free dofs
    Md = np.diag(M)
    Cd = np.diag(C)
    U, Up = np.zeros(nt), np.zeros(nt)
    hc = np.zeros((200, nt))
    for i in range(200):
        R = _fext(L, nt, 1 + i) - K @ U + (Md / dt ** 2) * (U - Up) - C @ (U - Up) / (2 * dt)
        du = np.zeros(nt)
        du[fr] = R[fr] / (Md / dt ** 2 + Cd / (2 * dt))[fr]
        Up = U
        U = U + du
        hc[i] = U
    h2, *_ = O.cd_run(m, L, dt, 200)
    assert np.abs(h2).max() > 0
    assert rel_l2(h2, hc) <= 1e-10
    # a dashpot between two free dofs makes the explicit solve non-diagonal
    m.dashpot_dof = np.array([[int(m.totaldof[20, 0]), int(m.totaldof[21, 0])]], np.int32)
    m.dashpot_eta = np.array([1.0e5])
    with pytest.raises(RuntimeError):
        O.cd_run(m, L, dt, 5)
