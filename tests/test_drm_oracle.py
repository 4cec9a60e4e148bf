"""Domain-reduction (DRM) loads in the oracle, against a dense restatement of
ComputeDomainReductionForces (lin2DQuad4.cpp:564-614): for each DRM element
M~ Ao + C~ Vo + K~ Uo with the equal-condition blocks zeroed and the exterior
motions negated (Driver.hpp:1700-1719)."""
import numpy as np

from oracle import oracle as O
from tests.helpers import drm_box, rel_l2
from tests.test_rayleigh_oracle import _assemble


def _drm_force(m, elems, motion, k, ray=None):
    nt = m.ntotal
    F = np.zeros(nt)
    for e in elems:
        Ke, Ml, Mc = O.element_matrices(m, e)
        Me = Ml if m.lumped else Mc
        Ce = np.zeros_like(Ke) if ray is None else ray[e, 0] * Me + ray[e, 1] * Ke
        nodes = m.conn[e]
        cond = np.repeat([1 if motion[n][1] else 0 for n in nodes], 2)
        sg = np.repeat([-1.0 if motion[n][1] else 1.0 for n in nodes], 2)
        U = np.concatenate([motion[n][0][k, 0:2] for n in nodes]) * sg
        V = np.concatenate([motion[n][0][k, 2:4] for n in nodes]) * sg
        A = np.concatenate([motion[n][0][k, 4:6] for n in nodes]) * sg
        mask = cond[:, None] != cond[None, :]
        f = (Me * mask) @ A + (Ce * mask) @ V + (Ke * mask) @ U
        F[m.totaldof[nodes].reshape(-1)] += f
    return F


def test_drm_newmark_matches_dense_restatement():
    m, L, dt, elems, motion = drm_box(10, 7, nt=60)
    m.rayleigh = np.tile([2.0, 5e-4], (m.nelem, 1))
    K, M, C, fr = _assemble(m, m.rayleigh)
    nt = m.ntotal
    dtn = 3 * dt
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    Keff = (K + 4.0 / dtn ** 2 * M + 2.0 / dtn * C)[np.ix_(fr, fr)]
    hd = np.zeros((40, nt))
    for i in range(40):
        F = _drm_force(m, elems, motion, 1 + i, m.rayleigh) - K @ U + M @ (4.0 / dtn * V + A) + C @ V
        du = np.zeros(nt)
        du[fr] = np.linalg.solve(Keff, F[fr])
        An = 4.0 / dtn ** 2 * du - 4.0 / dtn * V - A
        V = 2.0 / dtn * du - V
        A = An
        U = U + du
        hd[i] = U
    ho, _ = O.newmark_run(m, L, dtn, 40, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(ho, hd) <= 1e-9


def test_drm_central_difference_matches_dense_restatement():
    m, L, dt, elems, motion = drm_box(10, 7, nt=120)
    K, M, _, fr = _assemble(m, np.zeros((m.nelem, 2)))
    Md = np.diag(M)
    nt = m.ntotal
    U, Up = np.zeros(nt), np.zeros(nt)
    hd = np.zeros((110, nt))
    for i in range(110):
        R = _drm_force(m, elems, motion, 1 + i) - K @ U + (Md / dt ** 2) * (U - Up)
        du = np.zeros(nt)
        du[fr] = R[fr] / (Md / dt ** 2)[fr]
        Up = U
        U = U + du
        hd[i] = U
    ho, *_ = O.cd_run(m, L, dt, 110)
    assert np.abs(ho).max() > 0
    assert rel_l2(ho, hd) <= 1e-10
