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
