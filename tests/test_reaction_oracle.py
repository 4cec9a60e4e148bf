"""Reaction forces in the oracle (Sim::reaction) against a dense restatement.

DynamicAnalysis::UpdateDomain stores, at every fixed node (a free-dof entry of
-1), R = m A + sum over elements with a fixed node of (Fint_e + C_e V_e +
M_e A_e) - Fext(k) (DynamicAnalysis.cpp:128-150, CentralDifference.cpp:
156-171, Assembler.cpp:273-287, 569-619, lin2DQuad4.cpp:416-434).  Every
element that touches a fixed node's dof has that node, so on those dofs R
equals the assembled K U + C V + M A - Fext(k) of an elastic model."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import h8_box, lysmer_box, q4_box


def _fext(L, ntotal, k):
    f = np.zeros(ntotal)
    for d, s, c in zip(L.force_dof, L.force_series, L.force_coef):
        ser = L.series[s]
        if 0 <= k < ser.size:
            f[d] += c * ser[k]
    return f


def _dense(m):
    nt = m.ntotal
    K, M, Cm = (np.zeros((nt, nt)) for _ in range(3))
    ray = m.rayleigh if m.rayleigh is not None else np.zeros((m.nelem, 2))
    for e in range(m.nelem):
        Ke, Ml, _ = O.element_matrices(m, e)
        dofs = m.totaldof[m.conn[e]].reshape(-1)
        K[np.ix_(dofs, dofs)] += Ke
        M[np.ix_(dofs, dofs)] += Ml
        Cm[np.ix_(dofs, dofs)] += ray[e, 0] * Ml + ray[e, 1] * Ke
    if m.dashpot_dof is not None:
        for (a, b), eta in zip(m.dashpot_dof, m.dashpot_eta):
            Cm[a, a] += eta; Cm[b, b] += eta; Cm[a, b] -= eta; Cm[b, a] -= eta
    fixed = np.zeros(nt, bool)
    for n in range(m.nnode):
        nd = m.dof_mask()[n].sum()
        if np.any(m.freedof[n, :nd] == -1):
            fixed[m.totaldof[n, :nd]] = True
    return K, M, Cm, fixed


def _newmark_state(m, L, dt, nsteps):
    """Dense NewmarkBeta (Linear) run: U, V, A after nsteps."""
    K, M, Cm, _ = _dense(m)
    nt = m.ntotal
    free = np.full(nt, -1)
    free[m.totaldof.reshape(-1)] = m.freedof.reshape(-1)
    idx = np.flatnonzero(free >= 0)
    fr = idx[np.argsort(free[idx])]
    Keff = (K + 4.0 / dt ** 2 * M + 2.0 / dt * Cm)[np.ix_(fr, fr)]
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    for i in range(nsteps):
        F = _fext(L, nt, 1 + i) - K @ U + M @ (4.0 / dt * V + A) + Cm @ V
        du = np.zeros(nt)
        du[fr] = np.linalg.solve(Keff, F[fr])
        A = 4.0 / dt ** 2 * du - 4.0 / dt * V - A
        V = 2.0 / dt * du - V
        U = U + du
    return U, V, A


@pytest.mark.parametrize("builder", ["q4", "h8", "lysmer"])
def test_newmark_reaction_matches_dense(builder):
    if builder == "q4":
        m, L, dt = q4_box(8, 5, nt=40)
        m.rayleigh = np.tile([2.0, 1.0e-3], (m.nelem, 1))
    elif builder == "h8":
        m, L, dt = h8_box(3, 3, 2, nt=40)
    else:
        m, L, dt = lysmer_box(8, 5, nt=40)
    dt = 4 * dt
    n = 30
    R = O.reaction_run(m, L, dt, n, integrator="newmark")
    U, V, A = _newmark_state(m, L, dt, n)
    K, M, Cm, fixed = _dense(m)
    Rd = np.where(fixed, K @ U + Cm @ V + M @ A - _fext(L, m.ntotal, n), 0.0)
    assert np.abs(Rd).max() > 0
    assert np.abs(R - Rd).max() <= 1e-8 * np.abs(Rd).max()


def test_central_difference_reaction_balances_the_model():
    """Explicit run: on the fixed nodes R = K U + C V + M A - Fext with the
    oracle's own final state (elastic, mass-proportional damping)."""
    m, L, dt = q4_box(10, 6, nt=120)
    m.rayleigh = np.tile([3.0, 0.0], (m.nelem, 1))
    n = 100
    R = O.reaction_run(m, L, dt, n, integrator="cd")
    hist, U, V, A = O.cd_run(m, L, dt, n)[:4]
    K, M, Cm, fixed = _dense(m)
    Rd = np.where(fixed, K @ U + Cm @ V + M @ A - _fext(L, m.ntotal, n), 0.0)
    assert np.abs(Rd).max() > 0
    assert np.abs(R - Rd).max() <= 1e-8 * np.abs(Rd).max()


@pytest.mark.parametrize("ndim,integ", [(2, "xnewmark"), (3, "xnewmark"), (2, "xnewmark_nm")])
def test_pml_reaction_matches_dense(ndim, integ):
    """PML models (ExtendedNewmarkBeta / NewmarkBeta): every element with a
    fixed node adds K_e u_e + C_e v_e + M_e a_e over all its dofs
    (PML3DHexa8.cpp:746-767, no history term), so on the fixed nodes' dofs R
    equals the assembled K U + C V + M A - Fext(k) with the PML element
    matrices (consistent PML mass) and the run's own final state."""
    from tests.helpers import pml_box
    if ndim == 2:
        m, L, dt = pml_box(ndim=2, ni=(6, 4), npml=2, nt=40)
        n = 30
    else:
        m, L, dt = pml_box(ndim=3, ni=(2, 2, 2), npml=1, nt=20)
        n = 12
    R = O.reaction_run(m, L, dt, n, integrator=integ)
    _, U, V, A, _ = O.xnewmark_run(m, L, dt, n, newmark=integ == "xnewmark_nm")
    K, M, Cm, _ = O.xnewmark_matrices(m)
    fixed = np.zeros(m.ntotal, bool)
    mask = m.dof_mask()
    for i in range(m.nnode):
        nd = mask[i].sum()
        if np.any(m.freedof[i, :nd] == -1):
            fixed[m.totaldof[i, :nd]] = True
    Rd = np.where(fixed, K @ U + Cm @ V + M @ A - _fext(L, m.ntotal, n), 0.0)
    assert np.abs(Rd).max() > 0
    assert np.abs(R - Rd).max() <= 1e-8 * np.abs(Rd).max()
    # the stress dofs of fixed PML nodes carry (nonzero) reactions too
    pnodes = [i for i in range(m.nnode) if mask[i].sum() > ndim and np.any(m.freedof[i, :ndim] == -1)]
    sd = np.concatenate([m.totaldof[i, ndim:mask[i].sum()] for i in pnodes])
    assert np.abs(R[sd]).max() > 0
