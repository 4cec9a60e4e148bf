"""The oracle's ExtendedNewmarkBeta with PML elements (XNewmark in
oracle/svl_oracle.cpp): assembled operators, reduction to NewmarkBeta without
PML, the support-motion step index, and absorption by the layers."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300.model import Loads
from tests.helpers import h8_box, pml_box, q4_box, q4_j2_columns, rel_l2


@pytest.mark.parametrize("ndim", [2, 3])
def test_pml_model_operators(ndim):
    m, L, dt = pml_box(ndim, (4, 3) if ndim == 2 else (2, 2, 2), npml=2)
    assert m.elem_pml.sum() > 0 and m.ntotal > m.nnode * ndim
    K, M, Cm, G = O.xnewmark_matrices(m)
    for A in (K, M, Cm, G):
        assert np.allclose(A, A.T, rtol=0, atol=1e-12 * max(np.abs(A).max(), 1.0))
    stress = np.zeros(m.ntotal, bool)
    for n in range(m.nnode):
        stress[m.totaldof[n, ndim:m.node_ndof[n]]] = True
    d = np.diag(M)
    assert np.all(d[stress] < 0) and np.all(d[~stress] > 0)
    assert (np.abs(G).max() == 0.0) == (ndim == 2)          # PML2DQuad4 has no history matrix
    assert np.count_nonzero(K[np.ix_(~stress, stress)]) > 0


def test_without_pml_equals_newmark_linear():
    for m, L, dt in (q4_box(8, 5, nt=40), h8_box(3, 3, 2, nt=40)):
        m.rayleigh = np.tile([1.5, 1.0e-3], (m.nelem, 1))
        h0, _ = O.newmark_run(m, L, 4 * dt, 30, solver=0)
        h1, *_ = O.xnewmark_run(m, L, 4 * dt, 30)
        assert np.abs(h0).max() > 0
        assert rel_l2(h1, h0) <= 1e-12


def test_support_motion_index_is_the_current_step():
    """ExtendedNewmarkBeta takes the increment of step k (ExtendedNewmarkBeta.cpp:196),
    NewmarkBeta that of step k - 1 (NewmarkBeta.cpp:187): with the series shifted
    by one the two runs coincide."""
    m, L, dt = q4_j2_columns(ncol=1, width=3, heights=(6,), nt=60)
    E_nu = np.zeros_like(m.mat_param)
    G, K, rho = m.mat_param[:, 1], m.mat_param[:, 0], m.mat_param[:, 2]
    E_nu[:, 0] = 9 * K * G / (3 * K + G)
    E_nu[:, 1] = (3 * K - 2 * G) / (2 * (3 * K + G))
    E_nu[:, 2] = rho
    m.mat_param = E_nu
    from svl_gb300 import _capi as capi
    m.mat_type = np.full_like(m.mat_type, capi.SVL_MAT_ELASTIC2DPLANESTRAIN)
    assert L.series[0][0] == 0.0
    Ls = Loads()
    Ls.series = [np.concatenate([s[1:], s[-1:]]) for s in L.series]
    Ls.sm_dof, Ls.sm_series, Ls.sm_factor = list(L.sm_dof), list(L.sm_series), list(L.sm_factor)
    hx, *_ = O.xnewmark_run(m, L, 2 * dt, 40)
    hn, _ = O.newmark_run(m, Ls, 2 * dt, 40, solver=0)
    assert np.abs(hx).max() > 0
    assert rel_l2(hx, hn) <= 1e-12


def test_layers_absorb_the_outgoing_wave():
    m, L, dt = pml_box(2, (12, 6), npml=3, nt=260, f0=10.0, dt_factor=1.0)
    h, U, V, A, Ub = O.xnewmark_run(m, L, dt, 250)
    interior = m.totaldof[m.node_ndof == 2][:, :2].ravel()
    e = (h[:, interior] ** 2).sum(axis=1)
    assert np.all(np.isfinite(h)) and np.abs(Ub).max() > 0
    assert e[-1] < 1e-4 * e.max()


def test_j2_linear_without_pml_equals_newmark_linear():
    """With G = 0, no support motion and the Linear algorithm the two
    integrators solve the same system; with J2 elements both take one
    tangent solve and one state update per step."""
    from tests.test_gpu_newton import j2_box
    m, L, dt = j2_box(2, (8, 6), amp=4e5, nt=40)
    h0, _ = O.newmark_run(m, L, dt, 30, algo=0, solver=0)
    h1, *_ = O.xnewmark_run(m, L, dt, 30)
    assert np.abs(h0).max() > 0
    assert rel_l2(h1, h0) <= 1e-12


def _dense_xnewton(m, L, dt, nsteps, niter):
    """ExtendedNewmarkBeta + NewtonRaphson on an elastic model without PML or
    support motion, restated densely: every iteration solves
    Keff du = T^T (Fext - K (U + dU) + C V + M (4/dt V + A)) -- the effective
    force has no increment terms (ExtendedNewmarkBeta.cpp:208-229), only Fint
    follows dU through the element states."""
    K, M, Cm, _ = O.xnewmark_matrices(m)
    nt = m.ntotal
    free = np.full(nt, -1)
    free[m.totaldof.reshape(-1)] = m.freedof.reshape(-1)
    idx = np.flatnonzero(free >= 0)
    fr = idx[np.argsort(free[idx])]
    Keff = (K + 4.0 / dt ** 2 * M + 2.0 / dt * Cm)[np.ix_(fr, fr)]
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    hist = np.zeros((nsteps, nt))
    for i in range(nsteps):
        f = np.zeros(nt)
        for d, sidx, c in zip(L.force_dof, L.force_series, L.force_coef):
            ser = L.series[sidx]
            if 1 + i < ser.size:
                f[d] += c * ser[1 + i]
        dU = np.zeros(nt)
        for _ in range(niter):
            F = f - K @ (U + dU) + Cm @ V + M @ (4.0 / dt * V + A)
            dU[fr] += np.linalg.solve(Keff, F[fr])
        A = 4.0 / dt ** 2 * dU - 4.0 / dt * V - A
        V = 2.0 / dt * dU - V
        U = U + dU
        hist[i] = U
    return hist


def test_newton_effective_force_has_no_increment_terms():
    m, L, dt = q4_box(8, 5, nt=40)
    m.rayleigh = np.tile([1.5, 1.0e-3], (m.nelem, 1))
    h3, *_ = O.xnewmark_run(m, L, 4 * dt, 30, algo=2, maxit=3, cnvgtol=0.0)
    h1, *_ = O.xnewmark_run(m, L, 4 * dt, 30)
    assert rel_l2(h3, _dense_xnewton(m, L, 4 * dt, 30, 3)) <= 1e-9
    assert rel_l2(h1, _dense_xnewton(m, L, 4 * dt, 30, 1)) <= 1e-9
    assert rel_l2(h3, h1) > 1e-3                      # the extra iterations change the answer


def test_extended_newton_iterates_without_increment_terms_grow():
    """ExtendedNewmarkBeta + NewtonRaphson iterates dU <- dU + Keff^-1 (R0 -
    (Fint(U + dU) - Fint(U))): without the increment's inertia terms in the
    force the iterates drift to the static solution of each step and the time
    stepping grows without bound.  Recorded here as the reference's behaviour
    (ExtendedNewmarkBeta.cpp:208-229 reads dU and does not use it)."""
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(2, (10, 6), npml=2, nj2=3, nt=60, dt_factor=1.0, f0=10.0)
    its = np.zeros(40, np.int32)
    hn, *_ = O.xnewmark_run(m, L, dt, 40, algo=2, maxit=3, cnvgtol=0.0, step_iters=its)
    hl, *_ = O.xnewmark_run(m, L, dt, 40)
    assert np.all(its == 3)
    assert np.abs(hn[-1]).max() > 1e6 * np.abs(hl).max()


def test_newmark_mode_without_pml_equals_newmark():
    """The oracle's PML-capable integrator in NewmarkBeta mode reproduces the
    NewmarkBeta oracle on J2 soil columns with EQUAL constraints and support
    motion, Linear and Newton."""
    from tests.test_gpu_newton import _columns
    m, L, dt = _columns(elastic=False)
    m.rayleigh = np.tile([1.0, 5.0e-4], (m.nelem, 1))
    for algo, maxit in ((0, 1), (2, 3)):
        hn, _ = O.newmark_run(m, L, 4 * dt, 40, algo=algo, maxit=maxit, cnvgtol=0.0, solver=0)
        hx, *_ = O.xnewmark_run(m, L, 4 * dt, 40, algo=algo, maxit=maxit, cnvgtol=0.0, newmark=True)
        assert np.abs(hn).max() > 0
        assert rel_l2(hx, hn) <= 1e-12


def test_newmark_mode_on_2d_pml_equals_extended_linear():
    """PML2DQuad4 has no history matrix and, without support motion, the two
    integrators' Linear steps coincide."""
    m, L, dt = pml_box(2, (10, 6), npml=2, nt=60, dt_factor=1.0, f0=10.0)
    hx, *_ = O.xnewmark_run(m, L, dt, 50)
    hn, *_ = O.xnewmark_run(m, L, dt, 50, newmark=True)
    assert np.abs(hx).max() > 0
    assert rel_l2(hn, hx) <= 1e-12


def test_newmark_newton_j2_over_pml_converges():
    """NewmarkBeta + NewtonRaphson on J2 layers over PML: the effective force
    carries the increment terms, so the iterations converge (ExtendedNewmarkBeta's
    do not, its force lacks them)."""
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(2, (10, 6), npml=2, nj2=3, nt=60, dt_factor=1.0, f0=10.0)
    its = np.zeros(50, np.int32)
    hn, *_ = O.xnewmark_run(m, L, dt, 50, algo=2, maxit=10, cnvgtol=1e-8, newmark=True, step_iters=its)
    hl, *_ = O.xnewmark_run(m, L, dt, 50, newmark=True)
    assert its.max() < 10 and its.max() >= 2
    assert np.abs(hn).max() < 10 * np.abs(hl).max()
    assert rel_l2(hn, hl) > 1e-4


@pytest.mark.parametrize("test", [1, 2, 3, 4, 5, 6, 7, 8])
def test_convergence_tests_match_a_restatement(test):
    """Algorithm::ComputeConvergence (Algorithm.cpp:122-188), tests 1-8: the
    first iteration's value of a NewmarkBeta + Newton run against the dense
    restatement's (elastic box: later iterations only see round-off); the
    relative forms of later iterations are checked on J2 models on the GPU."""
    m, L, dt = q4_box(8, 5, nt=20)
    dt4 = 4 * dt
    res = np.zeros(1)
    its = np.zeros(6, np.int32)
    O.xnewmark_run(m, L, dt4, 6, algo=10 + test, maxit=1, cnvgtol=0.0, newmark=True, step_iters=its,
                   last_res=res)
    hn, _ = O.newmark_run(m, L, dt4, 6, algo=10 + test, maxit=2, cnvgtol=0.0, solver=0)
    hx, *_ = O.xnewmark_run(m, L, dt4, 6, algo=10 + test, maxit=2, cnvgtol=0.0, newmark=True)
    assert rel_l2(hx, hn) <= 1e-12
    K, M, _, _ = O.xnewmark_matrices(m)
    nt = m.ntotal
    free = np.full(nt, -1)
    free[m.totaldof.reshape(-1)] = m.freedof.reshape(-1)
    idx = np.flatnonzero(free >= 0)
    fr = idx[np.argsort(free[idx])]
    Keff = (K + 4.0 / dt4 ** 2 * M)[np.ix_(fr, fr)]
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    n = np.linalg.norm
    for i in range(6):
        f = np.zeros(nt)
        for d, s_, c in zip(L.force_dof, L.force_series, L.force_coef):
            if 1 + i < L.series[s_].size:
                f[d] += c * L.series[s_][1 + i]
        F = (f - K @ U + M @ (4.0 / dt4 * V + A))[fr]
        du = np.linalg.solve(Keff, F)
        dU = np.zeros(nt)
        dU[fr] = du
        A = 4.0 / dt4 ** 2 * dU - 4.0 / dt4 * V - A
        V = 2.0 / dt4 * dU - V
        U = U + dU
    want = {1: n(F), 2: n(du), 3: n(du * F), 4: n(F), 5: n(du), 6: n(du * F), 7: 1.0, 8: -1.0}[test]
    assert np.all(its == 1)
    assert abs(res[0] - want) <= 1e-9 * abs(want)


def test_config5_pml_workload_structure():
    """workloads.config5_pml: PML3DHexa8 layers on the sides and the bottom
    with 9 dofs at their nodes, J2 only in the solid top layers, the outer PML
    boundary fixed in displacement, dofs numbered node by node; a few
    NewmarkBeta + Newton steps on it in the oracle stay finite (the GPU parity
    test runs 25 steps)."""
    from svl_gb300 import _capi as capi
    from svl_gb300 import workloads
    m, L, dt = workloads.config5_pml(6, 6, 6, npml=1, n_j2=2, nt=30)
    assert m.elem_pml.sum() == 6 * 6 * 6 - 4 * 4 * 5
    mt = m.mat_type[m.elem_mat]
    assert np.all(mt[m.elem_pml == 1] == capi.SVL_MAT_ELASTIC3DLINEAR)
    assert (mt == capi.SVL_MAT_PLASTIC3DJ2).sum() == 4 * 4 * 2
    nd = m.node_ndof
    assert set(np.unique(nd)) == {3, 9}
    td = np.concatenate([m.totaldof[n, :nd[n]] for n in range(m.nnode)])
    assert np.array_equal(td, np.arange(m.ntotal))
    X = m.coords
    outer = np.isclose(X[:, 0], 0) | np.isclose(X[:, 0], 12) | np.isclose(X[:, 1], 0) | np.isclose(X[:, 1], 12) \
        | np.isclose(X[:, 2], 0)
    assert np.all(m.freedof[outer, :3] == -1) and np.all(m.freedof[~outer, :3] >= 0)
    its = np.zeros(4, np.int32)
    h, *_ = O.xnewmark_run(m, L, dt, 4, algo=2, maxit=2, cnvgtol=0.0, newmark=True, step_iters=its)
    disp = m.totaldof[:, :3].ravel()
    assert np.all(its == 2) and np.all(np.isfinite(h)) and 0 < np.abs(h[:, disp]).max() < 1.0
