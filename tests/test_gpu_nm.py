"""GPU parity of the implicit path (svl_nm_*): Newmark average acceleration
with the Linear algorithm and a matrix-free FP64 Jacobi-PCG solve of the
effective stiffness, against the oracle's assembled-matrix Newmark
(dense LDL^T or CSR Jacobi-PCG).

Both sides solve every step to a relative residual of 1e-12 (the GPU checks
the true residual), so the histories agree to the conditioning of K_eff times
that tolerance; the bar written here is 1e-9 relative L2 over the history."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import NewmarkBeta, SvlError
from svl_gb300 import _capi as capi
from tests.helpers import h8_box, q4_box, q4_j2_columns, rel_l2

pytestmark = pytest.mark.gpu
TOL_SOLVE = 1e-12
TOL_HIST = 1e-9


def test_nm_q4_matches_oracle_dense(gpu):
    m, L, dt = q4_box(16, 8, nt=120)
    dt *= 5.0                         # implicit: a step well above the CFL limit
    nt = 60
    nm = NewmarkBeta(m, L, dt, pcg_tol=TOL_SOLVE)
    nm.Initialize()
    hist = nm.run(1, nt, history=True)
    its, _, res = nm.stats()
    nm.close()
    ho, _ = O.newmark_run(m, L, dt, nt, solver=0)
    assert np.abs(ho).max() > 0
    assert res <= TOL_SOLVE and its > 0
    assert rel_l2(hist, ho) <= TOL_HIST


def test_nm_h8_heterogeneous_matches_oracle_pcg(gpu):
    m, L, dt = h8_box(7, 6, 5, seed=3, nt=80)
    dt *= 10.0                        # the implicit workload's dt = 10 x CFL
    nt = 40
    nm = NewmarkBeta(m, L, dt, pcg_tol=TOL_SOLVE)
    nm.Initialize()
    hist = nm.run(1, nt, history=True)
    V, A = nm.GetVelocities(), nm.GetAccelerations()
    nm.close()
    ho, _ = O.newmark_run(m, L, dt, nt, solver=1, pcg_tol=TOL_SOLVE)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= TOL_HIST
    # velocity / acceleration from the last increment, same recurrences
    hv, _ = O.newmark_run(m, L, dt, nt, solver=0)
    assert rel_l2(hist, hv) <= TOL_HIST
    assert np.all(np.isfinite(V)) and np.all(np.isfinite(A))


def test_nm_loose_tolerance_reaches_true_residual(gpu):
    m, L, dt = h8_box(8, 8, 6, seed=4, nt=40)
    dt *= 10.0
    tight = NewmarkBeta(m, L, dt, pcg_tol=TOL_SOLVE)
    loose = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    for h in (tight, loose):
        h.Initialize()
    ht = tight.run(1, 20, history=True)
    hl = loose.run(1, 20, history=True)
    it_t, _, _ = tight.stats()
    it_l, _, res_l = loose.stats()
    tight.close()
    loose.close()
    assert res_l <= 1e-8
    assert it_l < it_t
    assert rel_l2(hl, ht) <= 1e-6


def test_nm_reference_interface_and_determinism(gpu):
    m, L, dt = q4_box(12, 6, nt=40)
    dt *= 4.0
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-10)
    b = NewmarkBeta(m, L, dt, pcg_tol=1e-10)
    a.Initialize()
    b.Initialize()
    for k in range(1, 21):
        assert a.ComputeNewStep(k) is False
    b.run(1, 20)
    for w in range(3):
        assert np.array_equal(a._get(w), b._get(w))     # fixed-order reductions, no atomics
    a.close()
    b.close()


def test_nm_iteration_cap_is_reported(gpu):
    m, L, dt = h8_box(6, 6, 5, seed=1, nt=20)
    nm = NewmarkBeta(m, L, 10.0 * dt, pcg_tol=1e-14, pcg_maxit=3)
    nm.Initialize()
    with pytest.raises(SvlError) as ei:
        nm.run(1, 5)
    assert ei.value.code == capi.SVL_ERR_MAXITER
    nm.close()


def test_nm_rejects_models_it_does_not_cover(gpu):
    m, L, dt = q4_j2_columns(ncol=2, heights=(4, 5), nt=10)
    with pytest.raises(SvlError) as ei:        # learned preconditioner off the node lattice
        NewmarkBeta(m, L, dt, precond=capi.SVL_PRECOND_LEARNED)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED


@pytest.mark.parametrize("shape", [(16, 8), (6, 5, 4)], ids=["quad", "hexa"])
def test_nm_consistent_mass_matches_oracle(gpu, shape):
    """massform Consistent, the pre-processor's default: the element mass
    matrices act element by element (operator and effective force) against
    the oracle's assembled consistent mass and dense LDL^T."""
    if len(shape) == 2:
        m, L, dt = q4_box(*shape, nt=120)
        dt *= 5.0
    else:
        m, L, dt = h8_box(*shape, seed=5, nt=80)
        dt *= 10.0
    m.lumped = False
    nt = 40
    nm = NewmarkBeta(m, L, dt, pcg_tol=TOL_SOLVE)
    nm.Initialize()
    hist = nm.run(1, nt, history=True)
    res = nm.stats()[2]
    nm.close()
    ho, _ = O.newmark_run(m, L, dt, nt, solver=0)
    m.lumped = True
    hl, _ = O.newmark_run(m, L, dt, nt, solver=0)
    assert np.abs(ho).max() > 0 and res <= TOL_SOLVE
    assert rel_l2(ho, hl) > 1e-4               # the mass form matters
    assert rel_l2(hist, ho) <= TOL_HIST


@pytest.mark.parametrize("case", ["column_rayleigh", "j2_columns_newton"])
def test_nm_consistent_mass_constraints_support_motion_damping(gpu, case):
    """massform Consistent on the general path: EQUAL constraints (periodic
    columns), base support motion and Rayleigh (am with the consistent
    element mass, ak with K0): T^T (K + 4/dt^2 M + 2/dt C) T solved by PCG,
    the effective force's mass and damping terms through the element mass
    action, against the oracle's assembled matrices and dense LDL^T."""
    from tests.test_cd_general_oracle import _column
    if case == "column_rayleigh":
        m, L, dt = _column(nt=120)
        dt *= 4.0
        kw = {}
    else:
        m, L, dt = q4_j2_columns(ncol=2, heights=(6, 9), nt=80)
        m.lumped = False
        m.rayleigh = np.tile([1.0, 1.0e-4], (m.nelem, 1))
        dt *= 2.0
        kw = dict(algorithm="newton", maxit=3, cnvgtol=0.0)
    nt = 40
    nm = NewmarkBeta(m, L, dt, pcg_tol=TOL_SOLVE, **kw)
    nm.Initialize()
    hist = nm.run(1, nt, history=True)
    nm.close()
    if kw:
        ho, _ = O.newmark_run(m, L, dt, nt, algo=1, maxit=3, cnvgtol=0.0, solver=0)
    else:
        ho, _ = O.newmark_run(m, L, dt, nt, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= TOL_HIST
