"""GPU parity of CentralDifference with a non-diagonal effective stiffness
K = M/dt^2 + C/2dt (consistent mass, stiffness-proportional Rayleigh damping;
CentralDifference.cpp:64-70, 122-152, 204-231) against the oracle, which
factorises K once.  The GPU solves K du = Feff by Jacobi-PCG to a true relative
residual of 1e-12 every step; bar: relative L2 over the displacement history
<= 1e-9 and over the final velocities / accelerations <= 1e-8."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference, CentralDifferenceSolve, SvlError
from tests.helpers import h8_box, q4_box, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _case(name):
    if name.startswith("q4"):
        m, L, dt = q4_box(16, 9, nt=200)
    else:
        m, L, dt = h8_box(5, 4, 3, nt=200)
    if "consistent" in name:
        m.lumped = False
        dt *= 0.5                                   # the consistent mass lowers the stable step
    if "ak" in name or "rayleigh" in name:
        rng = np.random.default_rng(3)
        r = np.zeros((m.nelem, 2))
        r[:, 1] = 2.0e-4 * (0.5 + rng.random(m.nelem))
        if "rayleigh" in name:
            r[:, 0] = 2.0 * (0.5 + rng.random(m.nelem))
        m.rayleigh = r
    return m, L, dt


CASES = ["q4_consistent", "h8_consistent", "q4_lumped_ak", "h8_lumped_ak", "q4_consistent_rayleigh",
         "h8_consistent_rayleigh", "q4_lumped_rayleigh_ak"]


@pytest.mark.parametrize("case", CASES)
def test_nondiagonal_central_difference_parity(case, gpu):
    m, L, dt = _case(case)
    n = 150
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, CentralDifferenceSolve)
    cd.Initialize()
    hg = cd.run(1, n, history=True)
    Vg, Ag = cd.GetVelocities(), cd.GetAccelerations()
    cd.close()
    ho, _, Vo, Ao = O.cd_run(m, L, dt, n)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= TOL
    assert rel_l2(Vg, Vo) <= 1e-8 and rel_l2(Ag, Ao) <= 1e-8


def test_nondiagonal_central_difference_initial_conditions(gpu):
    m, L, dt = _case("q4_consistent_rayleigh")
    rng = np.random.default_rng(5)
    nt = m.ntotal
    free = np.zeros(nt, bool)
    free[m.totaldof[m.freedof >= 0]] = True
    U0 = np.where(free, 1e-4 * rng.standard_normal(nt), 0.0)
    V0 = np.where(free, 1e-3 * rng.standard_normal(nt), 0.0)
    cd = CentralDifference(m, L, dt)
    cd.Initialize(U0, V0, None)
    hg = cd.run(1, 80, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 80, U0=U0, V0=V0)
    assert rel_l2(hg, ho) <= TOL


def test_nondiagonal_central_difference_steps_and_responses(gpu):
    """ComputeNewStep one step at a time equals one batched run; element
    responses after the run match the oracle's."""
    m, L, dt = _case("h8_consistent_rayleigh")
    a = CentralDifference(m, L, dt)
    a.Initialize()
    for k in range(1, 41):
        assert not a.ComputeNewStep(k)
    b = CentralDifference(m, L, dt)
    b.Initialize()
    b.run(1, 40)
    assert np.array_equal(a.GetDisplacements(), b.GetDisplacements())
    elems = [0, 7, m.nelem - 1]
    for resp in ("STRESS", "INTERNALFORCE"):
        g = a.element_response(resp, elems)
        o = O.element_response_run(m, L, dt, 40, resp, elems, integrator="cd")
        assert rel_l2(g, o) <= 1e-8, resp
    with pytest.raises(SvlError):
        a.ComputeReactionForce(40)
    a.close()
    b.close()


def test_nondiagonal_central_difference_rejects_what_it_does_not_cover(gpu):
    """Domain-reduction loads are not covered by the solve mode."""
    from tests.helpers import drm_box
    m, L, dt, _, _ = drm_box(nt=20)
    m.lumped = False
    with pytest.raises(SvlError):
        CentralDifference(m, L, dt)


def _j2_h8():
    from svl_gb300 import _capi as capi
    m, L, dt = h8_box(5, 4, 3, nt=200, amp=4.0e8)
    ne = m.nelem
    G = m.mat_param[:, 0] / (2 * 1.3)
    K = m.mat_param[:, 0] / (3 * (1 - 0.6))
    m.mat_type = np.full(ne, capi.SVL_MAT_PLASTIC3DJ2, np.int32)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2], mp[:, 3], mp[:, 4], mp[:, 5] = K, G, 2100.0, 0.02 * G, 1.0, 2.0e5
    m.mat_param = mp
    m.lumped = False
    return m, L, 0.5 * dt


GENERAL = ["h8_j2_consistent", "q4_j2_columns_consistent_rayleigh", "lysmer_consistent"]


def _general(case):
    from tests.helpers import lysmer_box, q4_j2_columns
    if case == "h8_j2_consistent":
        return _j2_h8()
    if case == "q4_j2_columns_consistent_rayleigh":
        m, L, dt = q4_j2_columns(3, 4, (10, 16, 22), nt=300, pga=6.0)
        m.lumped = False
        m.rayleigh = np.tile([1.0, 1.0e-4], (m.nelem, 1))
        return m, L, 0.5 * dt
    m, L, dt = lysmer_box(16, 8, nt=300)
    m.lumped = False
    return m, L, 0.5 * dt


@pytest.mark.parametrize("case", GENERAL)
def test_nondiagonal_central_difference_j2_constraints_support_motion_dashpots(case, gpu):
    """J2 materials (element update once per step), EQUAL constraints with
    support motion (periodic soil columns shaken at the base: Feff = T^T R -
    T^T K SM(k), dU = T du + SM(k)) and Lysmer dashpots in K, with a
    consistent mass, against the oracle's factorised solve."""
    m, L, dt = _general(case)
    n = 200
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, CentralDifferenceSolve)
    cd.Initialize()
    hg = cd.run(1, n, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, n)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= 1e-8


def test_nondiagonal_central_difference_periodic_column_support_motion(gpu):
    """Elastic periodic soil column shaken at the base, consistent mass and
    Rayleigh (am, ak): T^T K T solve with T^T K SM(k) on the GPU against the
    oracle (itself pinned to a dense restatement with T and SM)."""
    from tests.test_cd_general_oracle import _column
    m, L, dt = _column()
    n = 150
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, CentralDifferenceSolve)
    cd.Initialize()
    hg = cd.run(1, n, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, n)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= 1e-9
