"""GPU parity of the FP64 explicit central-difference path against the CPU
oracle, through the C ABI.  Bar: relative L2 over the full displacement
history <= 1e-12 (FP64 plain form), bitwise run-to-run determinism."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference
from tests.helpers import h8_box, q4_box, q4_j2_columns, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gpu_hist(m, L, dt, n, **kw):
    cd = CentralDifference(m, L, dt, **kw)
    cd.Initialize()
    h = cd.run(1, n, history=True)
    V, A = cd.GetVelocities(), cd.GetAccelerations()
    cd.close()
    return h, V, A


def test_q4_elastic_box_parity(gpu):
    m, L, dt = q4_box(40, 20, nt=600)
    hg, Vg, Ag = _gpu_hist(m, L, dt, 600)
    ho, _, Vo, Ao = O.cd_run(m, L, dt, 600, mode=1)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= TOL
    assert rel_l2(Vg, Vo) <= 1e-11 and rel_l2(Ag, Ao) <= 1e-10


def test_h8_heterogeneous_box_parity(gpu):
    m, L, dt = h8_box(8, 7, 6, nt=250)
    hg, _, _ = _gpu_hist(m, L, dt, 250)
    ho, *_ = O.cd_run(m, L, dt, 250, mode=1)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= TOL


def test_q4_j2_periodic_columns_support_motion_parity(gpu):
    m, L, dt = q4_j2_columns(3, 4, (10, 16, 22), nt=400, pga=6.0)
    hg, _, _ = _gpu_hist(m, L, dt, 400)
    ho, *_ = O.cd_run(m, L, dt, 400, mode=1)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= 1e-10


def test_h8_j2_parity(gpu):
    from svl_gb300 import _capi as capi
    m, L, dt = h8_box(6, 5, 4, nt=200, amp=4.0e8)
    ne = m.nelem
    G = m.mat_param[:, 0] / (2 * 1.3)
    K = m.mat_param[:, 0] / (3 * (1 - 0.6))
    m.mat_type = np.full(ne, capi.SVL_MAT_PLASTIC3DJ2, np.int32)
    mp = np.zeros((ne, 8))
    mp[:, 0], mp[:, 1], mp[:, 2], mp[:, 3], mp[:, 4], mp[:, 5] = K, G, 2100.0, 0.02 * G, 1.0, 2.0e5
    m.mat_param = mp
    hg, _, _ = _gpu_hist(m, L, dt, 200)
    ho, *_ = O.cd_run(m, L, dt, 200, mode=1)
    assert np.abs(ho).max() > 0
    assert rel_l2(hg, ho) <= 1e-10


def test_runs_are_bitwise_deterministic(gpu):
    m, L, dt = q4_box(30, 15, nt=300)
    h1, _, _ = _gpu_hist(m, L, dt, 300)
    h2, _, _ = _gpu_hist(m, L, dt, 300)
    assert np.array_equal(h1, h2)
    # graph replay (no history) gives the same final state as the recorded run
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    cd.run(1, 300)
    assert np.array_equal(cd.GetDisplacements(), h1[-1])
    cd.close()


def test_step_by_step_interface_matches_batch(gpu):
    m, L, dt = q4_box(12, 6, nt=50)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    for k in range(1, 41):
        assert cd.ComputeNewStep(k) is False
    u_steps = cd.GetDisplacements()
    cd.close()
    h, _, _ = _gpu_hist(m, L, dt, 40)
    assert np.array_equal(u_steps, h[-1])


def test_initial_conditions_parity(gpu):
    m, L, dt = q4_box(10, 6, nt=100)
    rng = np.random.default_rng(3)
    U0 = 1e-4 * rng.standard_normal(m.ntotal)
    V0 = 1e-3 * rng.standard_normal(m.ntotal)
    U0[m.freedof.ravel() < 0] = 0.0
    V0[m.freedof.ravel() < 0] = 0.0
    cd = CentralDifference(m, L, dt)
    cd.Initialize(U0, V0, None)
    hg = cd.run(1, 100, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 100, mode=1, U0=U0, V0=V0)
    assert rel_l2(hg, ho) <= TOL


def test_nonfinite_state_is_reported(gpu):
    """A step far above the stability limit blows up; the status word turns
    that into SVL_ERR_NONFINITE instead of silently returning NaNs."""
    from svl_gb300 import SvlError
    m, L, dt = q4_box(8, 4, nt=2000)
    cd = CentralDifference(m, L, dt * 40.0, check_every=1)
    cd.Initialize()
    with pytest.raises(SvlError) as ei:
        cd.run(1, 2000)
    assert ei.value.code == 3
    cd.close()


def test_config1_full_size_parity(gpu):
    """200 x 100 Q4 box, 2000 steps: the full configuration against the oracle."""
    m, L, dt = q4_box(200, 100, nt=2000, amp=1.0e6)
    hg, _, _ = _gpu_hist(m, L, dt, 2000)
    ho, *_ = O.cd_run(m, L, dt, 2000, mode=1)
    assert rel_l2(hg, ho) <= TOL
