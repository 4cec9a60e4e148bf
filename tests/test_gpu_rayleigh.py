"""Rayleigh damping on the GPU paths, against the oracle.

NewmarkBeta takes C = sum_e (am_e M_e + ak_e K0_e) in its effective force
C (V - 2/dt dU) and stiffness K + 4/dt^2 M + 2/dt C (NewmarkBeta.cpp:215,
231): the mass part as a diagonal, the stiffness part as a second element
action with the initial elastic moduli.  CentralDifference takes the
mass-proportional part (its effective stiffness stays diagonal,
CentralDifference.cpp:70, 217) and rejects ak != 0."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference, NewmarkBeta, SvlError
from svl_gb300 import _capi as capi
from tests.helpers import h8_box, q4_box, rel_l2
from tests.test_gpu_newton import _columns, j2_box

pytestmark = pytest.mark.gpu


def _ray(m, am, ak, seed=0):
    rng = np.random.default_rng(seed)
    r = np.zeros((m.nelem, 2))
    r[:, 0] = am * (0.5 + rng.random(m.nelem))
    r[:, 1] = ak * (0.5 + rng.random(m.nelem))
    return r


@pytest.mark.parametrize("builder", ["q4", "h8"])
def test_linear_newmark_rayleigh(gpu, builder):
    if builder == "q4":
        m, L, dt = q4_box(16, 8, nt=80)
    else:
        m, L, dt = h8_box(6, 5, 4, nt=80)
    dt = 4 * dt
    m.rayleigh = _ray(m, 3.0, 2.0e-3)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-13)
    nm.Initialize()
    hist = nm.run(1, 60, history=True)
    nm.close()
    ho, _ = O.newmark_run(m, L, dt, 60, solver=0)
    m.rayleigh = None
    hu, _ = O.newmark_run(m, L, dt, 60, solver=0)
    assert rel_l2(ho, hu) > 1e-2
    assert rel_l2(hist, ho) <= 1e-9


def test_linear_newmark_rayleigh_constraints_support_motion(gpu):
    m, L, dt = _columns(elastic=True)
    m.rayleigh = _ray(m, 2.0, 1.0e-3, seed=3)
    nm = NewmarkBeta(m, L, 4 * dt, pcg_tol=1e-13)
    nm.Initialize()
    hist = nm.run(1, 60, history=True)
    nm.close()
    ho, _ = O.newmark_run(m, L, 4 * dt, 60, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-9


def test_newton_j2_rayleigh_fixed_iterations(gpu):
    m, L, dt = j2_box(2, (8, 6), amp=4e5, nt=60)
    m.rayleigh = _ray(m, 2.0, 5.0e-4, seed=5)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-13, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    nm.Initialize()
    hist = nm.run(1, 60, history=True)
    nm.close()
    ho, _ = O.newmark_run(m, L, dt, 60, algo=2, maxit=3, cnvgtol=0.0, solver=0)
    assert rel_l2(hist, ho) <= 1e-9


def test_central_difference_mass_proportional(gpu):
    m, L, dt = q4_box(20, 10, nt=300)
    m.rayleigh = _ray(m, 8.0, 0.0, seed=1)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    hist = cd.run(1, 300, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 300)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-12


def test_central_difference_stiffness_proportional(gpu):
    """ak != 0 makes M/dt^2 + C/2dt non-diagonal: the diagonal handle rejects
    it, CentralDifference goes to the PCG-solving handle and matches the
    oracle's factorised solve."""
    import ctypes as C
    from svl_gb300 import CentralDifferenceSolve
    m, L, dt = q4_box(6, 4, nt=60)
    m.rayleigh = _ray(m, 0.0, 1e-3)
    md, ld = m.desc(), L.desc()
    opts = capi.CdOpts(dt=dt, ftol=1e-12, mtol=1e-12, precision=capi.SVL_PREC_FP64, check_every=0)
    h = C.c_void_p()
    assert capi.lib().svl_cd_create(C.byref(md), C.byref(ld), C.byref(opts), C.byref(h)) == capi.SVL_ERR_UNSUPPORTED
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, CentralDifferenceSolve)
    cd.Initialize()
    hist = cd.run(1, 50, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 50)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-9


def test_lysmer_dashpots_on_all_paths(gpu):
    """ZeroLength1D dashpots to fixed anchors: explicit CD (diagonal), NewmarkBeta
    and ExtendedNewmarkBeta, against the oracle."""
    from svl_gb300 import ExtendedNewmarkBeta
    from tests.helpers import lysmer_box
    m, L, dt = lysmer_box(16, 8, nt=300)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    hc = cd.run(1, 300, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 300)
    assert np.abs(ho).max() > 0 and rel_l2(hc, ho) <= 1e-12
    nm = NewmarkBeta(m, L, 4 * dt, pcg_tol=1e-13)
    nm.Initialize()
    hn = nm.run(1, 60, history=True)
    nm.close()
    hno, _ = O.newmark_run(m, L, 4 * dt, 60, solver=0)
    assert rel_l2(hn, hno) <= 1e-9
    x = ExtendedNewmarkBeta(m, L, 4 * dt, tol=1e-13)
    x.Initialize()
    hx = x.run(1, 60, history=True)
    x.close()
    assert rel_l2(hx, hno) <= 1e-9


def test_newton_j2_with_lysmer_dashpots(gpu):
    """The SPD alternative to a PML half-space under J2 layers: Newton with the
    consistent tangent plus dashpot damping, fixed iteration count."""
    from svl_gb300 import j2_params
    from tests.helpers import lysmer_box
    m, L, dt = lysmer_box(10, 6, nt=60, amp=4.0e5)
    G = 2000.0 * 200.0 ** 2
    K = 2 * G * 1.25 / (3 * 0.5)
    m.mat_type = np.array([capi.SVL_MAT_PLASTICPLANESTRAINJ2], np.int32)
    m.mat_param = j2_params(K, G, 2000.0, 0.02 * G, 0.5, np.sqrt(3.0) * 15e3)[None, :]
    nm = NewmarkBeta(m, L, 2 * dt, pcg_tol=1e-13, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    nm.Initialize()
    hist = nm.run(1, 50, history=True)
    nm.close()
    ho, _ = O.newmark_run(m, L, 2 * dt, 50, algo=2, maxit=3, cnvgtol=0.0, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-9


def test_central_difference_rejects_free_free_dashpot(gpu):
    m, L, dt = q4_box(6, 4, nt=20)
    assert m.freedof[9, 0] >= 0 and m.freedof[10, 0] >= 0           # two interior nodes
    m.dashpot_dof = np.array([[int(m.totaldof[9, 0]), int(m.totaldof[10, 0])]], np.int32)
    m.dashpot_eta = np.array([1.0e5])
    with pytest.raises(SvlError) as ei:
        CentralDifference(m, L, dt)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED


def test_domain_reduction_central_difference_and_newmark(gpu):
    """DRM forces (elastic, lumped mass: factor * K~ (U_o + ak V_o)) on the
    explicit and implicit paths against the oracle's faithful element matrices."""
    from tests.helpers import drm_box
    m, L, dt, elems, motion = drm_box(16, 10, nt=200)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    hc = cd.run(1, 200, history=True)
    cd.close()
    ho, *_ = O.cd_run(m, L, dt, 200)
    assert np.abs(ho).max() > 0 and rel_l2(hc, ho) <= 1e-12
    m.rayleigh = np.tile([1.0, 4e-4], (m.nelem, 1))
    nm = NewmarkBeta(m, L, 3 * dt, pcg_tol=1e-13)
    nm.Initialize()
    hn = nm.run(1, 60, history=True)
    nm.close()
    hno, _ = O.newmark_run(m, L, 3 * dt, 60, solver=0)
    assert rel_l2(hn, hno) <= 1e-9
