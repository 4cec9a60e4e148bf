"""ExtendedNewmarkBeta with PML layers on the GPU (svl_xnm_*), against the
oracle's ExtendedNewmarkBeta (dense LDL^T of the assembled K + 4/dt^2 M +
2/dt C + dt/3 G): PML2DQuad4 and PML3DHexa8 boxes, the PML history vector,
the reduction to NewmarkBeta without PML, constraints with support motion,
J2 layers over a PML half-space with Linear and NewtonRaphson, and the paths
that reject PML models."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference, ExtendedNewmarkBeta, NewmarkBeta, SvlError
from svl_gb300 import _capi as capi
from tests.helpers import h8_box, pml_box, q4_box, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ndim,ni,npml,nt", [(2, (10, 6), 2, 120), (3, (3, 3, 2), 1, 40)], ids=["quad", "hexa"])
def test_pml_box_matches_oracle(gpu, ndim, ni, npml, nt):
    m, L, dt = pml_box(ndim, ni, npml=npml, nt=nt, f0=10.0, dt_factor=1.0)
    x = ExtendedNewmarkBeta(m, L, dt, tol=1e-12)
    x.Initialize()
    hist = x.run(1, nt, history=True)
    Ub = x.GetPMLHistoryVector()
    V = x.GetVelocities()
    its, last, res = x.stats()
    x.close()
    ho, Uo, Vo, Ao, Ubo = O.xnewmark_run(m, L, dt, nt)
    assert np.abs(ho).max() > 0 and res <= 1e-12 and its > 0
    # the effective matrix's condition number is ~1e13 (stress rows ~1e-4,
    # displacement rows ~1e9): a solve is good to ~1e-10 at best
    assert rel_l2(hist, ho) <= 1e-8
    assert rel_l2(Ub, Ubo) <= 1e-8
    assert rel_l2(V, Vo) <= 1e-7


def test_without_pml_matches_newmark_with_rayleigh(gpu):
    m, L, dt = h8_box(5, 4, 3, nt=40)
    m.rayleigh = np.tile([1.5, 1.0e-3], (m.nelem, 1))
    x = ExtendedNewmarkBeta(m, L, 4 * dt, tol=1e-13)
    x.Initialize()
    hist = x.run(1, 30, history=True)
    x.close()
    ho, _ = O.newmark_run(m, L, 4 * dt, 30, solver=0)
    assert rel_l2(hist, ho) <= 1e-9


def test_constraints_and_support_motion(gpu):
    from tests.test_gpu_newton import _columns
    m, L, dt = _columns(elastic=True)
    x = ExtendedNewmarkBeta(m, L, 4 * dt, tol=1e-13)
    x.Initialize()
    hist = x.run(1, 50, history=True)
    x.close()
    ho, *_ = O.xnewmark_run(m, L, 4 * dt, 50)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-9


def test_other_paths_reject_pml_models(gpu):
    m, L, dt = pml_box(2, (4, 3), npml=2, nt=10)
    # CentralDifference on a PML model is the explicit PML scheme of the
    # PML-capable handle (tests/test_gpu_cdpml.py); the learned preconditioner
    # does not cover PML models
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, ExtendedNewmarkBeta)
    cd.close()
    with pytest.raises(SvlError) as ei:
        NewmarkBeta(m, L, dt, precond=capi.SVL_PRECOND_LEARNED)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED
    # a PML element needs an elastic material
    m2, L2, dt2 = pml_box(2, (4, 3), npml=2, nt=10)
    m2.mat_type = np.array([capi.SVL_MAT_PLASTICPLANESTRAINJ2], np.int32)
    with pytest.raises(SvlError) as ei:
        ExtendedNewmarkBeta(m2, L2, dt2)
    assert ei.value.code == capi.SVL_ERR_INVALID


def test_domain_reduction_with_pml_layers(gpu):
    """DRM ring inside the solid region of a PML box: ExtendedNewmarkBeta on the
    GPU against the oracle (same faithful DRM forces, dense solve)."""
    from svl_gb300.model import Loads
    m, _, dt = pml_box(2, (12, 8), npml=2, nt=80, dt_factor=1.0)
    X = m.coords
    lo, hi, top = 3.0, 11.0, X[:, 1].max()
    inner = lambda p: lo - 1e-9 <= p[0] <= hi + 1e-9 and p[1] >= lo - 1e-9  # noqa: E731
    elems = []
    for e in range(m.nelem):
        if m.elem_pml[e]:
            continue
        ins = [inner(X[n]) for n in m.conn[e]]
        if any(ins) and not all(ins):
            elems.append(e)
    assert elems
    t = np.arange(90) * dt
    motion = {}
    for n in sorted({int(n) for e in elems for n in m.conn[e]}):
        u = 1e-3 * np.sin(2 * np.pi * 8.0 * (t - (top - X[n, 1]) / 200.0)) * (t > (top - X[n, 1]) / 200.0)
        sig = np.zeros((90, 6))
        sig[:, 0] = u
        sig[:, 2] = np.gradient(u, dt)
        sig[:, 4] = np.gradient(sig[:, 2], dt)
        motion[n] = (sig, not inner(X[n]))
    L = Loads()
    L.add_drm(m, elems, motion)
    x = ExtendedNewmarkBeta(m, L, dt, tol=1e-12)
    x.Initialize()
    hist = x.run(1, 60, history=True)
    x.close()
    ho, *_ = O.xnewmark_run(m, L, dt, 60)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-8


@pytest.mark.parametrize("ndim,ni,npml,nj2,nt,amp", [(2, (10, 6), 2, 3, 60, 1.0e6), (3, (3, 3, 2), 1, 1, 30, 4.0e6)],
                         ids=["quad", "hexa"])
def test_newmark_newton_j2_layers_over_pml(gpu, ndim, ni, npml, nj2, nt, amp):
    """Config-5 form: J2 top layers over an elastic half-space with PML,
    NewmarkBeta + NewtonRaphson with 3 iterations per step (test 4, cnvgtol 0):
    NewmarkBeta(model with PML) runs on the PML-capable handle."""
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(ndim, ni, npml=npml, nj2=nj2, nt=nt, dt_factor=1.0, f0=10.0, amp=amp)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-12, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    assert isinstance(nm, ExtendedNewmarkBeta)
    nm.Initialize()
    hist = nm.run(1, nt, history=True)
    its, last, _ = nm.newton_stats()
    nm.close()
    ho, *_ = O.xnewmark_run(m, L, dt, nt, algo=2, maxit=3, cnvgtol=0.0, newmark=True)
    hl, *_ = O.xnewmark_run(m, L, dt, nt, newmark=True)
    assert its == 3 * nt and last == 3
    assert rel_l2(ho, hl) > 1e-4                     # the layers yield
    assert rel_l2(hist, ho) <= 1e-8


def test_newmark_newton_displacement_test_with_tolerance(gpu):
    """Test 5 (relative displacement increment) with a tolerance: the GPU
    takes the oracle's iteration count on every step."""
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(2, (10, 6), npml=2, nj2=3, nt=40, dt_factor=1.0, f0=10.0)
    its_o = np.zeros(40, np.int32)
    ho, *_ = O.xnewmark_run(m, L, dt, 40, algo=1, maxit=10, cnvgtol=1e-3, step_iters=its_o, newmark=True)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-12, algorithm="newton", maxit=10, cnvgtol=1e-3, cnvgtest=5)
    nm.Initialize()
    hist = nm.run(1, 40, history=True)
    its, _, _ = nm.newton_stats()
    nm.close()
    assert its == int(its_o.sum()) and its_o.max() > 1
    assert rel_l2(hist, ho) <= 1e-8


def test_extended_j2_layers_over_pml_linear(gpu):
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(2, (10, 6), npml=2, nj2=3, nt=60, dt_factor=1.0, f0=10.0)
    x = ExtendedNewmarkBeta(m, L, dt, tol=1e-12)
    x.Initialize()
    hist = x.run(1, 60, history=True)
    x.close()
    ho, *_ = O.xnewmark_run(m, L, dt, 60)
    m0, L0, _ = pml_box(2, (10, 6), npml=2, nt=60, dt_factor=1.0, f0=10.0)
    he, *_ = O.xnewmark_run(m0, L0, dt, 60)
    assert rel_l2(ho, he) > 1e-4
    assert rel_l2(hist, ho) <= 1e-8


def test_extended_newton_follows_the_reference_iteration(gpu):
    """ExtendedNewmarkBeta + NewtonRaphson: the effective force has no
    increment terms, only Fint (solid states and PML K_e (U + T dU)) follows
    the iterate.  The GPU reproduces the oracle's iterates over the first
    steps (the iteration grows without bound later, as the oracle's does)."""
    from tests.helpers import pml_j2_box
    m, L, dt = pml_j2_box(2, (10, 6), npml=2, nj2=3, nt=60, dt_factor=1.0, f0=10.0)
    nt = 8
    x = ExtendedNewmarkBeta(m, L, dt, tol=1e-12, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    x.Initialize()
    hist = x.run(1, nt, history=True)
    Ub = x.GetPMLHistoryVector()
    x.close()
    ho, _, _, _, Ubo = O.xnewmark_run(m, L, dt, nt, algo=2, maxit=3, cnvgtol=0.0)
    hl, *_ = O.xnewmark_run(m, L, dt, nt)
    assert rel_l2(ho, hl) > 1e-3
    assert rel_l2(hist, ho) <= 1e-8
    assert rel_l2(Ub, Ubo) <= 1e-8


def test_j2_columns_newton_constraints_support_motion(gpu):
    """Periodic-side J2 soil columns with base support motion through the
    PML-capable handle in both modes: NewmarkBeta mode against the NewmarkBeta
    oracle (increment of step k - 1), ExtendedNewmarkBeta Linear against its
    oracle (increment of step k)."""
    from tests.test_gpu_newton import _columns
    m, L, dt = _columns(elastic=False)
    x = ExtendedNewmarkBeta(m, L, 4 * dt, tol=1e-13, algorithm="newton", maxit=3, cnvgtol=0.0, integrator="newmark")
    x.Initialize()
    hist = x.run(1, 50, history=True)
    x.close()
    ho, _ = O.newmark_run(m, L, 4 * dt, 50, algo=2, maxit=3, cnvgtol=0.0, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-9
    x = ExtendedNewmarkBeta(m, L, 4 * dt, tol=1e-13)
    x.Initialize()
    hist = x.run(1, 50, history=True)
    x.close()
    ho, *_ = O.xnewmark_run(m, L, 4 * dt, 50)
    assert rel_l2(hist, ho) <= 1e-9


def test_config5_pml_small_matches_oracle(gpu):
    """The config-5 model with a PML half-space (workloads.config5_pml) at a
    small size: NewmarkBeta-Newton, 3 iterations per step, against the oracle."""
    from svl_gb300 import workloads
    m, L, dt = workloads.config5_pml(6, 6, 6, npml=1, n_j2=2, nt=30)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-12, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    nm.Initialize()
    hist = nm.run(1, 25, history=True)
    nm.close()
    ho, *_ = O.xnewmark_run(m, L, dt, 25, algo=2, maxit=3, cnvgtol=0.0, newmark=True)
    assert np.abs(ho).max() > 0
    assert rel_l2(hist, ho) <= 1e-8
