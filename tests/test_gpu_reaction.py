"""Reaction forces on the GPU (svl_cd_reaction, svl_nm_reaction) against the
oracle's Sim::reaction, itself pinned to a dense restatement
(tests/test_reaction_oracle.py): DynamicAnalysis::UpdateDomain's
R = m A + sum over elements with a fixed node of (Fint_e + C_e V_e + M_e A_e)
- Fext(k) on the dofs of fixed nodes."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference, NewmarkBeta
from tests.helpers import h8_box, q4_box

pytestmark = pytest.mark.gpu


def _close(R, Ro, tol):
    assert np.abs(Ro).max() > 0
    assert np.abs(R - Ro).max() <= tol * np.abs(Ro).max()


@pytest.mark.parametrize("builder", ["q4", "h8"])
def test_central_difference_reaction(gpu, builder):
    if builder == "q4":
        m, L, dt = q4_box(12, 6, nt=150)
    else:
        m, L, dt = h8_box(5, 4, 3, nt=150)
    m.rayleigh = np.tile([3.0, 0.0], (m.nelem, 1))
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    cd.run(1, 120)
    R = cd.ComputeReactionForce(120)
    cd.close()
    _close(R, O.reaction_run(m, L, dt, 120, integrator="cd"), 1e-11)


def test_central_difference_reaction_j2_columns(gpu):
    """J2 soil columns with EQUAL constraints and base support motion: the
    explicit path maps the last strain on a copy of the J2 states."""
    from tests.test_gpu_newton import _columns
    m, L, dt = _columns(elastic=False)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    cd.run(1, 70)
    R = cd.ComputeReactionForce(70)
    cd.close()
    _close(R, O.reaction_run(m, L, dt, 70, integrator="cd"), 1e-10)


def test_newmark_reaction_rayleigh(gpu):
    m, L, dt = q4_box(12, 6, nt=60)
    m.rayleigh = np.tile([2.0, 1.0e-3], (m.nelem, 1))
    nm = NewmarkBeta(m, L, 4 * dt, pcg_tol=1e-13)
    nm.Initialize()
    nm.run(1, 40)
    R = nm.ComputeReactionForce(40)
    nm.close()
    _close(R, O.reaction_run(m, L, 4 * dt, 40, integrator="newmark"), 1e-8)


def test_newmark_newton_j2_reaction_with_dashpots(gpu):
    from svl_gb300 import j2_params
    from svl_gb300 import _capi as capi
    from tests.helpers import lysmer_box
    m, L, dt = lysmer_box(10, 6, nt=60, amp=4.0e5)
    G = 2000.0 * 200.0 ** 2
    K = 2 * G * 1.25 / (3 * 0.5)
    m.mat_type = np.array([capi.SVL_MAT_PLASTICPLANESTRAINJ2], np.int32)
    m.mat_param = j2_params(K, G, 2000.0, 0.02 * G, 0.5, np.sqrt(3.0) * 15e3)[None, :]
    nm = NewmarkBeta(m, L, 2 * dt, pcg_tol=1e-13, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    nm.Initialize()
    nm.run(1, 40)
    R = nm.ComputeReactionForce(40)
    nm.close()
    _close(R, O.reaction_run(m, L, 2 * dt, 40, integrator="newmark", algo=2, maxit=3, cnvgtol=0.0), 1e-8)


@pytest.mark.parametrize("ndim,integ", [(2, "xnewmark"), (3, "xnewmark"), (2, "xnewmark_nm")])
def test_pml_model_reaction(gpu, ndim, integ):
    """PML models on the PML-capable handle (ExtendedNewmarkBeta, and the
    NewmarkBeta mode): PML elements with a fixed node add K u + C v + M a over
    all their dofs, so fixed PML nodes report stress-dof reactions too."""
    from svl_gb300 import ExtendedNewmarkBeta
    from tests.helpers import pml_box
    m, L, dt = pml_box(ndim=ndim, ni=(6, 4) if ndim == 2 else (3, 3, 2), npml=2, nt=40)
    n = 30
    h = ExtendedNewmarkBeta(m, L, dt, tol=1e-13, integrator="newmark" if integ == "xnewmark_nm" else "extendednewmark")
    h.Initialize()
    h.run(1, n)
    R = h.ComputeReactionForce(n)
    h.close()
    _close(R, O.reaction_run(m, L, dt, n, integrator=integ), 1e-8)


def test_explicit_pml_scheme_rejects_reactions(gpu):
    from svl_gb300 import SvlError
    from svl_gb300 import _capi as capi
    from tests.helpers import pml_box
    m, L, dt = pml_box(ndim=2, ni=(6, 4), npml=2, nt=20, dt_factor=0.5)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    cd.run(1, 5)
    with pytest.raises(SvlError) as ei:
        cd.ComputeReactionForce(5)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED
    cd.close()
