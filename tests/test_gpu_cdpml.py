"""GPU parity of the explicit central difference with PML layers (the
library's staggered scheme, svl_xnm_* with SVL_XNM_CENTRAL_DIFFERENCE;
CentralDifference(model with PML) dispatches there) against its FP64 CPU
oracle (CDPml, oracle/svl_oracle.cpp).  No solve is involved, so the bar is
the FP64 one of the plain central difference: relative L2 over the full
history <= 1e-12, displacement dofs and PML stress dofs checked separately;
in 3D 5e-12, because the device contracts the PML element action's
multiply-adds into fused multiply-adds (the oracle is compiled without
contraction) and the 72-dof element sums of 150 steps carry those last-bit
differences (measured 1.2e-12)."""
import json
import shutil
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import CentralDifference, ExtendedNewmarkBeta, SvlError
from svl_gb300 import _capi as capi
from svl_gb300.partition import load_partition
from tests.helpers import pml_box, pml_j2_box, q4_box, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12
GOLD = Path(__file__).resolve().parent / "golden"


def _split(m):
    nd = m.ndim
    u = np.concatenate([m.totaldof[n, :nd] for n in range(m.nnode)])
    s = np.concatenate([m.totaldof[n, nd:m.node_ndof[n]] for n in range(m.nnode)])
    return u, s


@pytest.mark.parametrize("ndim", [2, 3])
def test_explicit_pml_matches_oracle(gpu, ndim):
    nt = 400 if ndim == 2 else 150
    if ndim == 2:
        m, L, dt = pml_box(2, (12, 8), npml=3, nt=nt, dt_factor=0.5)
    else:
        m, L, dt = pml_box(3, (5, 4, 4), npml=2, nt=nt, dt_factor=0.5, f0=10.0)
    cd = CentralDifference(m, L, dt)
    assert isinstance(cd, ExtendedNewmarkBeta)
    cd.Initialize()
    hg = cd.run(1, nt, history=True)
    Vg, Ag, Ubg = cd.GetVelocities(), cd.GetAccelerations(), cd.GetPMLHistoryVector()
    cd.close()
    ho, Uo, Vo, Ao, Ubo = O.cdpml_run(m, L, dt, nt)
    u, s = _split(m)
    tol = TOL if ndim == 2 else 5e-12
    assert np.abs(ho[:, u]).max() > 0 and np.abs(ho[:, s]).max() > 0
    assert rel_l2(hg[:, u], ho[:, u]) <= tol
    assert rel_l2(hg[:, s], ho[:, s]) <= tol
    assert rel_l2(Vg[u], Vo[u]) <= 1e-10 and rel_l2(Ag[u], Ao[u]) <= 1e-9
    # the PML history integral sums every step's rounding: 1e-11
    assert rel_l2(Ubg, Ubo) <= 10 * tol


def test_explicit_pml_with_j2_layers_matches_oracle(gpu):
    nt = 300
    m, L, dt = pml_j2_box(2, (12, 8), npml=3, nj2=3, su=8e3, nt=nt, dt_factor=0.5, amp=3.0e6)
    cd = CentralDifference(m, L, dt)
    cd.Initialize()
    hg = cd.run(1, nt, history=True)
    cd.close()
    ho, *_ = O.cdpml_run(m, L, dt, nt)
    u, s = _split(m)
    assert rel_l2(hg[:, u], ho[:, u]) <= 1e-10
    assert rel_l2(hg[:, s], ho[:, s]) <= 1e-10


def test_explicit_mode_without_pml_is_the_plain_central_difference(gpu):
    m, L, dt = q4_box(20, 10, nt=200)
    a = CentralDifference(m, L, dt)
    a.Initialize()
    ha = a.run(1, 200, history=True)
    a.close()
    b = ExtendedNewmarkBeta(m, L, dt, integrator="centraldifference")
    b.Initialize()
    hb = b.run(1, 200, history=True)
    b.close()
    assert np.abs(ha).max() > 0 and rel_l2(hb, ha) <= TOL


def test_explicit_pml_partition_file(gpu, tmp_path):
    """The pre-processor's PML fixture with its integrator switched to
    CENTRALDIFFERENCE (and a step below the explicit limit) runs through the
    partition reader and matches the oracle."""
    src = GOLD / "partition_q4_pml_extended"
    shutil.copytree(src, tmp_path / "case")
    f = tmp_path / "case" / "Partition" / "Fixture.1.0.json"
    d = json.loads(f.read_text())
    integ = d["Simulations"]["attributes"]["integrator"]
    integ["name"] = "CENTRALDIFFERENCE"
    integ["dt"] = 2.0e-4
    d["Simulations"]["attributes"]["analysis"]["nt"] = 201
    f.write_text(json.dumps(d))
    p = load_partition(f)
    hg = p.run(write_recorders=False)
    ho, *_ = O.cdpml_run(p.model, p.loads, p.dt, p.nt - 1)
    assert np.abs(ho).max() > 0 and rel_l2(hg, ho) <= TOL


def test_explicit_pml_rejects_what_it_does_not_cover(gpu):
    m, L, dt = pml_box(2, (6, 4), npml=2, nt=20, dt_factor=0.5)
    with pytest.raises(SvlError) as ei:
        ExtendedNewmarkBeta(m, L, dt, integrator="centraldifference", algorithm="newton")
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED
    m.rayleigh = np.tile([0.0, 1e-3], (m.nelem, 1))
    with pytest.raises(SvlError) as ei:
        CentralDifference(m, L, dt)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED
