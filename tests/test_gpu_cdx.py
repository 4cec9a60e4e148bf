"""GPU parity of the mixed-precision batched structured path (svl_cdx_*):
tensor-core TF32 hi/lo element forces with FP32 accumulation and an FP64
displacement update, against the FP64 oracle.  Bar (stated for this path):
relative L2 over the full displacement history <= 1e-5 per instance."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import SvlError, StructuredCentralDifference
from svl_gb300 import _capi as capi
from tests.helpers import h8_box, rel_l2

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-5


def _instances(nx, ny, nz, seeds, nt, amp=1.0e7):
    inst = [h8_box(nx, ny, nz, seed=s, nt=nt, amp=amp) for s in seeds]
    dt = min(d for _, _, d in inst)        # one step for the batch
    return [(m, L) for m, L, _ in inst], dt


@pytest.mark.parametrize("shape", [(12, 10, 7), (17, 13, 9)], ids=["12x10x7", "17x13x9"])
def test_cdx_matches_oracle_per_instance(gpu, shape):
    nx, ny, nz = shape
    nt = 200
    inst, dt = _instances(nx, ny, nz, (0, 1, 2), nt)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    for b in range(len(inst)):
        cdx.Initialize(b)
    hist = cdx.run(1, nt, history=True)
    V, A = cdx.get(0, 1), cdx.get(0, 2)
    cdx.close()
    for b, (m, L) in enumerate(inst):
        ho, _, Vo, Ao = O.cd_run(m, L, dt, nt, mode=1)
        assert np.abs(ho).max() > 0
        err = rel_l2(hist[:, b, :], ho)
        assert err <= TOL_MIXED, (b, err)
        if b == 0:
            assert rel_l2(V, Vo) <= 1e-4 and rel_l2(A, Ao) <= 1e-3


def test_cdx_long_run_error_stays_bounded(gpu):
    nx, ny, nz = 16, 16, 8
    nt = 1500
    inst, dt = _instances(nx, ny, nz, (3,), nt)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    cdx.Initialize(0)
    hist = cdx.run(1, nt, history=True)
    cdx.close()
    ho, *_ = O.cd_run(inst[0][0], inst[0][1], dt, nt, mode=1)
    assert rel_l2(hist[:, 0, :], ho) <= TOL_MIXED


def test_cdx_timed_run_equals_recorded_run(gpu):
    nx, ny, nz = 10, 9, 8
    inst, dt = _instances(nx, ny, nz, (5, 6), 120)
    a = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    b = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    for i in range(2):
        a.Initialize(i)
        b.Initialize(i)
    a.run(1, 100)
    ms = b.run_timed(1, 100)
    assert ms > 0
    for i in range(2):
        assert np.array_equal(a.get(i), b.get(i))      # deterministic, no atomics
    a.close()
    b.close()


def test_cdx_rejects_unsupported_models(gpu):
    m, L, dt = h8_box(6, 5, 4, nt=10)
    m.mat_type = np.full(m.nelem, capi.SVL_MAT_PLASTIC3DJ2, np.int32)
    with pytest.raises(SvlError) as ei:
        StructuredCentralDifference((6, 5, 4), (2.0, 2.0, 2.0), [(m, L)], dt)
    assert ei.value.code == capi.SVL_ERR_UNSUPPORTED
    m, L, dt = h8_box(6, 5, 4, nt=10)
    with pytest.raises(SvlError) as ei:     # wrong grid spacing
        StructuredCentralDifference((6, 5, 4), (1.0, 2.0, 2.0), [(m, L)], dt)
    assert ei.value.code == capi.SVL_ERR_INVALID
