"""svl_cd_run_noalloc: stepping for callers that must not let the library
allocate device memory (they own all of it through their own pool).

It has to give the same displacements as svl_cd_run on the same model, on
two calls in a row (the static scratch keeps the previous call's contents),
and reject models whose element force block does not fit the static array.
The caller-owned output buffer comes from torch, standing in for the
caller's own allocator.  Collected last (file name) so a run that stops at
the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from svl_gb300 import CentralDifference
from svl_gb300 import _capi as capi
from svl_gb300.model import Model
from tests.helpers import drm_box, h8_box, q4_box, q4_j2_columns, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12   # the FP64 parity tolerance used by the other GPU tests


def _models():
    yield "q4_box", q4_box(40, 20, nt=200)
    yield "q4_j2_periodic_columns", q4_j2_columns(3, 4, (10, 16, 22), nt=200, pga=6.0)
    yield "h8_box", h8_box(10, 9, 8, nt=200)
    m, L, dt, _, _ = drm_box(nt=140)
    yield "q4_drm_box", (m, L, dt)


@pytest.mark.parametrize("name", ["q4_box", "q4_j2_periodic_columns", "h8_box", "q4_drm_box"])
def test_noalloc_matches_run_on_two_calls_in_a_row(gpu, name):
    torch = pytest.importorskip("torch")
    m, L, dt = dict(_models())[name]
    ref = CentralDifference(m, L, dt)
    ref.Initialize()
    ref.run(1, 60)
    U1 = ref.GetDisplacements()
    ref.run(61, 70)
    U2 = ref.GetDisplacements()
    ref.close()

    na = CentralDifference(m, L, dt)
    na.Initialize()
    out = torch.zeros(m.ntotal, dtype=torch.float64, device="cuda")
    capi.check(capi.lib().svl_cd_run_noalloc(na._h, 1, 60, C.c_void_p(out.data_ptr())))
    na.sync()
    V1 = out.cpu().numpy().copy()
    capi.check(capi.lib().svl_cd_run_noalloc(na._h, 61, 70, C.c_void_p(out.data_ptr())))
    na.sync()
    V2 = out.cpu().numpy().copy()
    launches = na.launches()
    na.close()
    # the no-alloc call reports its own kernel count: one step-index set-up
    # plus the same kernels per step as svl_cd_run
    per_step = 2 if m.nconstraint == 0 else 4
    if L is not None and len(L.drm_elem):
        per_step += 1
    assert launches == 1 + 70 * per_step
    assert np.abs(U2).max() > 0
    assert rel_l2(V1, U1) <= TOL
    assert rel_l2(V2, U2) <= TOL


def test_noalloc_rejects_models_beyond_the_scratch(gpu):
    m = Model.grid(3, (36, 36, 34), (1.0, 1.0, 1.0), fix_mask=(0, 0, 0, 0, 7, 0))
    assert m.nelem * 24 * 8 > capi.SVL_NOALLOC_SCRATCH_BYTES
    cd = CentralDifference(m, None, 1e-4)
    cd.Initialize()
    st = capi.lib().svl_cd_run_noalloc(cd._h, 1, 1, None)
    assert st == capi.SVL_ERR_UNSUPPORTED
    assert b"no-alloc scratch" in capi.lib().svl_last_error()
    cd.close()
