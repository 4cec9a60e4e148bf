"""Drop-in boundary checks that need no GPU.

* The library's structured-grid generator reproduces the reference
  pre-processor's node order, connectivity, PlainScheme total/free dof
  numbers and EQUAL-constraint records bit for bit (tests/golden fixtures
  generated by running PP/ itself).
* libsvl_gb300.so loads and exports every entry point include/svl_gb300.h
  declares.
* Host-side validation rejects malformed models with SVL_ERR_INVALID.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from svl_gb300 import _capi as capi
from svl_gb300.model import Loads, Model

GOLD = Path(__file__).resolve().parent / "golden"

CASES = {
    "q4_box": dict(ndim=2, ne=(6, 4), h=(1.0, 1.0), fix=(1, 1, 3, 0, 0, 0), periodic=False),
    "q4_column_periodic": dict(ndim=2, ne=(3, 5), h=(0.5, 0.5), fix=(0, 0, 3, 0, 0, 0), periodic=True),
    "h8_box": dict(ndim=3, ne=(3, 2, 2), h=(2.0, 2.0, 2.0), fix=(1, 1, 2, 2, 7, 0), periodic=False),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_grid_numbering_matches_reference_preprocessor(name):
    gold = json.loads((GOLD / ("numbering_%s.json" % name)).read_text())
    c = CASES[name]
    m = Model.grid(c["ndim"], c["ne"], c["h"], fix_mask=c["fix"], periodic_x=c["periodic"])
    assert m.ntotal == gold["ntotal"] and m.nfree == gold["nfree"]
    assert gold["node_tags"] == list(range(1, m.nnode + 1))
    assert np.array_equal(m.totaldof, np.array(gold["totaldof"]))
    assert np.array_equal(m.freedof, np.array(gold["freedof"]))
    assert np.array_equal(m.coords, np.array(gold["coords"], dtype=float))
    assert np.array_equal(m.conn + 1, np.array(gold["conn"]))
    cons = gold["constraints"]
    assert m.nconstraint == len(cons)
    for i, (tag, rec) in enumerate(sorted(cons.items(), key=lambda kv: -int(kv[0]))):
        assert int(tag) == -2 - i
        assert m.con_slave[i] == rec["stag"]
        assert [m.con_master[i]] == rec["mtag"]
        assert [m.con_factor[i]] == rec["factor"]


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = capi.exported_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.svl_version().decode().startswith("svl_gb300")


def test_grid_sizes_edge_cases():
    L = capi.lib()
    spec = capi.GridSpec()
    spec.ndim = 2
    spec.ne[0], spec.ne[1] = 0, 3
    out = [C.c_int32() for _ in range(5)]
    assert L.svl_grid_sizes(C.byref(spec), *[C.byref(o) for o in out]) == capi.SVL_ERR_INVALID
    spec.ne[0] = 1
    assert L.svl_grid_sizes(C.byref(spec), *[C.byref(o) for o in out]) == capi.SVL_OK
    assert out[0].value == 8 and out[1].value == 3 and out[2].value == 16 and out[3].value == 16
    spec.ndim = 4
    assert L.svl_grid_sizes(C.byref(spec), *[C.byref(o) for o in out]) == capi.SVL_ERR_INVALID


def test_host_validation_rejects_bad_models():
    m = Model.grid(2, (3, 2), (1.0, 1.0), fix_mask=(0, 0, 3, 0, 0, 0))
    bad = Model(**{k: getattr(m, k) for k in ("ndim", "coords", "totaldof", "freedof", "conn", "elem_type",
                                              "elem_mat", "mat_type", "mat_param")})
    bad.conn = bad.conn.copy()
    bad.conn[0, 0] = 999
    fe = np.zeros(8)
    q = np.ones(2)
    d = bad.desc()
    st = capi.lib().svl_element_body_force(C.byref(d), 0, capi.ptr(q, C.c_double), capi.ptr(fe, C.c_double))
    assert st == capi.SVL_ERR_INVALID
    assert b"out of range" in capi.lib().svl_last_error()
    bad2 = Model(**{k: getattr(m, k) for k in ("ndim", "coords", "totaldof", "freedof", "conn", "elem_type",
                                               "elem_mat", "mat_type", "mat_param")})
    bad2.mat_type = np.array([capi.SVL_MAT_ELASTIC3DLINEAR], np.int32)
    d2 = bad2.desc()
    st = capi.lib().svl_element_body_force(C.byref(d2), 0, capi.ptr(q, C.c_double), capi.ptr(fe, C.c_double))
    assert st == capi.SVL_ERR_INVALID


def test_cd_create_without_gpu_reports_no_device():
    """On a machine without a GPU the product fails loudly (no CPU fallback)."""
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    m = Model.grid(2, (3, 2), (1.0, 1.0), fix_mask=(0, 0, 3, 0, 0, 0))
    md, ld = m.desc(), Loads().desc()
    opts = capi.CdOpts(dt=1e-3, ftol=1e-12, mtol=1e-12, precision=0, check_every=0)
    h = C.c_void_p()
    st = capi.lib().svl_cd_create(C.byref(md), C.byref(ld), C.byref(opts), C.byref(h))
    assert st == capi.SVL_ERR_NODEVICE


def test_xnm_options_are_checked_before_any_device_work():
    """svl_xnm_create rejects an unknown algorithm and Newton settings outside
    the reference's (nstep > 0, cnvgtest 1-8, cnvgtol >= 0) with
    SVL_ERR_INVALID, on any machine; valid options without a GPU give
    SVL_ERR_NODEVICE."""
    from tests.conftest import gpu_available
    from tests.helpers import pml_box
    m, L, dt = pml_box(2, (4, 3), npml=2, nt=10)
    md, ld = m.desc(), L.desc()

    def create(**kw):
        o = dict(dt=dt, ftol=1e-12, mtol=1e-12, tol=1e-10, maxit=1000, algorithm=capi.SVL_ALGO_LINEAR,
                 newton_maxit=0, cnvgtest=4, cnvgtol=0.0, integrator=capi.SVL_XNM_EXTENDED_NEWMARK, single_inner=1)
        o.update(kw)
        h = C.c_void_p()
        st = capi.lib().svl_xnm_create(C.byref(md), C.byref(ld), C.byref(capi.XnmOpts(**o)), C.byref(h))
        if st == capi.SVL_OK:
            capi.lib().svl_xnm_destroy(h)
        return st

    assert create(algorithm=7) == capi.SVL_ERR_INVALID
    assert create(algorithm=capi.SVL_ALGO_NEWTON, newton_maxit=0) == capi.SVL_ERR_INVALID
    assert create(algorithm=capi.SVL_ALGO_NEWTON, newton_maxit=3, cnvgtest=9) == capi.SVL_ERR_INVALID
    assert create(algorithm=capi.SVL_ALGO_NEWTON, newton_maxit=3, cnvgtol=-1.0) == capi.SVL_ERR_INVALID
    assert create(dt=0.0) == capi.SVL_ERR_INVALID
    if not gpu_available():
        assert create(algorithm=capi.SVL_ALGO_NEWTON, newton_maxit=3, cnvgtest=1) == capi.SVL_ERR_NODEVICE


def test_nm_options_layout_and_central_difference_dispatch():
    """svl_nm_opts ends with the integrator field (SVL_NM_NEWMARK or
    SVL_NM_CENTRAL_DIFFERENCE), checked before any device work; the Python
    CentralDifference sends a model with a non-diagonal K = M/dt^2 + C/2dt
    (consistent mass, or ak != 0) to the PCG-solving handle."""
    from tests.conftest import gpu_available
    from svl_gb300.integrators import _cd_nondiagonal
    assert C.sizeof(capi.NmOpts) == 72 and capi.NmOpts.integrator.offset == 64
    m = Model.grid(2, (3, 2), (1.0, 1.0), fix_mask=(0, 0, 3, 0, 0, 0))
    md, ld = m.desc(), Loads().desc()

    def create(integrator):
        o = capi.NmOpts(dt=1e-3, ftol=1e-12, mtol=1e-12, pcg_tol=1e-12, pcg_maxit=100, precond=0, algorithm=0,
                        maxit=1, cnvgtol=0.0, cnvgtest=4, single_inner=0, integrator=integrator)
        h = C.c_void_p()
        st = capi.lib().svl_nm_create(C.byref(md), C.byref(ld), C.byref(o), C.byref(h))
        if st == capi.SVL_OK:
            capi.lib().svl_nm_destroy(h)
        return st

    assert create(7) == capi.SVL_ERR_INVALID
    if not gpu_available():
        assert create(capi.SVL_NM_CENTRAL_DIFFERENCE) == capi.SVL_ERR_NODEVICE
    assert not _cd_nondiagonal(m)
    m.rayleigh = np.tile([2.0, 0.0], (m.nelem, 1))
    assert not _cd_nondiagonal(m)
    m.rayleigh[1, 1] = 1e-4
    assert _cd_nondiagonal(m)
    m.rayleigh = None
    m.lumped = False
    assert _cd_nondiagonal(m)


def test_external_force_sums_the_load_entries():
    """Loads.external_force(k) (ComputeProgressiveForce without a stage
    force): coef * series[k] summed per dof, 0 past a series' end; DRM loads
    are refused on the host."""
    from tests.helpers import drm_box, q4_box
    m, L, dt = q4_box(6, 4, nt=30)
    s2 = L.add_series(np.linspace(1.0, 2.0, 10))
    L.add_point_load(m, 5, (0.5, -1.0), s2, factor=2.0)
    for k in (0, 3, 9, 10, 40):
        f = L.external_force(m.ntotal, k)
        ref = np.zeros(m.ntotal)
        for d, s_, c in zip(L.force_dof, L.force_series, L.force_coef):
            if k < L.series[s_].size:
                ref[d] += c * L.series[s_][k]
        assert np.array_equal(f, ref)
    assert np.abs(L.external_force(m.ntotal, 3)).max() > 0
    assert not L.external_force(m.ntotal, 40).any()
    md, Ld, dt2, _, _ = drm_box(nt=10)
    with pytest.raises(ValueError):
        Ld.external_force(md.ntotal, 1)
