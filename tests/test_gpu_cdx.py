"""GPU parity of the mixed-precision batched structured path (svl_cdx_*):
tensor-core TF32 hi/lo element forces with FP32 accumulation and an FP64
displacement update, against the FP64 oracle.  Bar (stated for this path):
relative L2 over the full displacement history <= 1e-5 per instance."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import SvlError, StructuredCentralDifference
from svl_gb300 import _capi as capi
from svl_gb300 import ricker
from tests.helpers import h8_box, rel_l2

pytestmark = pytest.mark.gpu
TOL_MIXED = 1e-5


def _instances(nx, ny, nz, seeds, nt, amp=1.0e7, corner_loads=False):
    inst = [h8_box(nx, ny, nz, seed=s, nt=nt, amp=amp) for s in seeds]
    dt = min(d for _, _, d in inst)        # one step for the batch
    if corner_loads:
        # vertical point loads on surface nodes near the far corner, i.e. in the
        # last node tiles of the instance, with a different delay per instance
        for b, (m, L, _) in enumerate(inst):
            s = L.add_series(ricker(nt + 1, dt, 4.0 + b, amp=amp * 8.0))
            for (i, j) in ((nx - 2, ny - 2), (nx - 1, ny - 3), (nx // 3, ny - 1 - b)):
                node = nz * (nx + 1) * (ny + 1) + j * (nx + 1) + i
                L.add_point_load(m, node, (0.0, 0.0, -1.0), s)
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


def test_cdx_persistent_tiles_match_oracle(gpu):
    """Every CTA of the persistent kernel runs many node tiles: 3 instances of
    20x18x14 elements (18 tiles each, 54 in all) on 8 CTAs, i.e. 6-7 tiles and
    40 MMA tiles per CTA, so the halo prefetch into reused buffers, the reload
    of the owned state, the mbarrier phase flips past the first pass, the reuse
    of the eight TMEM accumulator slots and the load-table walk of later tiles
    all run.  Loads sit in the last tiles.  The full history of every instance
    must match the FP64 oracle, and a one-CTA run (54 tiles in one CTA) must be
    bitwise identical to the one-CTA-per-SM run."""
    nx, ny, nz = 20, 18, 14
    nt = 250
    inst, dt = _instances(nx, ny, nz, (11, 12, 13), nt, corner_loads=True)
    runs = {}
    for ctas in (8, 1, 0):
        cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
        got = cdx.set_ctas(ctas)
        assert got == (54 if ctas == 0 else ctas) or (ctas == 0 and got < 54)
        for b in range(len(inst)):
            cdx.Initialize(b)
        runs[ctas] = cdx.run(1, nt, history=True)
        cdx.close()
    assert np.array_equal(runs[1], runs[0]) and np.array_equal(runs[8], runs[0])
    for b, (m, L) in enumerate(inst):
        ho, *_ = O.cd_run(m, L, dt, nt, mode=1)
        # the corner loads move the last tiles
        corner = nz * (nx + 1) * (ny + 1) + (ny - 2) * (nx + 1) + (nx - 2)
        assert np.abs(ho[:, 3 * corner + 2]).max() > 1e-3 * np.abs(ho).max()
        err = rel_l2(runs[8][:, b, :], ho)
        assert err <= TOL_MIXED, (b, err)


def test_cdx_many_tiles_per_sm_match_oracle(gpu):
    """Default grid (one CTA per SM) on 4 instances of 48x48x32 elements: 245
    tiles each, 980 in all, about 6.4 tiles per CTA on 152 SMs.  Full history
    of every instance against the FP64 oracle over 200 steps."""
    nx, ny, nz = 48, 48, 32
    nt = 200
    inst, dt = _instances(nx, ny, nz, (21, 22, 23, 24), nt, corner_loads=True)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    assert cdx.set_ctas(0) <= 980
    for b in range(len(inst)):
        cdx.Initialize(b)
    hist = cdx.run(1, nt, history=True)
    cdx.close()
    for b, (m, L) in enumerate(inst):
        ho, *_ = O.cd_run(m, L, dt, nt, mode=1, history=True)
        assert np.abs(ho).max() > 0
        err = rel_l2(hist[:, b, :], ho)
        assert err <= TOL_MIXED, (b, err)


def _pml_instances(nx, ny, nz, npml, seeds, nt):
    from svl_gb300 import workloads
    inst = [workloads.config2_pml(nx, ny, nz, npml=npml, nt=nt + 1, seed=s, amp=1.0e7) for s in seeds]
    dt = min(d for _, _, d in inst)
    return [(m, L) for m, L, _ in inst], dt


def _udofs(m):
    u = np.concatenate([m.totaldof[n, :3] for n in range(m.nnode)])
    s = np.concatenate([m.totaldof[n, 3:m.node_ndof[n]] for n in range(m.nnode)])
    return u, s


def test_cdx_pml_band_matches_oracle(gpu):
    """Config-2 layout at small size: lin3DHexa8 grid whose outer 3 element
    layers on the sides and the bottom are PML3DHexa8 (9 dofs at their nodes).
    The tensor-core kernel advances the elastic interior, the PML band runs
    the explicit staggered scheme in FP32 with compensated-pair state.  Two
    instances (different Vs fields), several tiles per CTA; the displacement
    and stress histories of every instance against the FP64 oracle of the
    scheme at the mixed bar."""
    nx, ny, nz, npml = 16, 16, 12, 3
    nt = 200
    inst, dt = _pml_instances(nx, ny, nz, npml, (1, 2), nt)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    cdx.set_ctas(3)
    for b in range(len(inst)):
        cdx.Initialize(b)
    hist = cdx.run(1, nt, history=True)
    ubar = cdx.get(0, 3)
    cdx.close()
    for b, (m, L) in enumerate(inst):
        ho, Uo, Vo, Ao, Ubo = O.cdpml_run(m, L, dt, nt)
        u, s = _udofs(m)
        assert np.abs(ho[:, u]).max() > 0 and np.abs(ho[:, s]).max() > 0
        eu = rel_l2(hist[:, b, u], ho[:, u])
        es = rel_l2(hist[:, b, s], ho[:, s])
        assert eu <= TOL_MIXED and es <= TOL_MIXED, (b, eu, es)
        if b == 0:
            pn = np.zeros(m.nnode, bool)
            pn[m.conn[m.elem_pml == 1].ravel()] = True
            pd = np.concatenate([m.totaldof[n, :m.node_ndof[n]] for n in np.flatnonzero(pn)])
            assert rel_l2(ubar[pd], Ubo[pd]) <= 1e-4


def test_cdx_pml_far_tiles_step_before_the_band(gpu):
    """With a PML band the tiles whose nodes and halo hold no PML node run in
    a launch that does not wait for the band's displacement update of the
    previous step, the others after it.  A grid with such tiles (32 x 24 x 20,
    3-element band: 4 far tiles of 60 per instance), two instances, several
    tiles per CTA in both launches: the displacement and stress histories
    against the FP64 explicit PML scheme of the PML-capable handle (itself
    pinned to the oracle) at the mixed bar, and the same bits for every
    schedule."""
    from svl_gb300 import CentralDifference
    nx, ny, nz, npml = 32, 24, 20, 3
    nt = 150
    inst, dt = _pml_instances(nx, ny, nz, npml, (3, 4), nt)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    ref = None
    for sched in (dict(ctas=5), dict(ctas=3, tile_order=3), dict(ctas=0, tile_order=2, band_threads=256)):
        cdx.set_schedule(**sched)
        for b in range(len(inst)):
            cdx.Initialize(b)
        hist = cdx.run(1, nt, history=True)
        if ref is None:
            ref = hist
        else:
            assert np.array_equal(hist, ref), sched
    cdx.close()
    for b, (m, L) in enumerate(inst):
        cd = CentralDifference(m, L, dt)
        cd.Initialize()
        h64 = cd.run(1, nt, history=True)
        cd.close()
        u, s = _udofs(m)
        assert np.abs(h64[:, u]).max() > 0 and np.abs(h64[:, s]).max() > 0
        eu = rel_l2(ref[:, b, u], h64[:, u])
        es = rel_l2(ref[:, b, s], h64[:, s])
        assert eu <= TOL_MIXED and es <= TOL_MIXED, (b, eu, es)


def test_uneven_ensemble_matches_oracle_and_single_runs(gpu):
    """Instances of uneven grids in one fused launch (svl_cdx_create_ensemble):
    each embedded in the bounding grid, only the tiles meeting its own nodes
    scheduled, several tiles per CTA.  Every instance's history against the
    oracle (<= 1e-5) and against the same instance run alone on its own grid
    (the embedding changes no arithmetic: bit for bit)."""
    from svl_gb300 import StructuredEnsemble
    shapes = [(10, 8, 6), (14, 6, 9), (7, 12, 5)]
    nt = 150
    models = [h8_box(*s, seed=10 + b, nt=nt) for b, s in enumerate(shapes)]
    dt = min(d for _, _, d in models)
    inst = [(m, L) for m, L, _ in models]
    ens = StructuredEnsemble([(s, (0.0, 0.0, 0.0)) for s in shapes], (2.0, 2.0, 2.0), inst, dt)
    assert ens.set_ctas(5) == 5
    for b in range(len(inst)):
        ens.Initialize(b)
    hist = ens.split(ens.run(1, nt, history=True))
    last = [ens.get(b) for b in range(len(inst))]
    ens.close()
    for b, ((m, L), s) in enumerate(zip(inst, shapes)):
        ho, *_ = O.cd_run(m, L, dt, nt, mode=1)
        assert np.abs(ho).max() > 0
        assert rel_l2(hist[b], ho) <= TOL_MIXED, b
        assert np.array_equal(hist[b][-1], last[b])
        one = StructuredCentralDifference(s, (2.0, 2.0, 2.0), [(m, L)], dt)
        one.Initialize(0)
        h1 = one.run(1, nt, history=True)
        one.close()
        assert np.array_equal(h1[:, 0, :], hist[b]), b


def test_ensemble_rejects_mismatched_element_size(gpu):
    from svl_gb300 import StructuredEnsemble
    a = h8_box(6, 5, 4, seed=1, nt=20)
    b = h8_box(6, 5, 4, seed=2, nt=20, h=1.0)
    with pytest.raises(SvlError) as ei:
        StructuredEnsemble([((6, 5, 4), (0.0, 0.0, 0.0))] * 2, (2.0, 2.0, 2.0), [a[:2], b[:2]], a[2])
    assert ei.value.code in (capi.SVL_ERR_INVALID, capi.SVL_ERR_UNSUPPORTED)


def test_schedules_give_identical_results_and_tuner_keeps_one(gpu):
    """Every schedule (tile order, CTA count, band block size and stream
    priority) gives the same bits: the per-node sums keep their element
    order whatever tile a CTA takes next.  The tuner returns a valid
    schedule and leaves it in effect."""
    nx, ny, nz, npml = 16, 16, 12, 3
    nt = 40
    inst, dt = _pml_instances(nx, ny, nz, npml, (1, 2), nt)
    cdx = StructuredCentralDifference((nx, ny, nz), (2.0, 2.0, 2.0), inst, dt)
    ref = None
    for sched in ({}, dict(tile_order=1, band_threads=256), dict(tile_order=2, ctas=7, band_stream_high_priority=0),
                  dict(tile_order=3, ctas=3, band_threads=128)):
        if sched:
            cdx.set_schedule(**sched)
        for b in range(len(inst)):
            cdx.Initialize(b)
        hist = cdx.run(1, nt, history=True)
        if ref is None:
            ref = hist
        else:
            assert np.array_equal(hist, ref), sched
    best = cdx.tune(1, 3)
    assert best["tile_order"] in (0, 1, 2, 3) and best["band_threads"] in (128, 256) and best["ms_per_step"] > 0
    assert {k: best[k] for k in cdx.SCHEDULE_KEYS} == cdx.schedule()
    for b in range(len(inst)):
        cdx.Initialize(b)
    assert np.array_equal(cdx.run(1, nt, history=True), ref)
    cdx.close()
