"""The partition-file reader against files written by the SeismoVLAB
pre-processor itself (tests/golden/partition_*, made by
tests/golden/make_partition_fixtures.py): numbering, materials, loads,
constraints, support motions, recorders, and a short oracle run of each."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import _capi as capi
from svl_gb300.partition import PartitionError, load_partition, read_series

GOLD = Path(__file__).resolve().parent / "golden"


def _part(case):
    return GOLD / ("partition_%s" % case) / "Partition" / "Fixture.1.0.json"


@pytest.mark.parametrize("case", ["q4_cd", "h8_newmark_body", "q4_j2_column", "q4_newmark_rayleigh", "q4_pml_extended",
                                  "q4_pml_j2_newton", "q4_lysmer_cd", "q4_drm_newmark", "q4_reaction_cd",
                                  "q4_bodypoint_cd"])
def test_numbering_and_connectivity_follow_the_file(case):
    p = load_partition(_part(case))
    d = json.loads(_part(case).read_text())
    tags = sorted(int(t) for t in d["Nodes"])
    assert list(p.node_tags) == tags
    nnd = p.model.dof_mask().sum(axis=1)
    for i, t in enumerate(tags):
        assert list(p.model.totaldof[i, :nnd[i]]) == d["Nodes"][str(t)]["totaldof"]
        assert list(p.model.freedof[i, :nnd[i]]) == d["Nodes"][str(t)]["freedof"]
    solid = [t for t in sorted(int(x) for x in d["Elements"]) if d["Elements"][str(t)]["name"] != "ZEROLENGTH1D"]
    for i, et in enumerate(solid):
        assert [tags[j] for j in p.model.conn[i]] == d["Elements"][str(et)]["conn"]
    assert p.model.ntotal == d["Global"]["ntotal"] and p.model.nfree == d["Global"]["nfree"]


def test_q4_loads_materials_and_recorder():
    p = load_partition(_part("q4_cd"))
    assert p.integrator == "CENTRALDIFFERENCE" and p.dt == 1e-3 and p.nt == 41
    assert set(p.model.mat_type) == {capi.SVL_MAT_ELASTIC2DPLANESTRAIN}
    assert np.allclose(p.model.mat_param[1, :3], [3.0e8, 0.3, 2100.0])
    ricker = read_series(GOLD / "partition_q4_cd" / "ricker.txt")
    assert np.array_equal(p.loads.series[0], ricker)
    assert np.array_equal(p.loads.series[1], np.full(41, 2500.0))   # constant load: every step
    # point loads: the time series on dof y of node 32 (factor 1), the constant on x of node 31 (factor 0.5)
    ty = int(p.model.totaldof[list(p.node_tags).index(32), 1])
    tx = int(p.model.totaldof[list(p.node_tags).index(31), 0])
    assert list(zip(p.loads.force_dof, p.loads.force_series, p.loads.force_coef)) == [(ty, 0, -1.0), (tx, 1, 0.5)]
    r = p.recorders[0]
    assert r.response == "DISP" and r.ids == [31, 32] and r.precision == 8 and r.file == "Disp.0.out"


def test_h8_body_load_and_solver_settings():
    p = load_partition(_part("h8_newmark_body"))
    assert p.integrator == "NEWMARK" and p.solver["name"] == "PETSC" and p.solver["tol"] == 1e-10
    # body load entries sum to factor * rho * volume * series for each loaded element
    coef = np.array(p.loads.force_coef)
    assert np.isclose(coef.sum(), 2.0e3 * 2000.0 * 8.0 * 2)
    assert all(s == 0 for s in p.loads.force_series)


def test_j2_column_constraints_and_support_motion():
    p = load_partition(_part("q4_j2_column"))
    m = p.model
    assert set(m.mat_type) == {capi.SVL_MAT_PLASTICPLANESTRAINJ2}
    d = json.loads(_part("q4_j2_column").read_text())
    assert m.nconstraint == len(d["Constraints"])
    for t, c in d["Constraints"].items():
        i = list(m.con_slave).index(c["stag"])
        assert list(m.con_master[m.con_ptr[i]:m.con_ptr[i + 1]]) == c["mtag"]
    base = read_series(GOLD / "partition_q4_j2_column" / "base.txt")
    assert len(p.loads.sm_dof) == 3 and all(np.array_equal(p.loads.series[s], base) for s in p.loads.sm_series)


@pytest.mark.parametrize("case", ["q4_cd", "q4_j2_column"])
def test_oracle_runs_the_parsed_model(case):
    p = load_partition(_part(case))
    h, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1, mode=1)
    assert np.all(np.isfinite(h)) and np.abs(h).max() > 0


def test_rayleigh_dampings_by_tag_order():
    """The pre-processor adds a FREE damping over the elements missing from the
    last damping's list (SeismoVLAB.py's damping check); assigned in ascending
    tag order (Mesh::SetDamping), it overrides tag 1 on the odd elements."""
    p = load_partition(_part("q4_newmark_rayleigh"))
    d = json.loads(_part("q4_newmark_rayleigh").read_text())
    assert d["Dampings"]["3"]["name"] == "FREE"
    etags = sorted(int(t) for t in d["Elements"])
    ray = p.model.rayleigh
    for i, t in enumerate(etags):
        assert tuple(ray[i]) == ((2.5, 1.5e-3) if t % 2 == 0 else (0.0, 0.0))
    assert p.integrator == "NEWMARK"
    h, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    p.model.rayleigh = None
    h0, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.all(np.isfinite(h)) and np.linalg.norm(h - h0) > 1e-3 * np.linalg.norm(h0)


def test_pml_layers_and_extended_newmark():
    """setPMLDomain + mergeDomain output: 5-dof PML nodes tied to the soil by
    EQUAL constraints, PML2DQuad4 parameters per element, ExtendedNewmark."""
    p = load_partition(_part("q4_pml_extended"))
    d = json.loads(_part("q4_pml_extended").read_text())
    m = p.model
    assert p.integrator == "EXTENDEDNEWMARK" and m.nconstraint > 0
    assert sorted(set(m.node_ndof.tolist())) == [2, 5]
    etags = sorted(int(t) for t in d["Elements"])
    for i, t in enumerate(etags):
        e = d["Elements"][str(t)]
        assert m.elem_pml[i] == (e["name"] == "PML2DQUAD4")
        if m.elem_pml[i]:
            a = e["attributes"]
            assert list(m.pml_param[i]) == [a["n"], a["L"], a["R"]] + a["x0"] + a["npml"]
    h, U, V, A, Ub = O.xnewmark_run(m, p.loads, p.dt, p.nt - 1)
    assert np.all(np.isfinite(h)) and np.abs(h).max() > 0 and np.abs(Ub).max() > 0


def test_zero_length_dashpots():
    """ZeroLength1D + Viscous1DLinear elements become dashpots on the element's
    direction (0-based in the file, Driver.hpp:1072-1078) between its two nodes."""
    p = load_partition(_part("q4_lysmer_cd"))
    d = json.loads(_part("q4_lysmer_cd").read_text())
    tags = sorted(int(t) for t in d["Nodes"])
    pos = {t: i for i, t in enumerate(tags)}
    zl = [d["Elements"][str(t)] for t in sorted(int(x) for x in d["Elements"])
          if d["Elements"][str(t)]["name"] == "ZEROLENGTH1D"]
    assert len(zl) == p.model.dashpot_eta.size and p.model.nelem == len(d["Elements"]) - len(zl)
    for e, (a, b), eta in zip(zl, p.model.dashpot_dof, p.model.dashpot_eta):
        j = e["attributes"]["dir"]
        n1, n2 = (pos[c] for c in e["conn"])
        assert (a, b) == (p.model.totaldof[n1, j], p.model.totaldof[n2, j])
        assert eta == d["Materials"][str(e["attributes"]["material"])]["attributes"]["eta"]
    h, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1)
    p.model.dashpot_dof = p.model.dashpot_eta = None
    h0, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1)
    assert np.all(np.isfinite(h)) and np.linalg.norm(h - h0) > 1e-6 * np.linalg.norm(h0)


def test_domain_reduction_load():
    """ELEMENTLOAD GENERALWAVE: DRM elements in load-list order, per-node files
    (`$` -> node tag) with `nt nFields cond` headers (Driver.hpp:1669-1722)."""
    p = load_partition(_part("q4_drm_newmark"))
    d = json.loads(_part("q4_drm_newmark").read_text())
    L = p.loads
    etags = sorted(int(t) for t in d["Elements"])
    assert [etags[e] for e in L.drm_elem] == d["Loads"]["1"]["attributes"]["list"]
    ntags = sorted(int(t) for t in d["Nodes"])
    for n, (sig, ext) in L.drm_motion.items():
        f = (GOLD / "partition_q4_drm_newmark" / "drm" / ("node%d.txt" % ntags[n])).read_text().split()
        assert int(f[0]) == sig.shape[0] and int(f[2]) == ext
        assert float(f[3]) == sig[0, 0]
    h, _ = O.newmark_run(p.model, L, p.dt, p.nt - 1, solver=0)
    assert np.all(np.isfinite(h)) and np.abs(h).max() > 0


def test_integrator_names_are_the_run_process_ones(tmp_path):
    d = json.loads(_part("h8_newmark_body").read_text())
    d["Simulations"]["attributes"]["integrator"]["name"] = "NEWMARKBETA"
    (tmp_path / "Partition").mkdir()
    f = tmp_path / "Partition" / "x.json"
    f.write_text(json.dumps(d))
    (tmp_path / "body.txt").write_text((GOLD / "partition_h8_newmark_body" / "body.txt").read_text())
    p = load_partition(f)
    with pytest.raises(PartitionError, match="NEWMARKBETA"):
        p.make_integrator()


def test_uncovered_content_is_named(tmp_path):
    d = json.loads(_part("q4_cd").read_text())
    d["Dampings"]["1"]["name"] = "CAUGHEY"
    (tmp_path / "Partition").mkdir()
    f = tmp_path / "Partition" / "x.json"
    f.write_text(json.dumps(d))
    (tmp_path / "ricker.txt").write_text((GOLD / "partition_q4_cd" / "ricker.txt").read_text())
    with pytest.raises(PartitionError, match="CAUGHEY"):
        load_partition(f)


def test_newton_algorithm_and_j2_layers_over_pml():
    """Newton settings (nstep, cnvgtol, cnvgtest as the pre-processor writes
    them) and a J2 material on the top solid layers of a PML model; the
    reference oracle in NewmarkBeta mode runs it."""
    from oracle import oracle as O
    p = load_partition(_part("q4_pml_j2_newton"))
    assert p.integrator == "NEWMARK"
    assert p.algorithm["name"] == "NEWTON" and p.algorithm["nstep"] == 3 and p.algorithm["cnvgtest"] == 1
    mt = p.model.mat_type[p.model.elem_mat]
    assert (mt == capi.SVL_MAT_PLASTICPLANESTRAINJ2).sum() == 12 and p.model.elem_pml.sum() == 36
    its = np.zeros(10, np.int32)
    h, *_ = O.xnewmark_run(p.model, p.loads, p.dt, 10, algo=10 + 1, maxit=3, cnvgtol=1e-12, newmark=True,
                           step_iters=its)
    assert np.abs(h).max() > 0 and np.all(its == 3)


def test_reaction_recorder_is_read():
    p = load_partition(_part("q4_reaction_cd"))
    resp = sorted(r.response for r in p.recorders)
    assert resp == ["DISP", "REACTION"]
    rec = [r for r in p.recorders if r.response == "REACTION"][0]
    assert len(rec.ids) == 4


def test_body_point_load_is_acceleration_times_nodal_mass():
    """POINTLOAD BODY (Assembler.cpp:373-394): Fn(i) * Mn(i) with Mn the
    node's mass entries, nothing at nodes without a Masses entry; every load
    is assembled into its own vector and added with its combination factor."""
    p = load_partition(_part("q4_bodypoint_cd"))
    d = json.loads(_part("q4_bodypoint_cd").read_text())
    tags = list(p.node_tags)
    L = p.loads
    acc = read_series(_part("q4_bodypoint_cd").parent.parent / "accel.txt")
    entries = {}
    for dof, ser, coef in zip(L.force_dof, L.force_series, L.force_coef):
        entries.setdefault(dof, []).append((ser, coef))
    n31, n32, n33 = tags.index(31), tags.index(32), tags.index(33)
    m = p.model
    # node 31: mass 120 on both dofs, body load only
    assert entries[int(m.totaldof[n31, 0])] == [(0, 0.6 * 120.0)]
    assert entries[int(m.totaldof[n31, 1])] == [(0, -0.8 * 120.0)]
    # node 32: body load with its masses, then the concentrated load (factor 0.5)
    assert entries[int(m.totaldof[n32, 0])] == [(0, 0.6 * 250.0), (1, 0.5 * 1.0)]
    assert entries[int(m.totaldof[n32, 1])] == [(0, -0.8 * 400.0)]
    # node 33 has no mass entry: no body load
    assert int(m.totaldof[n33, 0]) not in entries and int(m.totaldof[n33, 1]) not in entries
    assert np.allclose(L.series[0], acc)
    h, *_ = O.cd_run(m, L, p.dt, 20)
    assert np.abs(h[:, int(m.totaldof[n31, 1])]).max() > 0
