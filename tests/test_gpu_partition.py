"""Pre-processed SVL models (partition files written by the SeismoVLAB
pre-processor, tests/golden/partition_*) run end to end on the GPU through
the partition reader, against the oracle, with the node recorders written in
the run-process's format."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300.partition import load_partition
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _part(case):
    return load_partition(GOLD / ("partition_%s" % case) / "Partition" / "Fixture.1.0.json")


def _read_recorder(path):
    lines = path.read_text().splitlines()
    nn, ndofs, ntotal, nt = map(int, lines[0].split())
    head = [list(map(int, ln.split())) for ln in lines[1:1 + nn]]
    rows = np.array([[float(v) for v in ln.split()] for ln in lines[1 + nn:]])
    return (nn, ndofs, ntotal, nt), head, rows


@pytest.mark.parametrize("case", ["q4_cd", "q4_j2_column", "q4_lysmer_cd"])
def test_cd_partitions_match_oracle_and_record(gpu, case, tmp_path):
    p = _part(case)
    U = p.run(solution_dir=tmp_path)
    ho, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1, mode=1)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-12
    r = p.recorders[0]
    (nn, ndofs, ntotal, nt), head, rows = _read_recorder(tmp_path / r.file)
    assert (nn, ntotal, nt) == (len(r.ids), p.model.ntotal, p.nt) and rows.shape[0] == p.nt - 1
    cols = [d for h in head for d in h[2:]]
    assert [h[0] for h in head] == r.ids
    assert np.allclose(rows, U[:, cols], rtol=10.0 ** -r.precision, atol=0)


def test_newmark_partition_matches_oracle(gpu, tmp_path):
    p = _part("h8_newmark_body")
    U = p.run(solution_dir=tmp_path)
    ho, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-8            # the file's PETSc tolerance is 1e-10
    assert (tmp_path / p.recorders[0].file).exists()


def test_damped_newmark_partition_matches_oracle(gpu, tmp_path):
    p = _part("q4_newmark_rayleigh")
    assert np.any(p.model.rayleigh[:, 1] > 0)
    U = p.run(solution_dir=tmp_path)
    ho, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-9            # the file's PETSc tolerance is 1e-12


def test_pml_partition_extended_newmark_matches_oracle(gpu, tmp_path):
    p = _part("q4_pml_extended")
    U = p.run(solution_dir=tmp_path)
    ho, *_ = O.xnewmark_run(p.model, p.loads, p.dt, p.nt - 1)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-8
    (nn, ndofs, ntotal, nt), head, rows = _read_recorder(tmp_path / p.recorders[0].file)
    assert ntotal == p.model.ntotal and rows.shape == (p.nt - 1, ndofs)


def test_pml_j2_newton_partition_matches_oracle(gpu, tmp_path):
    """NEWMARK + NEWTON on J2 layers over PML: NewmarkBeta on a PML model runs
    on the PML-capable handle in NewmarkBeta mode."""
    p = _part("q4_pml_j2_newton")
    U = p.run(solution_dir=tmp_path)
    ho, *_ = O.xnewmark_run(p.model, p.loads, p.dt, p.nt - 1, algo=10 + int(p.algorithm["cnvgtest"]),
                            maxit=int(p.algorithm["nstep"]), cnvgtol=float(p.algorithm["cnvgtol"]), newmark=True)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-8


def test_reaction_recorder_matches_oracle(gpu, tmp_path):
    """A REACTION node recorder written by the pre-processor: its last row
    against the oracle's reactions after the last step."""
    p = _part("q4_reaction_cd")
    p.run(solution_dir=tmp_path)
    rec = [r for r in p.recorders if r.response == "REACTION"][0]
    (nn, ndofs, ntotal, nt), head, rows = _read_recorder(tmp_path / rec.file)
    Ro = O.reaction_run(p.model, p.loads, p.dt, p.nt - 1, integrator="cd")
    want = Ro[[d for h in head for d in h[2:]]]
    assert rows.shape[0] == p.nt - 1 and np.abs(want).max() > 0
    assert np.allclose(rows[-1], want, rtol=1e-6, atol=1e-6 * np.abs(want).max())


def test_drm_partition_newmark_matches_oracle(gpu, tmp_path):
    p = _part("q4_drm_newmark")
    U = p.run(solution_dir=tmp_path)
    ho, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-9


def test_consistent_mass_partition_newmark_matches_oracle(gpu, tmp_path):
    """The pre-processor's default massform (CONSISTENT) on a NEWMARK
    partition: the body-load fixture with its massform switched."""
    import json
    import shutil
    from svl_gb300.partition import load_partition
    src = Path(__file__).resolve().parent / "golden" / "partition_h8_newmark_body"
    shutil.copytree(src, tmp_path / "case")
    f = tmp_path / "case" / "Partition" / "Fixture.1.0.json"
    d = json.loads(f.read_text())
    d["Global"]["massform"] = "CONSISTENT"
    f.write_text(json.dumps(d))
    p = load_partition(f)
    assert not p.model.lumped
    U = p.run(write_recorders=False)
    ho, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-9


def test_consistent_mass_partition_cd_matches_oracle(gpu, tmp_path):
    """massform CONSISTENT with Rayleigh damping (am, ak) under
    CENTRALDIFFERENCE: the non-diagonal central-difference system, solved by
    PCG on the GPU, against the oracle's factorisation."""
    p = _part("q4_consistent_cd")
    assert not p.model.lumped and p.integrator == "CENTRALDIFFERENCE"
    U = p.run(solution_dir=tmp_path)
    ho, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-9
    r = p.recorders[0]
    (nn, ndofs, ntotal, nt), head, rows = _read_recorder(tmp_path / r.file)
    cols = [d for h in head for d in h[2:]]
    assert np.allclose(rows, U[:, cols], rtol=10.0 ** -r.precision, atol=0)


def test_consistent_mass_damped_partition_newmark_matches_oracle(gpu, tmp_path):
    """The Rayleigh (am and ak) NEWMARK fixture with its massform switched to
    CONSISTENT: the general path with the consistent element mass in the
    operator, the effective force and the damping."""
    import json
    import shutil
    src = GOLD / "partition_q4_newmark_rayleigh"
    shutil.copytree(src, tmp_path / "case")
    f = tmp_path / "case" / "Partition" / "Fixture.1.0.json"
    d = json.loads(f.read_text())
    d["Global"]["massform"] = "CONSISTENT"
    f.write_text(json.dumps(d))
    p = load_partition(f)
    assert not p.model.lumped and p.model.rayleigh is not None
    U = p.run(write_recorders=False)
    ho, _ = O.newmark_run(p.model, p.loads, p.dt, p.nt - 1, solver=0)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-9


def test_body_point_load_partition_cd_matches_oracle(gpu, tmp_path):
    """POINTLOAD BODY (nodal acceleration times the node's mass) beside a
    concentrated load, central difference, written by the pre-processor."""
    p = _part("q4_bodypoint_cd")
    U = p.run(solution_dir=tmp_path)
    ho, *_ = O.cd_run(p.model, p.loads, p.dt, p.nt - 1)
    assert np.abs(ho).max() > 0
    assert rel_l2(U, ho) <= 1e-12


def _read_element_recorder(path):
    lines = path.read_text().splitlines()
    ne, ntotal, nt = map(int, lines[0].split())
    head = [list(map(int, ln.split())) for ln in lines[1:1 + ne]]
    rows = np.array([[float(v) for v in ln.split()] for ln in lines[1 + ne:]])
    return (ne, ntotal, nt), head, rows


@pytest.mark.parametrize("case,integ", [("q4_j2_element_cd", "cd"), ("h8_element_newmark", "newmark")])
def test_element_recorders_match_oracle(gpu, case, integ, tmp_path):
    """ELEMENT recorders written by the pre-processor (stress, strain,
    internal force, strain rate; J2 and elastic elements): the format of
    Recorder.cpp and the last row against the oracle's element state after
    the last step."""
    p = _part(case)
    p.run(solution_dir=tmp_path)
    epos = {int(t): i for i, t in enumerate(p.elem_tags)}
    nrec = 0
    for r in p.recorders:
        if r.name != "ELEMENT":
            continue
        nrec += 1
        (ne, ntotal, nt), head, rows = _read_element_recorder(tmp_path / r.file)
        assert (ne, ntotal, nt) == (len(r.ids), p.model.ntotal, p.nt) and rows.shape[0] == p.nt - 1
        ngp, ncomp = (4, 3) if p.model.ndim == 2 else (8, 6)
        nc = p.model.conn.shape[1] * p.model.ndim
        if r.response == "INTERNALFORCE":
            assert all(h[1] == nc and len(h) == 2 + nc for h in head)
        else:
            assert all(h[1:] == [ngp, ncomp] for h in head)
        kw = dict(integrator=integ)
        if integ == "newmark":
            kw["algo"] = 0
        want = O.element_response_run(p.model, p.loads, p.dt, p.nt - 1, r.response, [epos[t] for t in r.ids],
                                      **kw).reshape(-1)
        if r.response == "STRAINRATE":
            assert not np.any(rows)
            continue
        assert np.abs(want).max() > 0
        scale = np.abs(want).max()
        # the recorder prints ndps digits; the solutions agree to the solver tolerance
        assert np.allclose(rows[-1], want, rtol=0, atol=max(10.0 ** (1 - r.precision), 1e-7) * scale), \
            (r.file, np.abs(rows[-1] - want).max() / scale)
    assert nrec >= 2


def test_pml_reaction_recorder_newmark(gpu, tmp_path):
    """REACTION recorder on restrained PML nodes of the pre-processor's merged
    PML mesh, NewmarkBeta: PML elements add K u + C v + M a over all their
    dofs, so the stress dofs of those nodes carry reactions too."""
    p = _part("q4_pml_reaction_newmark")
    p.run(solution_dir=tmp_path)
    rec = [r for r in p.recorders if r.response == "REACTION"][0]
    (nn, ndofs, ntotal, nt), head, rows = _read_recorder(tmp_path / rec.file)
    Ro = O.reaction_run(p.model, p.loads, p.dt, p.nt - 1, integrator="xnewmark_nm")
    cols = [d for h in head for d in h[2:]]
    want = Ro[cols]
    assert any(h[1] == 5 for h in head)                  # PML nodes: 2 displacement + 3 stress dofs
    assert rows.shape[0] == p.nt - 1 and np.abs(want).max() > 0
    assert np.allclose(rows[-1], want, rtol=1e-6, atol=1e-6 * np.abs(want).max())
