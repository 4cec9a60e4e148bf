"""The C++ partition reader (svl_gb300/host/svl_partition.hpp) against the
Python reader on the fixtures written by the reference pre-processor: the
same model and load descriptors array by array (CPU), and the same answer when
the simulation block runs through the C++ Integrator mirror (GPU)."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from svl_gb300.partition import load_partition

ROOT = Path(__file__).resolve().parent.parent
FIXTURES = sorted(p for p in (ROOT / "tests/golden").glob("partition_*") if (p / "Partition").is_dir())


def _file(fx):
    return sorted((fx / "Partition").glob("*.json"))[0]


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "partition_dump"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT), str(ROOT / "tests/cpp/partition_dump.cpp"),
                        "-L", str(ROOT / "svl_gb300/lib"), "-lsvl_gb300",
                        "-Wl,-rpath," + str(ROOT / "svl_gb300/lib"), "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _eq(a, b, name):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b if b is not None else [], dtype=np.float64).ravel()
    assert a.shape == b.shape, (name, a.shape, b.shape)
    assert np.array_equal(a, b), (name, np.max(np.abs(a - b)) if a.size else 0)


@pytest.mark.parametrize("fx", FIXTURES, ids=[p.name for p in FIXTURES])
def test_cpp_reader_gives_the_python_descriptors(exe, fx):
    r = subprocess.run([str(exe), "dump", str(_file(fx))], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    c = json.loads(r.stdout)
    p = load_partition(_file(fx))
    m, L = p.model, p.loads
    assert (c["ndim"], c["nnode"], c["ntotal"], c["nfree"], c["elem_type"]) == (m.ndim, m.nnode, m.ntotal, m.nfree, m.elem_type)
    assert c["lumped"] == int(bool(m.lumped)) and c["integrator"] == p.integrator and c["nt"] == p.nt
    assert c["dt"] == p.dt and c["nrecorder"] == len(p.recorders)
    _eq(c["coords"], m.coords, "coords")
    _eq(c["totaldof"], m.totaldof, "totaldof")
    _eq(c["freedof"], m.freedof, "freedof")
    _eq(c["conn"], m.conn, "conn")
    _eq(c["elem_mat"], m.elem_mat, "elem_mat")
    _eq(c["mat_type"], m.mat_type, "mat_type")
    _eq(c["mat_param"], m.mat_param, "mat_param")
    _eq(c["thickness"], m.thickness, "thickness")
    _eq(c["node_mass"], m.node_mass, "node_mass")
    _eq(c["rayleigh"], m.rayleigh, "rayleigh")
    if m.elem_pml is not None:
        _eq(c["elem_pml"], m.elem_pml, "elem_pml")
        _eq(c["pml_param"], m.pml_param, "pml_param")
        _eq(c["node_ndof"], m.node_ndof, "node_ndof")
    else:
        assert not any(c["elem_pml"])
    _eq(c["dashpot_dof"], m.dashpot_dof, "dashpot_dof")
    _eq(c["dashpot_eta"], m.dashpot_eta, "dashpot_eta")
    _eq(c["con_slave"], m.con_slave, "con_slave")
    _eq(c["con_master"], m.con_master, "con_master")
    _eq(c["con_factor"], m.con_factor, "con_factor")
    if m.con_slave is not None:
        _eq(c["con_ptr"], m.con_ptr, "con_ptr")
    _eq(c["series_val"], np.concatenate(L.series) if L.series else [], "series_val")
    _eq(np.diff(c["series_ptr"]), [s.size for s in L.series], "series lengths")
    _eq(c["force_dof"], L.force_dof, "force_dof")
    _eq(c["force_series"], L.force_series, "force_series")
    _eq(c["force_coef"], L.force_coef, "force_coef")
    _eq(c["sm_dof"], L.sm_dof, "sm_dof")
    _eq(c["sm_series"], L.sm_series, "sm_series")
    _eq(c["sm_factor"], L.sm_factor, "sm_factor")
    _eq(c["drm_elem"], L.drm_elem, "drm_elem")
    _eq(c["drm_factor"], L.drm_factor, "drm_factor")
    if L.drm_elem:
        nodes = sorted(L.drm_motion)
        rows = -np.ones(m.nnode)
        ext = np.zeros(m.nnode)
        for i, n in enumerate(nodes):
            rows[n] = i
            ext[n] = L.drm_motion[n][1]
        _eq(c["drm_node_row"], rows, "drm_node_row")
        _eq(c["drm_node_ext"], ext, "drm_node_ext")
        _eq(c["drm_motion"], np.concatenate([L.drm_motion[n][0] for n in nodes]), "drm_motion")


@pytest.mark.parametrize("fx", [f for f in FIXTURES if "drm" not in f.name], ids=lambda p: p.name)
def test_progressive_force_of_both_mirrors(exe, fx):
    """ComputeProgressiveForce(k) = Fext(k) (+ a zero stage force): the C++
    mirror's host sum over the load entries equals the Python one's on every
    step of the pre-processor fixtures."""
    r = subprocess.run([str(exe), "fext", str(_file(fx))], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    p = load_partition(_file(fx))
    rows = [ln.split() for ln in r.stdout.splitlines()]
    assert len(rows) == p.nt + 1
    for row in rows:
        k = int(row[0])
        fc = np.array([float(v) for v in row[1:]])
        fp = p.loads.external_force(p.model.ntotal, k)
        assert np.array_equal(fc, fp), k


def test_cpp_reader_reports_what_it_does_not_cover(exe, tmp_path):
    d = json.loads(_file(ROOT / "tests/golden/partition_q4_cd").read_text())
    tag = sorted(d["Materials"], key=int)[0]
    d["Materials"][tag]["name"] = "Elastic1DLinear"
    (tmp_path / "Partition").mkdir()
    f = tmp_path / "Partition" / "M.1.0.json"
    f.write_text(json.dumps(d))
    r = subprocess.run([str(exe), "dump", str(f)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 4 and "Elastic1DLinear" in r.stdout and "not covered" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("fx", FIXTURES, ids=[p.name for p in FIXTURES])
def test_cpp_reader_runs_like_the_python_reader(exe, fx, gpu):
    r = subprocess.run([str(exe), "run", str(_file(fx))], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr
    tok = r.stdout.split()
    assert tok[0] == "final"
    uc = np.array([float(x) for x in tok[1:]])
    p = load_partition(_file(fx))
    h = p.make_integrator()
    h.Initialize()
    U = h.run(1, p.nt - 1, history=True)
    h.close()
    assert np.abs(U[-1]).max() > 0
    # same descriptors, same library calls: the same numbers
    assert np.array_equal(uc, U[-1]), np.max(np.abs(uc - U[-1]))
