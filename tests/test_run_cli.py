"""The command-line runner (python -m svl_gb300.run) with the run-process's
-dir / -file arguments: argument parsing, `$` as the rank, partition
loading, and a loud failure without a GPU (no CPU fallback)."""
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

from svl_gb300 import run as R

ROOT = Path(__file__).resolve().parent.parent
GOLD = ROOT / "tests" / "golden"


def test_arguments_follow_the_run_process():
    path, files = R.parse_args(["-dir", "/x/Partition/", "-file", "A.1.$.json", "B.1.$.json"])
    assert path == Path("/x/Partition/") and files == ["A.1.$.json", "B.1.$.json"]
    path, files = R.parse_args(["-file", "A.1.$.json", "-dir", "/y"])
    assert path == Path("/y") and files == ["A.1.$.json"]
    assert R.resolve(Path("/y"), ["A.1.$.json"]) == [Path("/y/A.1.0.json")]


def test_loads_the_fixture_and_reports_missing_files(tmp_path):
    parts = R.load_all(GOLD / "partition_q4_cd" / "Partition", ["Fixture.1.$.json"])
    assert len(parts) == 1 and parts[0].integrator == "CENTRALDIFFERENCE"
    assert R.main(["-dir", str(tmp_path), "-file", "Nope.1.$.json"]) == 2
    assert R.main(["-file", "Fixture.1.$.json"]) == 2


def test_staged_multi_file_runs_are_rejected(capsys):
    """Several -file arguments are stages on one mesh in the run-process
    (Driver.hpp:2049-2101); they are refused, not run from rest one by one."""
    d = GOLD / "partition_q4_cd" / "Partition"
    assert R.main(["-dir", str(d), "-file", "Fixture.1.$.json", "Fixture.1.$.json"]) == 2
    assert "staged runs" in capsys.readouterr().out


def test_without_a_gpu_the_run_fails_loudly(tmp_path):
    from tests.conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    shutil.copytree(GOLD / "partition_q4_cd", tmp_path / "case")
    r = subprocess.run([sys.executable, "-m", "svl_gb300.run", "-dir", str(tmp_path / "case" / "Partition"),
                        "-file", "Fixture.1.$.json"], capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert r.returncode != 0
    assert "no CUDA device" in (r.stdout + r.stderr)


@pytest.mark.gpu
def test_runs_a_partition_and_writes_its_recorders(gpu, tmp_path):
    shutil.copytree(GOLD / "partition_q4_cd", tmp_path / "case")
    r = subprocess.run([sys.executable, "-m", "svl_gb300.run", "-dir", str(tmp_path / "case" / "Partition"),
                        "-file", "Fixture.1.$.json"], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    outs = list((tmp_path / "case" / "Solution").rglob("*.out"))
    assert outs and all(o.stat().st_size > 0 for o in outs)
