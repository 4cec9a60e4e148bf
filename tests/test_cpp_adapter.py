"""The C++ Integrator mirror compiles against include/svl_gb300.h, links
libsvl_gb300.so and runs (no GPU: reports SVL_ERR_NODEVICE loudly)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _build(tmp_path):
    exe = tmp_path / "adapter_smoke"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT), str(ROOT / "tests/cpp/adapter_smoke.cpp"),
                        "-L", str(ROOT / "svl_gb300/lib"), "-lsvl_gb300",
                        "-Wl,-rpath," + str(ROOT / "svl_gb300/lib"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_adapter_builds_and_runs(tmp_path):
    from tests.conftest import gpu_available
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    if not gpu_available():
        assert "nodevice" in r.stdout


@pytest.mark.gpu
def test_cpp_adapter_steps_on_gpu(tmp_path, gpu):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    tok = r.stdout.replace("(", " ").replace(")", " ").split()
    umax, unm, uxn, diff = float(tok[1]), float(tok[3]), float(tok[5]), float(tok[7])
    assert 0.0 < umax < 1.0 and 0.0 < unm < 1.0
    # ExtendedNewmarkBeta without PML, loads or damping is NewmarkBeta
    assert abs(uxn - unm) <= 1e-9 * unm and diff <= 1e-9 * unm
    # NewmarkBeta + NewtonRaphson on an elastic model: the Linear answer up to
    # the PCG tolerance of the Linear run (1e-8)
    assert tok[8] == "newton-diff" and float(tok[9]) <= 1e-6 * unm
    # reactions at the fixed base after 100 explicit steps
    assert tok[10] == "reaction" and float(tok[11]) > 0.0
