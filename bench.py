#!/usr/bin/env python3
"""Benchmark of the explicit central-difference hot path (DOF-steps/s).

A "step" is one time step of the whole batch.  Default workload: the 3D
configuration as specified -- lin3DHexa8 128 x 128 x 64, h = 2 m, log-normal
Vs field (mean 400 m/s, COV 0.2, exponential correlation 20 m), nu = 0.3,
rho = 2100, double-couple body force (Ricker 3 Hz), dt = 0.5 h / max Vp, with
10-element PML3DHexa8 layers on the four sides and the bottom (9 dofs at
their nodes) advanced by the library's explicit PML scheme -- as a batch of 4
seeded realisations on the mixed-precision path: the elastic interior by the
tcgen05 tensor-core step (TF32 hi/lo element forces, FP32 accumulation), the
PML band by FP32 kernels, the state as compensated FP32 pairs ("tf32x2+f32x2": two TF32 products, hi and lo displacements times the exact stiffness patterns).
The FP64 plain path (the same scheme in FP64 on the general handle) is timed
on one realisation beside it, with the mixed result's error against it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--instances B]
                    [--workload config2|config2_box|config1|config3]

value   : free displacement DOF x instances x steps / device time of the K
          steps (CUDA events on the library's stream, inputs resident in HBM,
          working set ~1.9 GB > L2, no flush needed).
e2e     : the same metric through the C ABI with host buffers: handle creation
          from the host model arrays, then the configured run length with every
          instance's full total-dof vector copied to a page-locked host buffer
          after every step.
roofline: the dominant kernel's algorithmic bytes over its own device time
          (per-kernel CUDA events), against MEASURED_PEAKS.json.
reference arm (--impl reference): the CPU oracle of the same scheme on the
          box's host cores, on the same workload and instance count (a bounded
          sample of steps), built without the product library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent

sys.path.insert(0, str(ROOT))

ALGO_BYTES_PER_DOF = {2: 40.0, 3: 37.0}
# steps of the end-to-end run per workload (the configured run lengths)
E2E_STEPS = {"config1": 2000, "config2": 4000, "config2_box": 4000, "config3": 4000}
# plane-strain J2 state read + written per element and step: 2 x 9 doubles x 4 Gauss points
J2_STATE_BYTES_PER_ELEMENT = 576.0


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """SM clock and clock-event reasons sampled DURING the timed region, read
    in-process through NVML (libnvidia-ml, read-only queries) every 2 ms on a
    helper thread; falls back to `nvidia-smi -lms 20` when NVML cannot be
    loaded.  Nothing is set."""

    # clock-event reason bits of nvmlDeviceGetCurrentClocksEventReasons
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self.max_mhz = None
        self._stop = False
        self._thread = None
        self._proc = None
        self._path = None
        self._nvml = None

    def _nvml_handle(self):
        import ctypes as C
        nv = C.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        h = C.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.gpu)
            bus = ("%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)).encode()
        except Exception:
            bus = None
        if bus is None or nv.nvmlDeviceGetHandleByPciBusId_v2(bus, C.byref(h)) != 0:
            if nv.nvmlDeviceGetHandleByIndex_v2(self.gpu, C.byref(h)) != 0:
                raise RuntimeError("no NVML handle")
        mx = C.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:          # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        return nv, h

    def _loop(self):
        import ctypes as C
        nv, h = self._nvml
        clk, rs = C.c_uint(), C.c_ulonglong()
        while not self._stop:
            a = nv.nvmlDeviceGetClockInfo(h, 1, C.byref(clk))
            b = nv.nvmlDeviceGetCurrentClocksEventReasons(h, C.byref(rs))
            if a == 0:
                self.samples.append((float(clk.value), int(rs.value) if b == 0 else 0))
            time.sleep(0.002)

    def __enter__(self):
        try:
            self._nvml = self._nvml_handle()
            import threading
            self._thread = threading.Thread(target=self._loop, daemon=True)
            self._thread.start()
        except Exception:
            self._nvml = None
            try:
                fd, self._path = tempfile.mkstemp(suffix=".csv")
                os.close(fd)
                self._proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.gpu),
                     "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                     "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                     "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "20"],
                    stdout=open(self._path, "w"), stderr=subprocess.DEVNULL)
            except Exception:
                self._proc = None
        return self

    def __exit__(self, *a):
        self._stop = True
        if self._thread is not None:
            self._thread.join(timeout=2)
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if self._nvml is not None:
            if not self.samples:
                return None
            reasons = sorted({n for _, r in self.samples for bit, n in self.REASONS.items() if r & bit})
            return {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                    "reasons": reasons, "samples": len(self.samples), "source": "nvml, 2 ms"}
        if not self._path or not os.path.exists(self._path):
            return None
        rows = [[x.strip() for x in line.split(",")] for line in open(self._path)]
        os.unlink(self._path)
        rows = [r for r in rows if len(r) >= 6 and r[0].replace(".", "").isdigit()]
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[2:6]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(float(r[0]) for r in rows), "sm_max_mhz": max(float(r[1]) for r in rows),
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi, 20 ms"}


def build_workload(name, seed=0, native=True):
    """(model, loads, dt, description) of a workload.  native=False builds the
    config-2 model without the product library (numpy grid and numbering, the
    oracle's element body force), for the reference arm."""
    from svl_gb300 import workloads
    if name == "config3":
        m, L, dt, info = workloads.config3(seed=seed, nt=4001)
        desc = ("ensemble of %d plane-strain J2 soil columns (lin2DQuad4, 10 wide, %d-%d elements high, h=0.5 m), "
                "periodic sides, base support motion, CD; dt=%.3g (stable step)" %
                (info["columns"], info["heights"][0], info["heights"][1], dt))
        return m, L, dt, desc
    if name == "config1":
        m, L, dt = workloads.config1()
        desc = "lin2DQuad4 200x100 plane-strain box, CD"
    elif name == "config2":
        m, L, dt = workloads.config2_pml(seed=seed, element_force=None if native else _oracle_body_force)
        desc = ("lin3DHexa8 128x128x64 (h=2 m, log-normal Vs mean 400 m/s, COV 0.2, corr 20 m, nu=0.3, rho=2100), "
                "10-element PML3DHexa8 layers on the sides and bottom (9 dofs at their nodes), double-couple Ricker "
                "3 Hz body force, explicit central difference with the staggered PML scheme, dt=0.5 h/max Vp")
    elif name == "config2_box":
        m, L, dt = workloads.config2(seed=seed)
        desc = ("lin3DHexa8 128x128x64 box (h=2 m, log-normal Vs, COV 0.2, corr 20 m), CD; fixed bottom and roller "
                "sides instead of the PML band")
    else:
        raise SystemExit("unknown workload %s" % name)
    return m, L, dt, desc


def _oracle_body_force(m, e, q):
    """Element body force by the CPU oracle (lin3DHexa8 rho * int(N^T q)), on a
    one-element model holding element e's nodes and material."""
    from oracle import oracle as O
    from svl_gb300.model import Model
    nodes = m.conn[e]
    one = Model(ndim=3, coords=np.ascontiguousarray(m.coords[nodes]), totaldof=np.arange(24, dtype=np.int32).reshape(8, 3),
                freedof=np.arange(24, dtype=np.int32).reshape(8, 3), conn=np.arange(8, dtype=np.int32)[None, :],
                elem_type=m.elem_type, elem_mat=np.zeros(1, np.int32),
                mat_type=np.ascontiguousarray(m.mat_type[[m.elem_mat[e]]]),
                mat_param=np.ascontiguousarray(m.mat_param[[m.elem_mat[e]]]))
    return O.body_force(one, 0, q)


def free_disp_dofs(m):
    """Free displacement dofs (the metric's DOF count; PML stress dofs excluded)."""
    return int(np.sum(np.asarray(m.freedof)[:, :m.ndim] >= 0))


def has_pml(m):
    return m.elem_pml is not None and bool(np.any(m.elem_pml))


def cpu_run(m, L, dt, nsteps, timing):
    """The CPU oracle of the workload's scheme: the explicit PML scheme on PML
    models, the plain central difference (fast mode) otherwise."""
    from oracle import oracle as O
    if has_pml(m):
        return O.cdpml_run(m, L, dt, nsteps, history=False, timing=timing)
    return O.cd_run(m, L, dt, nsteps, mode=1, history=False, timing=timing)


def cpu_baseline(insts, dt, steps_cap, budget_s=20.0):
    """Oracle (CPU port of the path) on all host threads.  The plain central
    difference: a bounded number of steps of every instance, sized to about
    budget_s.  The explicit PML scheme (whose oracle forms every PML element's
    72 x 72 matrices each step, as PML3DHexa8 does, about 10 s per step at the
    full configuration): 2 steps of instance 0, all instances being the same
    size.  Set-up is not timed."""
    from oracle import oracle as O
    nthreads = O.num_threads()
    t = {}
    m0, L0 = insts[0][0], insts[0][1]
    if has_pml(m0):
        n = max(1, min(steps_cap, 2))
        cpu_run(m0, L0, dt, n, t)
        val = free_disp_dofs(m0) * n / t["seconds"]
        return {"value": val, "unit": "DOF-steps/s", "cores": nthreads, "kind": "port",
                "sample": "%d time steps of instance 0 of the %d (same size) on the CPU oracle's explicit PML scheme "
                          "(CDPml: element matrices of PML3DHexa8 formed per step, OpenMP element loops, "
                          "element-order assembly); set-up not timed" % (n, len(insts))}
    cpu_run(m0, L0, dt, 1, t)                             # sizing step
    per = max(t["seconds"], 1e-6) * len(insts)
    n = int(max(1, min(steps_cap, budget_s / per)))
    secs, work = 0.0, 0
    for m, L in ((x[0], x[1]) for x in insts):
        cpu_run(m, L, dt, n, t)
        secs += t["seconds"]
        work += free_disp_dofs(m) * n
    out = {"value": work / secs, "unit": "DOF-steps/s", "cores": nthreads, "kind": "port",
           "sample": "%d time step(s) of each of the %d instances on the CPU oracle's central difference (fast "
                     "mode: OpenMP element loop, element-order assembly)" % (n, len(insts))}
    try:
        t1 = {}
        O.cd_run(m0, L0, dt, 1, mode=0, history=False, timing=t1)
        out["single_thread_reference_faithful"] = {
            "value": free_disp_dofs(m0) / t1["seconds"], "unit": "DOF-steps/s", "cores": 1,
            "sample": "1 time step of instance 0, the oracle's reference-faithful mode"}
    except Exception as exc:  # noqa: BLE001
        out["single_thread_reference_faithful"] = {"error": str(exc)[:200]}
    return out


def implicit_pcg(steps=500, warm=100, tol=1e-8):
    """Config 4 over its configured run: Newmark (average acceleration) +
    Linear on the 64^3 layered H8 model, each step's effective-stiffness solve
    to a true relative residual of `tol`.  Jacobi-PCG runs all `steps` steps;
    the learned arm runs the first `warm` steps with Jacobi-PCG (as the
    configuration's training window), trains the preconditioner (timed), then
    runs the remaining steps with it (flexible CG, Jacobi fallback).  Both arms
    apply the stiffness in single precision in their inner iterations and
    confirm every answer with the FP64 operator.  Device time per phase by
    CUDA events; training by the host clock."""
    from svl_gb300 import NewmarkBeta, workloads
    m, L, dt = workloads.config4(nt=steps + 2)
    jac = NewmarkBeta(m, L, dt, pcg_tol=tol)
    jac.Initialize()
    ms_j = jac.run_timed(1, steps)
    itj = jac.stats()[0]
    Uj = jac.GetDisplacements()
    jac.close()
    lrn = NewmarkBeta(m, L, dt, pcg_tol=tol)
    lrn.Initialize()
    ms_w = lrn.run_timed(1, warm)
    it_w = lrn.stats()[0]
    t0 = time.perf_counter()
    loss = lrn.train_preconditioner(1 + warm, **NN_TRAIN)
    train_s = time.perf_counter() - t0
    it0 = lrn.stats()[0]
    ms_l = lrn.run_timed(1 + warm, steps - warm)
    it1, _, res = lrn.stats()
    solves, fallbacks, jref = lrn.precond_stats()
    Ul = lrn.GetDisplacements()
    lrn.close()
    j_per = ms_j / steps
    l_per = ms_l / (steps - warm)
    end_j = ms_j / 1e3
    end_l = ms_w / 1e3 + train_s + ms_l / 1e3
    return {"workload": ("lin3DHexa8 64x64x64 (h=1 m), layered G (100x contrast) x 10%% log-normal, "
                         "Newmark beta=1/4 gamma=1/2, dt=10x explicit limit, fixed bottom, roller sides, %d steps" % steps),
            "free_dof": m.nfree, "steps": steps, "tol": tol, "residual": "true |b - K_eff x| / |b|, FP64",
            "operator": "single-precision stiffness action in the inner iterations, FP64 true residual",
            "jacobi": {"ms_per_step": j_per, "pcg_iters_per_step": itj / steps, "seconds": end_j},
            "learned": {"ms_per_step": l_per, "pcg_iters_per_step": (it1 - it0) / (steps - warm),
                        "rel_residual_last": res, "fallbacks": fallbacks, "solves": solves,
                        "jacobi_steps_first": warm, "jacobi_first_seconds": ms_w / 1e3,
                        "train_seconds": train_s, "train_loss": loss, "train": dict(NN_TRAIN),
                        "seconds": end_l},
            "speedup_per_solve_learned_over_jacobi": j_per / l_per,
            "end_to_end_ratio_jacobi_over_learned": end_j / end_l,
            "break_even_solves_after_training": (train_s * 1e3 / (j_per - l_per)) if j_per > l_per else None,
            "rel_l2_final_u_learned_vs_jacobi": float(np.linalg.norm(Ul - Uj) / max(np.linalg.norm(Uj), 1e-300))}


def uneven_ensemble(steps=200, warm=20):
    """Instances of uneven grids in one fused launch per step
    (svl_cdx_create_ensemble) against the same instances advanced one handle
    each: four config-2 style boxes (no PML band) of different sizes."""
    from svl_gb300 import StructuredCentralDifference, StructuredEnsemble, workloads
    shapes = [(128, 128, 64), (96, 128, 48), (112, 80, 64), (64, 64, 32)]
    inst = [workloads.config2(*s, seed=20 + b, nt=steps + warm + 10) for b, s in enumerate(shapes)]
    dt = min(d for _, _, d in inst)
    pairs = [(m, L) for m, L, _ in inst]
    ndof = sum(free_disp_dofs(m) for m, _ in pairs)
    ens = StructuredEnsemble([(s, (0.0, 0.0, 0.0)) for s in shapes], (2.0, 2.0, 2.0), pairs, dt)
    sched = ens.tune(1, 8)
    for b in range(len(pairs)):
        ens.Initialize(b)
    ens.run(1, warm)
    ms_ens = ens.run_timed(1 + warm, steps) / steps
    ens.close()
    ms_one = 0.0
    for s, pr in zip(shapes, pairs):
        one = StructuredCentralDifference(s, (2.0, 2.0, 2.0), [pr], dt)
        one.Initialize(0)
        one.run(1, warm)
        ms_one += one.run_timed(1 + warm, steps) / steps
        one.close()
    return {"workload": "4 lin3DHexa8 boxes %s (h=2 m, log-normal Vs), fixed bottom, roller sides, one fused "
                        "launch per step" % ", ".join("x".join(map(str, s)) for s in shapes),
            "free_dof": ndof, "steps": steps, "ms_per_step": ms_ens, "value": ndof / (ms_ens / 1e3),
            "unit": "DOF-steps/s", "separate_handles_ms_per_step": ms_one,
            "speedup_over_separate_handles": ms_one / ms_ens, "schedule": sched}


def nonlinear_newton(steps=8, warm=4, tol=1e-8, size=(64, 64, 32), n_j2=8):
    """Newmark + NewtonRaphson (3 iterations per step, test 4 disabled by
    cnvgtol = 0, as in the configuration) on the config-5 style model at a
    reduced size: J2 top layers over an elastic base on Lysmer dashpots, base
    plane wave as the Lysmer input force.  Jacobi-PCG per Newton iteration
    to a true relative residual of `tol`; FP64 return mapping and tangents."""
    from svl_gb300 import NewmarkBeta, workloads
    m, L, dt = workloads.config5(*size, n_j2=n_j2, nt=warm + steps + 2)
    nm = NewmarkBeta(m, L, dt, pcg_tol=tol, algorithm="newton", maxit=3, cnvgtol=0.0, cnvgtest=4)
    nm.Initialize()
    nm.run(1, warm)
    it0 = nm.stats()[0]
    n0 = nm.newton_stats()[0]
    ms = nm.run_timed(1 + warm, steps)
    it1, _, res = nm.stats()
    n1 = nm.newton_stats()[0]
    U = nm.GetDisplacements()
    nm.close()
    return {"workload": "lin3DHexa8 %dx%dx%d (h=2 m), top %d layers Plastic3DJ2 (su 40-150 kPa by depth), "
                        "elastic base on Lysmer dashpots, band-limited base plane wave (PGA 0.3 g), "
                        "Newmark-Newton 3 iterations per step" % (size + (n_j2,)),
            "free_dof": m.nfree, "steps": steps, "ms_per_step": ms / steps,
            "newton_iters_per_step": (n1 - n0) / steps, "pcg_iters_per_newton_iter": (it1 - it0) / max(n1 - n0, 1),
            "pcg_tol": tol, "rel_residual_last": res, "finite": bool(np.all(np.isfinite(U))),
            "dof_newton_iters_per_s": m.nfree * (n1 - n0) / (ms / 1e3)}


def nonlinear_newton_pml(steps=3, warm=2, tol=1e-8, size=(64, 64, 32), npml=5, n_j2=8):
    """NewmarkBeta + NewtonRaphson (3 iterations per step, cnvgtol = 0) on the
    config-5 model with a PML half-space at a reduced size: PML3DHexa8 layers
    on the sides and the bottom, J2 top layers, an up-going plane-wave source
    plane.  NewmarkBeta on a PML model runs on the MINRES handle (symmetric
    indefinite effective matrix) to a relative residual of `tol` in the
    |diag|^-1 norm.  Timed by the host clock around the step loop (the solver
    reads its scalars every iteration, so the stream is synchronous)."""
    from svl_gb300 import NewmarkBeta, workloads
    m, L, dt = workloads.config5_pml(*size, npml=npml, n_j2=n_j2, nt=warm + steps + 2)
    nm = NewmarkBeta(m, L, dt, pcg_tol=tol, pcg_maxit=200000, algorithm="newton", maxit=3, cnvgtol=0.0,
                     cnvgtest=4)
    nm.Initialize()
    nm.run(1, warm)
    it0 = nm.stats()[0]
    n0 = nm.newton_stats()[0]
    t0 = time.perf_counter()
    nm.run(1 + warm, steps)
    sec = time.perf_counter() - t0
    it1, _, res = nm.stats()
    n1 = nm.newton_stats()[0]
    U = nm.GetDisplacements()
    nm.close()
    return {"workload": "lin3DHexa8 %dx%dx%d (h=2 m) with %d-element PML3DHexa8 layers on the sides and bottom, "
                        "top %d solid layers Plastic3DJ2, plane-wave source plane (PGA 0.3 g), "
                        "NewmarkBeta-Newton 3 iterations per step, MINRES" % (size + (npml, n_j2)),
            "total_dof": m.ntotal, "free_dof": m.nfree, "pml_elements": int(m.elem_pml.sum()), "steps": steps,
            "ms_per_step": sec * 1e3 / steps, "newton_iters_per_step": (n1 - n0) / steps,
            "minres_iters_per_newton_iter": (it1 - it0) / max(n1 - n0, 1), "tol": tol,
            "rel_residual_last": res, "finite": bool(np.all(np.isfinite(U))),
            "dof_newton_iters_per_s": m.nfree * (n1 - n0) / sec}


def implicit_profile():
    from svl_gb300 import NewmarkBeta, workloads
    from svl_gb300 import _capi as capi
    m, L, dt = workloads.config4(nt=10)
    nm = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    nm.Initialize()
    nm.run(1, 2)
    w = (np.random.default_rng(0).standard_normal(capi.lib().svl_nn_num_weights()) * 0.02).astype(np.float32)
    nm.nn_weights(w)
    nm.set_preconditioner(capi.SVL_PRECOND_LEARNED)
    nm.run(3, 1)
    print(json.dumps({"implicit_profile": True, "pcg_iters_total": nm.stats()[0], "precond_stats": nm.precond_stats()}))
    nm.close()
    return 0


NN_TRAIN = {"solve_steps": 0, "n_synthetic": 300, "iters": 600, "batch": 8, "lr": 2e-3, "seed": 1, "max_sweeps": 5,
            "crop": 33}


def max_over_ranks(pg, ms, device="cuda"):
    """The slowest rank's time: all-reduce MAX (every rank receives it), then a
    barrier.  pg = None (one process) returns ms."""
    if not pg:
        return ms
    import torch
    t = torch.tensor([float(ms)], device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    pg.barrier()
    return float(t.item())


def job_value(world_size, nfree_per_rank, steps, ms):
    """Whole-job DOF-steps/s: every rank advances its own instances (weak
    scaling), so the job's work is world_size x one rank's."""
    return world_size * nfree_per_rank * steps / (ms / 1e3)


def rank_seed(rank, workload, b):
    """Seed of instance b on `rank`: ensembles (config 3) get different
    columns per rank; the single-mesh workloads run the same model as replicas."""
    return (rank * 1000 if workload == "config3" else 0) + b


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# Algorithmic bytes of the PML band per step (FP32 pairs): per PML node the
# state read (u_n, u_{n-1}, ubar: 3 pairs each; S^{n+1/2}, S^{n-1/2}, Sbar:
# 6 pairs each = 216 B) and written (u_{n+1}, ubar, S^{n+3/2}, Sbar = 144 B),
# its constants (1/d x3, c, Ku, Gu = 24 B; four 9-entry stress blocks = 144 B)
# and the solid force handed over by the tensor-core step (12 B): 540 B; per
# PML element its geometry, node indices and b0 (84 B).
PML_BYTES_PER_NODE = 540.0
PML_BYTES_PER_ELEMENT = 84.0
# DRAM bytes of one k_cdx_step launch on config 2 with 4 instances
# (dram__bytes_read.sum 298 MB + dram__bytes_write.sum 59 MB, one ncu capture
# of the 3-metric pass; the command is in the committed profile summary)
CDX_STEP_DRAM_BYTES_4INST = 357.0e6


def workload_config(desc, insts, dt, e2e_steps):
    """The workload's identity, the same dict on both arms."""
    m = insts[0][0]
    return {"workload": desc, "instances": len(insts), "free_dof_per_instance": free_disp_dofs(m),
            "total_dof_per_instance": int(m.ntotal), "elements_per_instance": int(m.nelem),
            "pml_elements_per_instance": int(np.sum(m.elem_pml)) if has_pml(m) else 0,
            "dt": dt, "run_steps": e2e_steps, "data": "synthetic (seeded realisations)"}


def reference_arm(args, warm):
    """The reference's CPU path of the hot path on the machine's host cores: the
    oracle of the same scheme (reference-faithful restatement; the SVL binary
    needs Eigen/PETSc/MUMPS, absent here) on the same workload and instance
    count, a bounded sample of steps of every instance; built without the
    product library."""
    nb = args.instances if args.workload in ("config2", "config2_box") else 1
    insts = [build_workload(args.workload, seed=b, native=False) for b in range(nb)]
    # the instances differ only in their Vs field; the PML scheme's sample runs instance 0
    dt = min(x[2] for x in insts)
    cb = cpu_baseline(insts, dt, steps_cap=max(1, min(args.steps, 20)), budget_s=25.0)
    line = {"metric": "DOF-steps/s", "value": cb["value"], "unit": "DOF-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": warm, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(insts[0][3], insts, dt, E2E_STEPS[args.workload]),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "DOF-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def fp64_plain_run(m, L, dt, steps):
    """The FP64 plain path on one realisation: the general handle (the explicit
    PML scheme in FP64 on a PML model, svl_cd otherwise); returns (ms per step,
    final total-dof vector, launches per step or None)."""
    from svl_gb300 import CentralDifference
    h = CentralDifference(m, L, dt)
    h.Initialize()
    h.run(1, 2)
    h.Initialize()
    if hasattr(h, "run_timed"):
        ms = h.run_timed(1, steps)
    else:
        t0 = time.perf_counter()
        h.run(1, steps)                   # synchronises at the end (reads its status)
        ms = (time.perf_counter() - t0) * 1e3
    U = h.GetDisplacements()
    h.close()
    return ms / steps, U


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config2_box", "config3"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--instances", type=int, default=4)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the uneven-ensemble leg")
    ap.add_argument("--implicit-steps", type=int, default=None,
                    help="Newmark steps of the 64^3 implicit workload timed beside the headline "
                         "(default 500, the configured run, with the default workload, else 0)")
    ap.add_argument("--implicit-profile", action="store_true",
                    help="profiling aid: 2 Jacobi-PCG steps and 1 flexible-CG step with a fixed untrained "
                         "network on the 64^3 implicit workload, then exit (for an ncu launch list)")
    ap.add_argument("--config5-pml", default=None, metavar="NX,NY,NZ,NPML,NJ2,STEPS",
                    help="time only NewmarkBeta-Newton on the config-5 model with PML layers at this size "
                         "(e.g. 64,64,32,5,8,3) and print it as one JSON line")
    args = ap.parse_args()
    if args.implicit_profile:
        return implicit_profile()
    if args.config5_pml:
        nx, ny, nz, npml, nj2, st = (int(v) for v in args.config5_pml.split(","))
        print(json.dumps({"nonlinear_newton_j2_pml": nonlinear_newton_pml(steps=st, size=(nx, ny, nz), npml=npml,
                                                                          n_j2=nj2)}))
        return 0
    if args.implicit_steps is None:
        args.implicit_steps = 500 if args.workload == "config2" else 0
    ws, rank, local = dist_info()
    warm = max(3, args.warmup)
    if args.workload in ("config1", "config3"):
        args.precision = "fp64"
    nb = args.instances if args.precision == "mixed" else 1

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args, warm)

    from svl_gb300 import CentralDifference, StructuredCentralDifference
    from svl_gb300 import _capi as capi

    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
        pg = dist
    capi.check(capi.lib().svl_set_device(local))

    # ensembles shard across ranks: every rank advances its own 256 columns (weak scaling)
    insts = [build_workload(args.workload, seed=rank_seed(rank, args.workload, b)) for b in range(nb)]
    m, L, dt0, desc = insts[0]
    dt = min(x[2] for x in insts)
    nd = m.ndim
    nfree_total = sum(free_disp_dofs(x[0]) for x in insts)
    grid = m.grid_shape
    pml = has_pml(m)

    def make_handle():
        if args.precision == "mixed":
            h = StructuredCentralDifference(grid, (2.0, 2.0, 2.0), [(x[0], x[1]) for x in insts], dt)
            for b in range(nb):
                h.Initialize(b)
        else:
            h = CentralDifference(m, L, dt)
            h.Initialize()
        return h

    cd = make_handle()
    cd.run(1, warm)                                   # warm-up
    # schedule autotuner of the fused step (svl_cdx_tune): CTA count, tile
    # order, band block size and stream priority; the state is reset below
    sched = cd.tune(1 + warm, 12) if hasattr(cd, "tune") else None
    prof = cd.profile(1 + warm + 200, 20) if hasattr(cd, "profile") else None
    prof_full = None
    if sched is not None:
        # the step kernel alone with one CTA per SM (the tuned schedule may give
        # SMs to the band instead): the kernel's own roofline
        tuned = {k: sched[k] for k in cd.SCHEDULE_KEYS}
        cd.set_schedule(ctas=0)
        if cd.schedule()["ctas"] != tuned["ctas"]:
            prof_full = (cd.schedule()["ctas"], cd.profile(1 + warm + 240, 20))
        cd.set_schedule(**tuned)
    if args.precision == "mixed":
        for b in range(nb):
            cd.Initialize(b)
    else:
        cd.Initialize()
    if pg:
        pg.barrier()
    if hasattr(cd, "run_timed"):
        with ClockSampler(local) as clk:
            ms = cd.run_timed(1, args.steps)
    else:
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            cd.run(1, args.steps)
            ms = (time.perf_counter() - t0) * 1e3
    ms = max_over_ranks(pg, ms)
    launches = cd.launches() if hasattr(cd, "launches") else None
    clocks = clk.summary()
    ms_step = ms / args.steps
    value = job_value(ws, nfree_total, args.steps, ms)
    U_last = cd.get(0, 0) if args.precision == "mixed" else cd.GetDisplacements()
    finite = bool(np.isfinite(U_last).all())
    cd.close()
    udofs = np.concatenate([m.totaldof[n, :nd] for n in range(m.nnode)]) if pml else np.arange(m.ntotal)

    # FP64 plain path on instance 0, same steps: speed and the mixed result's error
    fp64 = None
    if args.precision == "mixed" and not args.no_fp64_compare:
        ms64, U64 = fp64_plain_run(m, L, dt, args.steps)
        err = float(np.linalg.norm(U_last[udofs] - U64[udofs]) / max(np.linalg.norm(U64[udofs]), 1e-300))
        v64 = free_disp_dofs(m) * args.steps / (ms64 * args.steps / 1e3)
        fp64 = {"value": ws * v64, "unit": "DOF-steps/s", "ms_per_step": ms64,
                "speedup_mixed_over_fp64": value / (ws * v64),
                "mixed_rel_l2_final_u_vs_fp64": err, "steps": args.steps, "instance": 0,
                "path": ("the explicit PML scheme in FP64 on the general PML-capable handle (svl_xnm_*)" if pml
                         else "FP64 central difference (svl_cd_*)")}

    peak, peak_kind = measured_peaks()
    npml_nodes = int(np.sum(m.node_ndof == 9)) if pml else 0
    npml_el = int(np.sum(m.elem_pml)) if pml else 0
    if args.precision == "mixed":
        grid_dofs = 3 * int(np.prod([g + 1 for g in grid]))
        half = (PML_BYTES_PER_NODE * 0.5 * npml_nodes + PML_BYTES_PER_ELEMENT * npml_el) * nb
        # profile slots: 0 k_cdx_step, 1 k_cdp_fu, 2 k_cdp_uu, 3 k_cdp_fs, 4 k_cdp_su
        kinds = {"k_cdx_step (tensor-core interior step, all instances)": ((0,), ALGO_BYTES_PER_DOF[3] * grid_dofs * nb),
                 "k_cdp_fu + k_cdp_uu (PML band, displacement rows)": ((1, 2), half),
                 "k_cdp_fs + k_cdp_su (PML band, stress rows)": ((3, 4), half)}
        pms = {k: float(sum(prof[i] for i in v[0])) / 20.0 for k, v in kinds.items()}
        kinds = {k: v for k, v in kinds.items() if pms[k] > 0}
        kname = max(kinds, key=lambda k: pms[k])
        algo_bytes = kinds[kname][1]
        k_ms = pms[kname]
        tot = sum(pms[k] for k in kinds)
        shares = {k: round(pms[k] / max(tot, 1e-12), 4) for k in kinds}
        per_kernel = {k: {"ms_per_step": pms[k], "algorithmic_bytes": v[1],
                          "achieved_gbs": v[1] / (pms[k] / 1e3) / 1e9} for k, v in kinds.items()}
        if pml:
            per_kernel["band kernels, ms per step"] = {n: float(prof[i] / 20.0) for i, n in
                                                       enumerate(["k_cdp_fu", "k_cdp_uu", "k_cdp_fs", "k_cdp_su"], 1)}
        full_grid = None
        if prof_full is not None:
            fms = float(prof_full[1][0]) / 20.0
            fab = kinds["k_cdx_step (tensor-core interior step, all instances)"][1]
            full_grid = {"ctas": prof_full[0], "ms_per_step": fms, "achieved": fab / (fms / 1e3) / 1e9,
                         "frac": fab / (fms / 1e3) / 1e9 / measured_peaks()[0],
                         "note": "k_cdx_step with one CTA per SM, profiled alone; the tuned schedule gives SMs "
                                 "to the PML band's kernels, which then overlap the step"}
    else:
        algo_bytes = ALGO_BYTES_PER_DOF[nd] * nfree_total
        if args.workload == "config3":
            algo_bytes += J2_STATE_BYTES_PER_ELEMENT * m.nelem
        k_ms = ms_step
        kname = "one FP64 step (all its kernels)"
        shares, per_kernel, full_grid = None, None, None
        if prof is not None:
            names = ["k_element", "k_node", "k_residual", "k_free", "k_update"]
            shares = {names[i]: round(float(prof[i] / max(prof.sum(), 1e-12)), 4) for i in range(5) if prof[i] > 0}
    achieved = algo_bytes / (k_ms / 1e3) / 1e9
    traffic, traffic_src = None, None
    if args.precision == "mixed" and pml and kname.startswith("k_cdx_step") and args.workload == "config2":
        # DRAM bytes of one k_cdx_step launch on this workload (4 instances), one
        # ncu capture (dram__bytes_read.sum + dram__bytes_write.sum), scaled by
        # the instance count
        traffic = CDX_STEP_DRAM_BYTES_4INST * nb / 4.0
        traffic_src = ("ncu, 4-instance capture of the step kernel over all tiles in one launch (before the step "
                       "was split into far and near launches): 298 MB read + 59 MB write per step")

    e2e = None
    if not args.no_e2e:
        # the whole run through the public API: handle creation from host arrays,
        # then every step with every instance's full total-dof vector copied to a
        # page-locked host buffer (allocated once, outside the timed region)
        from svl_gb300 import pinned_empty
        ne2e = E2E_STEPS[args.workload]
        chunk = 20 if args.precision == "mixed" else (ne2e if args.workload == "config1" else 200)
        hbuf = pinned_empty((chunk, nb, m.ntotal) if args.precision == "mixed" else (chunk, m.ntotal))
        with ClockSampler(local) as clk2:
            t0 = time.perf_counter()
            cd2 = make_handle()                             # host arrays -> device
            t1 = time.perf_counter()
            call_ms = []
            for s0 in range(0, ne2e, chunk):
                n = min(chunk, ne2e - s0)
                tc = time.perf_counter()
                if args.precision == "mixed" or not pml:
                    cd2.run(1 + s0, n, out=hbuf[:n])
                else:                                       # the FP64 PML handle copies its history itself
                    hbuf[:n] = cd2.run(1 + s0, n, history=True)
                call_ms.append((time.perf_counter() - tc) * 1e3 / n)
            t2 = time.perf_counter()
        cd2.close()
        md_bytes = nb * (m.coords.nbytes + m.totaldof.nbytes + m.freedof.nbytes + m.conn.nbytes +
                         m.elem_mat.nbytes + m.mat_param.nbytes + m.mat_type.nbytes +
                         (m.pml_param.nbytes if pml else 0) +
                         sum(x.nbytes for x in L.series) + 20 * len(L.force_dof) + 16 * len(L.sm_dof))
        e2e = {"value": ws * nfree_total * ne2e / (t2 - t0), "unit": "DOF-steps/s",
               "h2d_bytes_per_step": int(md_bytes / ne2e), "d2h_bytes_per_step": int(nb * m.ntotal * 8),
               "steps": ne2e, "create_seconds": t1 - t0, "run_seconds": t2 - t1,
               "run_only_value": ws * nfree_total * ne2e / (t2 - t1),
               "chunk_steps": chunk,
               "call_ms_per_step_p10_p50_p90": [float(x) for x in np.percentile(call_ms, [10, 50, 90])],
               "calls_slower_than_1.5x_median": int(np.sum(np.array(call_ms[1:]) > 1.5 * np.median(call_ms))),
               "calls": len(call_ms),
               "first_call_ms_per_step": float(call_ms[0]),
               "clocks": clk2.summary(),
               "includes": "handle creation from host arrays (model, loads) + the whole run with every instance's "
                           "full total-dof vector (displacements and PML stress dofs) copied to page-locked host "
                           "memory every step"}
        del hbuf

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline([(x[0], x[1]) for x in insts], dt, steps_cap=10)
    implicit = (implicit_pcg(args.implicit_steps, warm=min(100, max(1, args.implicit_steps // 5)))
                if (rank == 0 and args.implicit_steps > 1) else None)
    newton = nonlinear_newton() if (rank == 0 and args.implicit_steps > 0 and args.workload == "config2") else None
    ensemble = None
    if rank == 0 and args.precision == "mixed" and args.workload == "config2" and not args.no_ensemble:
        ensemble = uneven_ensemble()
    newton_pml = None
    if rank == 0 and args.implicit_steps > 0 and args.workload == "config2":
        # the config-5 model with its PML half-space at 64x64x32 (3 steps); a
        # failure here is reported in the line instead of ending the run
        try:
            newton_pml = nonlinear_newton_pml()
        except Exception as exc:  # noqa: BLE001
            newton_pml = {"error": str(exc)[:300]}

    if rank == 0:
        ws_mb = (nb * m.ntotal * 8 * 2 + nb * npml_el * 72 * 4 * 2) // 2 ** 20
        line = {
            "metric": "DOF-steps/s", "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "tf32x2+f32x2" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded)",
            "config": workload_config(desc, insts, dt, E2E_STEPS[args.workload]),
            "precision": ("mixed: tensor-core element forces in the elastic interior (displacements split into "
                          "TF32 hi + lo, the element stiffness patterns exact in TF32, FP32 accumulation), FP32 "
                          "PML-band kernels, state as compensated FP32 pairs (~48 bits)"
                          if args.precision == "mixed" else "fp64 plain"),
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "l2": "no flush; working set ~%d MB > 129 MB L2" % ws_mb,
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind + " (HBM copy)",
                         "traffic": traffic, "traffic_unit": "bytes per step" if traffic else None,
                         "traffic_source": traffic_src,
                         "algorithmic_bytes_per_step": algo_bytes, "kernel_ms_per_step": k_ms,
                         "kernel_share": shares, "per_kernel": per_kernel, "kernel_one_cta_per_sm": full_grid},
            "fp64_plain": fp64, "implicit_pcg_time_to_1e-8": implicit, "nonlinear_newton_j2": newton,
            "nonlinear_newton_j2_pml": newton_pml,
            "cpu_baseline": cb, "e2e": e2e, "gpu_launches": int(launches) if launches is not None else None,
            "schedule": sched, "uneven_ensemble": ensemble,
            "clocks": clocks, "finite": finite,
        }
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
