#!/usr/bin/env python3
"""Benchmark of the explicit central-difference hot path (DOF-steps/s).

A "step" is one time step of the whole batch: element forces, the ordered
node gather, the diagonal solve and the state update.  Default workload: the
3D configuration (lin3DHexa8 128 x 128 x 64, h = 2 m, log-normal Vs field,
double-couple body force), as a batch of 4 seeded realisations advanced by
the mixed-precision path (tensor-core TF32 hi/lo element forces, compensated
FP32-pair state update); the FP64
plain path is timed on one realisation beside it, and the mixed result's
error against it is reported.  The PML layers of that configuration are not
built yet; the box has fixed/roller faces instead (stated in the config).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision mixed|fp64] [--instances B] [--workload config2|config1|config3]

value   : free DOF x instances x steps / device time of the K steps (CUDA
          events on the library's stream, inputs resident in HBM, working
          set > L2: 4 instances hold ~300 MB of state).
e2e     : the same metric through the C ABI with host buffers: model arrays
          copied in by the create call and every instance's full displacement
          field copied back to a host buffer after every step.
roofline: algorithmic bytes of one step (37 B per free DOF for H8, 40 for
          Q4) over the measured step time, against MEASURED_PEAKS.json.
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

# DRAM bytes (read + write) per free DOF of one k_cdx_step launch on the
# lin3DHexa8 128x128x64 workload, from an ncu capture (dram__bytes_read.sum,
# dram__bytes_write.sum) of the 2-instance case: 148.05 MB read + 20.07 MB
# written per launch over 6 324 096 free DOF.  Part of the state written by one step is
# still in L2 when the next step reads it, so this is below the 37 B/DOF of
# algorithmic traffic.
DRAM_BYTES_PER_DOF_STEP_MIXED_H8 = 26.585
sys.path.insert(0, str(ROOT))

ALGO_BYTES_PER_DOF = {2: 40.0, 3: 37.0}
# steps of the end-to-end run per workload (the configured run lengths)
E2E_STEPS = {"config1": 2000, "config2": 4000, "config3": 4000}
# plane-strain J2 state read + written per element and step: 2 x 9 doubles x 4 Gauss points
J2_STATE_BYTES_PER_ELEMENT = 576.0


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def build_workload(name, seed=0):
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
        m, L, dt = workloads.config2(seed=seed)
        desc = ("lin3DHexa8 128x128x64 box (h=2 m, log-normal Vs, COV 0.2, corr 20 m), CD; "
                "PML layers not built (fixed bottom, roller sides)")
    else:
        raise SystemExit("unknown workload %s" % name)
    return m, L, dt, desc


def cpu_baseline(m, L, dt, steps_cap, budget_s=20.0):
    """Oracle (CPU port of the reference path), fast mode, all host threads."""
    from oracle import oracle as O
    nthreads = O.num_threads()
    t = {}
    n = max(1, steps_cap)
    O.cd_run(m, L, dt, 1, mode=1, history=False, timing=t)   # warm-up / sizing step
    per = max(t["seconds"], 1e-6)
    n = int(max(1, min(steps_cap, budget_s / per)))
    O.cd_run(m, L, dt, n, mode=1, history=False, timing=t)
    val = m.nfree * n / t["seconds"]
    out = {"value": val, "unit": "DOF-steps/s", "cores": nthreads, "kind": "port",
           "sample": "%d time steps of the same model on the CPU oracle (OpenMP element loop, ordered scatter)" % n}
    # the reference's own structure, single-threaded per rank: J, J^-1 and B
    # recomputed per Gauss point per call (one step)
    try:
        t1 = {}
        O.cd_run(m, L, dt, 1, mode=0, history=False, timing=t1)
        out["single_thread_reference_faithful"] = {
            "value": m.nfree / t1["seconds"], "unit": "DOF-steps/s", "cores": 1,
            "sample": "1 time step of the same model, the oracle's reference-faithful mode"}
    except Exception as exc:  # noqa: BLE001
        out["single_thread_reference_faithful"] = {"error": str(exc)[:200]}
    return out


def implicit_pcg(steps, warm=20, tol=1e-8):
    """Newmark (average acceleration) + Linear on the 64^3 layered H8 model:
    mean wall time per step of the effective-stiffness solve to a true
    relative residual of `tol`, Jacobi-PCG against the learned preconditioner
    (flexible CG, Jacobi fallback), both FP64 matrix-free.  The learned handle
    runs the same `warm` Jacobi steps first, then trains (timed separately)."""
    from svl_gb300 import NewmarkBeta, workloads
    m, L, dt = workloads.config4(nt=warm + steps + 2)
    jac = NewmarkBeta(m, L, dt, pcg_tol=tol)
    lrn = NewmarkBeta(m, L, dt, pcg_tol=tol)
    for h in (jac, lrn):
        h.Initialize()
        h.run(1, warm)
    t0 = time.perf_counter()
    loss = lrn.train_preconditioner(1 + warm, **NN_TRAIN)
    train_s = time.perf_counter() - t0
    out = {}
    for name, h in (("jacobi", jac), ("learned", lrn)):
        it0 = h.stats()[0]
        ms = h.run_timed(1 + warm, steps)
        it1, _, res = h.stats()
        out[name] = {"ms_per_step": ms / steps, "pcg_iters_per_step": (it1 - it0) / steps, "rel_residual_last": res,
                     "gpu_launches": int(h.launches())}
    solves, fallbacks, jref = lrn.precond_stats()
    Uj, Ul = jac.GetDisplacements(), lrn.GetDisplacements()
    jac.close()
    lrn.close()
    out["learned"].update({"train_seconds": train_s, "train_loss": loss, "fallbacks": fallbacks, "solves": solves,
                           "train": dict(NN_TRAIN)})
    return {"workload": "lin3DHexa8 64x64x64 (h=1 m), layered G (100x contrast) x 10% log-normal, "
                        "Newmark beta=1/4 gamma=1/2, dt=10x explicit limit, fixed bottom, roller sides",
            "free_dof": m.nfree, "steps": steps, "tol": tol, "residual": "true |b - K_eff x| / |b|, FP64",
            "jacobi": out["jacobi"], "learned": out["learned"],
            "speedup_learned_over_jacobi": out["jacobi"]["ms_per_step"] / out["learned"]["ms_per_step"],
            "iteration_ratio": out["jacobi"]["pcg_iters_per_step"] / max(out["learned"]["pcg_iters_per_step"], 1e-9),
            "rel_l2_final_u_learned_vs_jacobi": float(np.linalg.norm(Ul - Uj) / max(np.linalg.norm(Uj), 1e-300))}


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


NN_TRAIN = {"solve_steps": 0, "n_synthetic": 300, "iters": 1500, "batch": 8, "lr": 2e-3, "seed": 1, "max_sweeps": 5}


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--instances", type=int, default=4)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--implicit-steps", type=int, default=None,
                    help="Newmark steps of the 64^3 implicit workload timed beside the headline "
                         "(default 10 with the default workload, else 0)")
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
        args.implicit_steps = 10 if args.workload == "config2" else 0
    ws, rank, local = dist_info()
    warm = max(3, args.warmup)
    if args.workload in ("config1", "config3"):
        args.precision = "fp64"
    nb = args.instances if args.precision == "mixed" else 1

    if args.impl == "reference":
        if rank != 0:
            return 0
        m, L, dt, desc = build_workload(args.workload)
        cb = cpu_baseline(m, L, dt, steps_cap=min(args.steps, 20))
        line = {"metric": "DOF-steps/s", "value": cb["value"], "unit": "DOF-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": warm, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
                "config": {"workload": desc, "free_dof": m.nfree, "elements": m.nelem},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "DOF-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

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
    nfree_total = sum(x[0].nfree for x in insts)
    grid = m.grid_shape

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
    prof = None
    if args.precision == "fp64":
        prof = cd.profile(1 + warm, 20)
    if args.precision == "mixed":
        for b in range(nb):
            cd.Initialize(b)
    else:
        cd.Initialize()
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        ms = cd.run_timed(1, args.steps)
    ms = max_over_ranks(pg, ms)
    launches = cd.launches()
    clocks = clk.summary()
    ms_step = ms / args.steps
    value = job_value(ws, nfree_total, args.steps, ms)
    U_last = cd.get(0, 0) if args.precision == "mixed" else cd.GetDisplacements()
    finite = bool(np.isfinite(U_last).all())
    cd.close()

    # FP64 plain path on instance 0, same steps: speed and the mixed result's error
    fp64 = None
    if args.precision == "mixed" and not args.no_fp64_compare:
        ref = CentralDifference(m, L, dt)
        ref.Initialize()
        ms64 = ref.run_timed(1, args.steps)
        U64 = ref.GetDisplacements()
        ref.close()
        err = float(np.linalg.norm(U_last - U64) / max(np.linalg.norm(U64), 1e-300))
        v64 = m.nfree * args.steps / (ms64 / 1e3)
        fp64 = {"value": ws * v64, "unit": "DOF-steps/s", "ms_per_step": ms64 / args.steps,
                "speedup_mixed_over_fp64": value / (ws * v64),
                "mixed_rel_l2_final_u_vs_fp64": err, "steps": args.steps, "instance": 0}

    peak, peak_kind = measured_peaks()
    algo_bytes = ALGO_BYTES_PER_DOF[nd] * nfree_total
    if args.workload == "config3":
        algo_bytes += J2_STATE_BYTES_PER_ELEMENT * m.nelem
    achieved = algo_bytes / (ms_step / 1e3) / 1e9
    if args.precision == "fp64":
        kernel_names = ["k_element", "k_node", "k_residual", "k_free", "k_update"]
        shares = {kernel_names[i]: round(float(prof[i] / max(prof.sum(), 1e-12)), 4) for i in range(5) if prof[i] > 0}
        kname = "one FP64 CD step (all its kernels)"
    else:
        shares = None
        kname = "k_cdx_step (fused mixed-precision step, all instances) + k_cdx_loads"

    e2e = None
    if not args.no_e2e:
        # the whole run through the public API: handle creation from host arrays,
        # then every step with every instance's full displacement field copied to a
        # page-locked host buffer (allocated once, outside the timed region)
        # (the configured run length: 4000 steps for the 3D and ensemble
        # workloads, 2000 for the 2D box; the history goes through one reused
        # page-locked chunk, as a recorder writing it out would)
        from svl_gb300 import pinned_empty
        ne2e = E2E_STEPS[args.workload]
        chunk = 100 if args.precision == "mixed" else (ne2e if args.workload == "config1" else 200)
        hbuf = pinned_empty((chunk, nb, m.ntotal) if args.precision == "mixed" else (chunk, m.ntotal))
        t0 = time.perf_counter()
        cd2 = make_handle()                             # host arrays -> device
        t1 = time.perf_counter()
        for s0 in range(0, ne2e, chunk):
            n = min(chunk, ne2e - s0)
            cd2.run(1 + s0, n, out=hbuf[:n])
        t2 = time.perf_counter()
        cd2.close()
        md_bytes = nb * (m.coords.nbytes + m.totaldof.nbytes + m.freedof.nbytes + m.conn.nbytes +
                         m.elem_mat.nbytes + m.mat_param.nbytes + m.mat_type.nbytes +
                         sum(x.nbytes for x in L.series) + 20 * len(L.force_dof) + 16 * len(L.sm_dof))
        e2e = {"value": ws * nfree_total * ne2e / (t2 - t0), "unit": "DOF-steps/s",
               "h2d_bytes_per_step": int(md_bytes / ne2e), "d2h_bytes_per_step": int(nb * m.ntotal * 8),
               "steps": ne2e, "create_seconds": t1 - t0, "run_seconds": t2 - t1,
               "run_only_value": ws * nfree_total * ne2e / (t2 - t1),
               "chunk_steps": chunk,
               "includes": "handle creation from host arrays (model, loads) + the whole run with every instance's "
                           "full displacement field copied to page-locked host memory every step"}
        del hbuf

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(m, L, dt, steps_cap=10)
    implicit = implicit_pcg(args.implicit_steps) if (rank == 0 and args.implicit_steps > 0) else None
    newton = nonlinear_newton() if (rank == 0 and args.implicit_steps > 0 and args.workload == "config2") else None
    newton_pml = None
    if rank == 0 and args.implicit_steps > 0 and args.workload == "config2":
        # the config-5 model with its PML half-space at 64x64x32 (3 steps); a
        # failure here is reported in the line instead of ending the run
        try:
            newton_pml = nonlinear_newton_pml()
        except Exception as exc:  # noqa: BLE001
            newton_pml = {"error": str(exc)[:300]}

    if rank == 0:
        ws_mb = (nb * m.ntotal * 8 * (2 if args.precision == "mixed" else 7) + nb * m.ntotal * 4
                 + (m.nelem * 24 * 8 if args.precision == "fp64" else nb * m.nelem * 8)) // 2 ** 20
        line = {
            "metric": "DOF-steps/s", "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "tf32x3+f32x2" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": desc, "instances": nb, "free_dof_per_instance": m.nfree,
                       "elements_per_instance": m.nelem, "dt": dt,
                       "precision": ("mixed: TF32 hi/lo tensor-core element forces, FP32 accumulate, "
                                     "compensated FP32-pair displacement state (~48 bits)"
                                     if args.precision == "mixed" else "fp64 plain"),
                       "parallelism": "replicas" if ws > 1 else "single GPU",
                       "l2": "no flush; working set ~%d MB > 129 MB L2" % ws_mb},
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (DRAM_BYTES_PER_DOF_STEP_MIXED_H8 * nfree_total
                                     if args.precision == "mixed" and args.workload == "config2" else None),
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of k_cdx_step, "
                                            "2-instance case (6.3 M DOF), scaled per free DOF to this launch"
                                            if args.precision == "mixed" and args.workload == "config2" else None),
                         "algorithmic_bytes_per_step": algo_bytes, "kernel_share": shares},
            "fp64_plain": fp64, "implicit_pcg_time_to_1e-8": implicit, "nonlinear_newton_j2": newton,
            "nonlinear_newton_j2_pml": newton_pml,
            "cpu_baseline": cb, "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks,
            "finite": finite,
        }
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
