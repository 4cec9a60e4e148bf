"""Python mirror of the reference's Integrator interface over the C ABI.

`CentralDifference` stands in for RP/10-Integrators/02-CentralDifference
(CentralDifference.hpp) driven by the Linear algorithm with the diagonal
EigenSolver solve: Initialize / ComputeNewStep(k) -> stop flag /
GetDisplacements / GetVelocities / GetAccelerations keep the reference's
names and meaning; `run` advances many steps in one call (device-resident).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as capi
from ._capi import check, lib, ptr
from .model import Loads, Model


class CentralDifference:
    """A model with PML layers is served by the PML-capable handle with the
    library's explicit PML scheme (svl_xnm_*, integrator
    SVL_XNM_CENTRAL_DIFFERENCE); the object returned is then an
    ExtendedNewmarkBeta instance with the same step methods.  A model whose
    central-difference system K = M/dt^2 + C/2dt is not diagonal (consistent
    mass, or stiffness-proportional Rayleigh damping) is served by
    CentralDifferenceSolve (a PCG solve of K every step)."""

    def __new__(cls, model: Model, *args, **kw):
        if cls is CentralDifference and getattr(model, "elem_pml", None) is not None and np.any(model.elem_pml):
            return _central_difference_pml(model, *args, **kw)
        if cls is CentralDifference and _cd_nondiagonal(model):
            return CentralDifferenceSolve(model, *args, **kw)
        return super().__new__(cls)

    def __init__(self, model: Model, loads: Loads | None, dt: float, ftol: float = 1e-12,
                 mtol: float = 1e-12, check_every: int = 0):
        self.model = model
        self.dt = float(dt)
        self._md = model.desc()
        self.loads = loads or Loads()
        self._ld = self.loads.desc()
        opts = capi.CdOpts(dt=self.dt, ftol=ftol, mtol=mtol, precision=capi.SVL_PREC_FP64,
                           check_every=check_every)
        h = C.c_void_p()
        check(lib().svl_cd_create(C.byref(self._md), C.byref(self._ld), C.byref(opts), C.byref(h)))
        self._h = h
        self.ntotal = model.ntotal

    # -- reference-style interface --------------------------------------
    def Initialize(self, U0=None, V0=None, A0=None):
        arrs = [None if a is None else capi.as_f64(a) for a in (U0, V0, A0)]
        check(lib().svl_cd_set_initial(self._h, *(ptr(a, C.c_double) for a in arrs)))

    def ComputeNewStep(self, k: int) -> bool:
        """One step k; returns True on failure (the reference's `stop`)."""
        return lib().svl_cd_run(self._h, int(k), 1, ptr(None, C.c_double)) != capi.SVL_OK

    def GetDisplacements(self) -> np.ndarray:
        return self._get(0)

    def GetVelocities(self) -> np.ndarray:
        return self._get(1)

    def GetAccelerations(self) -> np.ndarray:
        return self._get(2)

    def ComputeProgressiveForce(self, k: int) -> np.ndarray:
        """Fext(k) + Fbar (ComputeProgressiveForce of the reference's
        integrators, e.g. CentralDifference.cpp:174-186): the stage force Fbar
        of earlier stages is zero in a single-stage run."""
        return self.loads.external_force(self.ntotal, int(k))

    def ComputeReactionForce(self, k: int) -> np.ndarray:
        """Reaction forces after step k (CentralDifference.cpp:156-171): total-dof
        vector, zeros off the fixed nodes."""
        R = np.zeros(self.ntotal)
        check(lib().svl_cd_reaction(self._h, int(k), ptr(R, C.c_double)))
        return R

    def element_response(self, response: str, elems) -> np.ndarray:
        """ELEMENT recorder values after the last step (Recorder.cpp:272-323)
        of the element positions `elems`: STRAIN / STRESS / STRAINRATE
        [n, ngp, 3|6], INTERNALFORCE [n, NC]."""
        return _element_response(lib().svl_cd_element_response, self._h, self.model, response, elems)

    # -- batch interface -------------------------------------------------
    def run(self, k_first: int, nsteps: int, history: bool = False, out=None):
        """Steps k_first .. k_first+nsteps-1; with history=True (or a
        C-contiguous float64 `out` of shape [nsteps, ntotal], e.g. from
        svl_gb300.pinned_empty) returns the displacement after every step."""
        hist = out if out is not None else (np.zeros((nsteps, self.ntotal)) if history else None)
        if hist is not None:
            assert hist.shape == (nsteps, self.ntotal) and hist.dtype == np.float64 and hist.flags["C_CONTIGUOUS"]
        check(lib().svl_cd_run(self._h, int(k_first), int(nsteps), ptr(hist, C.c_double)))
        return hist

    def run_timed(self, k_first: int, nsteps: int) -> float:
        """Device time (ms) of nsteps, CUDA events on the handle's stream."""
        ms = C.c_float()
        check(lib().svl_cd_run_timed(self._h, int(k_first), int(nsteps), C.byref(ms)))
        return float(ms.value)

    def profile(self, k_first: int, nsteps: int) -> np.ndarray:
        """Per-kernel-kind device time (ms) summed over nsteps."""
        out = np.zeros(5)
        check(lib().svl_cd_profile(self._h, int(k_first), int(nsteps), ptr(out, C.c_double)))
        return out

    def launches(self) -> int:
        n = C.c_int64()
        check(lib().svl_cd_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def sync(self):
        check(lib().svl_cd_sync(self._h))

    def _get(self, which):
        out = np.zeros(self.ntotal)
        check(lib().svl_cd_get(self._h, which, ptr(out, C.c_double)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().svl_cd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StructuredCentralDifference:
    """Mixed-precision batched central difference for `ninst` instances of one
    uniform lin3DHexa8 grid (svl_cdx_*): tensor-core element forces (TF32
    hi/lo, FP32 accumulation), displacement state as a compensated FP32 pair
    (hi + lo, ~48 significant bits; not FP64).  Same step as
    CentralDifference; `instances` is a list of (Model, Loads) built on the
    grid given by `ne`, `h`, `origin`."""

    def __init__(self, ne, h, instances, dt: float, origin=(0.0, 0.0, 0.0), mtol: float = 1e-12):
        self.dt = float(dt)
        self.ninst = len(instances)
        spec = capi.GridSpec()
        spec.ndim = 3
        for i in range(3):
            spec.ne[i] = int(ne[i])
            spec.h[i] = float(h[i])
            spec.origin[i] = float(origin[i])
        self._spec = spec
        md = (capi.ModelDesc * self.ninst)()
        ld = (capi.LoadDesc * self.ninst)()
        self._keep = []
        for i, (m, L) in enumerate(instances):
            md[i] = m.desc()
            self._keep.append(m)
            L = L or Loads()
            ld[i] = L.desc()
            self._keep.append(L)
        self._md, self._ld = md, ld
        opts = capi.CdOpts(dt=self.dt, ftol=0.0, mtol=mtol, precision=capi.SVL_PREC_MIXED, check_every=0)
        hnd = C.c_void_p()
        check(lib().svl_cdx_create(C.byref(spec), self.ninst, md, ld, C.byref(opts), C.byref(hnd)))
        self._h = hnd
        self.ntotal = instances[0][0].ntotal

    def Initialize(self, inst: int = 0, U0=None, V0=None, A0=None):
        arrs = [None if a is None else capi.as_f64(a) for a in (U0, V0, A0)]
        check(lib().svl_cdx_set_initial(self._h, int(inst), *(ptr(a, C.c_double) for a in arrs)))

    def run(self, k_first: int, nsteps: int, history: bool = False, out=None):
        """Steps of every instance; history (or `out`, float64 [nsteps, ninst,
        ntotal], e.g. from svl_gb300.pinned_empty) receives all displacements."""
        hist = out if out is not None else (np.zeros((nsteps, self.ninst, self.ntotal)) if history else None)
        if hist is not None:
            assert hist.shape == (nsteps, self.ninst, self.ntotal) and hist.dtype == np.float64 and hist.flags["C_CONTIGUOUS"]
        check(lib().svl_cdx_run(self._h, int(k_first), int(nsteps), ptr(hist, C.c_double)))
        return hist

    def run_timed(self, k_first: int, nsteps: int) -> float:
        ms = C.c_float()
        check(lib().svl_cdx_run_timed(self._h, int(k_first), int(nsteps), C.byref(ms)))
        return float(ms.value)

    def get(self, inst: int, which: int = 0) -> np.ndarray:
        out = np.zeros(self.ntotal)
        check(lib().svl_cdx_get(self._h, int(inst), int(which), ptr(out, C.c_double)))
        return out

    def launches(self) -> int:
        n = C.c_int64()
        check(lib().svl_cdx_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def profile(self, k_first: int, nsteps: int) -> np.ndarray:
        """Device time (ms) per kernel over nsteps: [tensor-core step, PML
        band k_cdp_fu, k_cdp_uu, k_cdp_fs, k_cdp_su] (band zeros without PML)."""
        out = np.zeros(5)
        check(lib().svl_cdx_profile(self._h, int(k_first), int(nsteps), ptr(out, C.c_double)))
        return out

    SCHEDULE_KEYS = ("ctas", "tile_order", "band_threads", "band_stream_high_priority")

    def schedule(self) -> dict:
        ch = np.zeros(4, np.int32)
        check(lib().svl_cdx_get_schedule(self._h, ptr(ch, C.c_int32)))
        return dict(zip(self.SCHEDULE_KEYS, (int(x) for x in ch)))

    def set_schedule(self, **kw):
        cur = self.schedule()
        cur.update(kw)
        ch = np.array([cur[k] for k in self.SCHEDULE_KEYS], np.int32)
        check(lib().svl_cdx_set_schedule(self._h, ptr(ch, C.c_int32)))

    def tune(self, k_first: int, nsteps: int = 5) -> dict:
        """Times a small grid of schedules and keeps the fastest (svl_cdx_tune);
        the state advances: Initialize again afterwards."""
        ch = np.zeros(4, np.int32)
        ms = C.c_float()
        check(lib().svl_cdx_tune(self._h, int(k_first), int(nsteps), ptr(ch, C.c_int32), C.byref(ms)))
        out = dict(zip(self.SCHEDULE_KEYS, (int(x) for x in ch)))
        out["ms_per_step"] = float(ms.value)
        return out

    def set_ctas(self, ctas: int) -> int:
        """CTAs of the persistent step kernel (0 = one per SM); returns the
        grid size in effect."""
        check(lib().svl_cdx_set_ctas(self._h, int(ctas)))
        n = C.c_int32()
        check(lib().svl_cdx_get_ctas(self._h, C.byref(n)))
        return int(n.value)

    def close(self):
        if getattr(self, "_h", None):
            lib().svl_cdx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ExtendedNewmarkBeta:
    """ExtendedNewmarkBeta (RP/10-Integrators/03-Newmark/ExtendedNewmarkBeta.cpp)
    for meshes with PML2DQuad4 / PML3DHexa8 layers and elastic or J2 solid
    elements (svl_xnm_*): the PML history term G (Ubar + dt U + dt^2/6 V),
    Rayleigh and PML damping, support motion of step k, and a matrix-free
    MINRES solve of the symmetric indefinite effective matrix to the relative
    true residual `tol` in the |diag|^-1 norm (at most `solver_maxit`
    iterations).  algorithm "linear" (Linear.cpp) or "newton"
    (NewtonRaphson.cpp with `maxit` iterations, tolerance `cnvgtol`, test
    `cnvgtest`).  GetPMLHistoryVector returns Ubar."""

    def __init__(self, model: Model, loads: Loads | None, dt: float, tol: float = 1e-10,
                 solver_maxit: int = 100000, ftol: float = 1e-12, mtol: float = 1e-12, algorithm: str = "linear",
                 maxit: int = 50, cnvgtol: float = 1e-6, cnvgtest: int = 4, integrator: str = "extendednewmark",
                 single_inner: bool = True):
        """integrator "extendednewmark" (ExtendedNewmarkBeta.cpp), "newmark"
        (NewmarkBeta.cpp on the same elements: the PML history matrix is not
        used; NewmarkBeta(model with PML layers, ...) builds this) or
        "centraldifference" (the library's explicit scheme for PML models:
        stress dofs at the half steps, lumped N N blocks; tol and solver_maxit
        are not used; CentralDifference(model with PML layers, ...) builds
        this).
        single_inner: the inner MINRES iterations apply the element operators
        in single precision, the restarts' true residual and the stopping test
        stay in double (iterative refinement)."""
        self.model = model
        self.dt = float(dt)
        self._md = model.desc()
        self.loads = loads or Loads()
        self._ld = self.loads.desc()
        algo = {"linear": capi.SVL_ALGO_LINEAR, "newton": capi.SVL_ALGO_NEWTON}[algorithm.lower()]
        integ = {"extendednewmark": capi.SVL_XNM_EXTENDED_NEWMARK, "newmark": capi.SVL_XNM_NEWMARK,
                 "centraldifference": capi.SVL_XNM_CENTRAL_DIFFERENCE}[integrator.lower()]
        opts = capi.XnmOpts(dt=self.dt, ftol=ftol, mtol=mtol, tol=float(tol), maxit=int(solver_maxit),
                            algorithm=algo, newton_maxit=int(maxit), cnvgtest=int(cnvgtest), cnvgtol=float(cnvgtol),
                            integrator=integ, single_inner=1 if single_inner else 0)
        h = C.c_void_p()
        check(lib().svl_xnm_create(C.byref(self._md), C.byref(self._ld), C.byref(opts), C.byref(h)))
        self._h = h
        self.ntotal = model.ntotal

    def Initialize(self, U0=None, V0=None, A0=None, Ubar0=None):
        arrs = [None if a is None else capi.as_f64(a) for a in (U0, V0, A0, Ubar0)]
        check(lib().svl_xnm_set_initial(self._h, *(ptr(a, C.c_double) for a in arrs)))

    def ComputeNewStep(self, k: int) -> bool:
        """One step k; returns True on failure (the reference's `stop`)."""
        return lib().svl_xnm_run(self._h, int(k), 1, ptr(None, C.c_double)) != capi.SVL_OK

    def _get(self, which):
        out = np.zeros(self.ntotal)
        check(lib().svl_xnm_get(self._h, int(which), ptr(out, C.c_double)))
        return out

    def GetDisplacements(self) -> np.ndarray:
        return self._get(0)

    def GetVelocities(self) -> np.ndarray:
        return self._get(1)

    def GetAccelerations(self) -> np.ndarray:
        return self._get(2)

    def ComputeProgressiveForce(self, k: int) -> np.ndarray:
        """Fext(k) + Fbar (ComputeProgressiveForce of the reference's
        integrators, e.g. CentralDifference.cpp:174-186): the stage force Fbar
        of earlier stages is zero in a single-stage run."""
        return self.loads.external_force(self.ntotal, int(k))

    def GetPMLHistoryVector(self) -> np.ndarray:
        return self._get(3)

    def ComputeReactionForce(self, k: int) -> np.ndarray:
        """Reactions after step k on the fixed nodes' dofs (ExtendedNewmarkBeta /
        NewmarkBeta::ComputeReactionForce as DynamicAnalysis::UpdateDomain
        applies it); PML elements add K u + C v + M a over all their dofs."""
        out = np.zeros(self.ntotal)
        check(lib().svl_xnm_reaction(self._h, int(k), ptr(out, C.c_double)))
        return out

    def run(self, k_first: int, nsteps: int, history: bool = False):
        hist = np.zeros((nsteps, self.ntotal)) if history else None
        check(lib().svl_xnm_run(self._h, int(k_first), int(nsteps), ptr(hist, C.c_double)))
        return hist

    def stats(self):
        """(MINRES iterations in total, in the last solve, last relative true residual)."""
        a, b, r = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().svl_xnm_stats(self._h, C.byref(a), C.byref(b), C.byref(r)))
        return a.value, b.value, r.value

    def newton_stats(self):
        """(Newton iterations over all steps, of the last step, last convergence-test value)."""
        a, b, r = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().svl_xnm_newton_stats(self._h, C.byref(a), C.byref(b), C.byref(r)))
        return a.value, b.value, r.value

    def close(self):
        if getattr(self, "_h", None):
            lib().svl_xnm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NewmarkBeta:
    """Implicit Newmark, average acceleration (beta = 1/4, gamma = 1/2), with
    the Linear algorithm: one effective-stiffness solve per step by a
    matrix-free Jacobi-preconditioned conjugate gradient in FP64 that stops
    on the true relative residual (svl_nm_*).  Mirrors NewmarkBeta
    (RP/10-Integrators/03-Newmark/NewmarkBeta.cpp) driven by Linear
    (RP/09-Algorithms/01-Linear/Linear.cpp) over an iterative LinearSystem
    (RP/11-Solvers/02-Iterative/PetscSolver.cc, KSPCG, rtol `pcg_tol`).

    A model with PML layers (symmetric indefinite effective matrix) is served
    by the PML-capable handle in NewmarkBeta mode (svl_xnm_*, MINRES to
    `pcg_tol`); the object returned is then an ExtendedNewmarkBeta instance
    with the same step methods."""

    _integrator = capi.SVL_NM_NEWMARK

    def __new__(cls, model: Model, *args, **kw):
        if cls is NewmarkBeta and getattr(model, "elem_pml", None) is not None and np.any(model.elem_pml):
            return _newmark_pml(model, *args, **kw)
        return super().__new__(cls)

    def __init__(self, model: Model, loads: Loads | None, dt: float, pcg_tol: float = 1e-8,
                 pcg_maxit: int = 20000, ftol: float = 1e-12, mtol: float = 1e-12, precond: int = 0,
                 algorithm: str = "linear", maxit: int = 50, cnvgtol: float = 1e-6, cnvgtest: int = 4,
                 single_inner: bool = True):
        """algorithm "linear" (Linear.cpp) or "newton" (NewtonRaphson.cpp, with
        `maxit` iterations, tolerance `cnvgtol` and convergence test `cnvgtest`:
        4 relative unbalanced force, 5 relative displacement increment).
        single_inner: the inner iterations of each solve apply the effective
        stiffness in single precision on elastic models without damping or
        constraints; every answer is confirmed with the FP64 operator (true
        residual) and the solve restarts from it, so the tolerance holds."""
        self.model = model
        self.dt = float(dt)
        self._md = model.desc()
        self.loads = loads or Loads()
        self._ld = self.loads.desc()
        algo = {"linear": capi.SVL_ALGO_LINEAR, "newton": capi.SVL_ALGO_NEWTON}[algorithm.lower()]
        opts = capi.NmOpts(dt=self.dt, ftol=ftol, mtol=mtol, pcg_tol=float(pcg_tol), pcg_maxit=int(pcg_maxit),
                           precond=int(precond), algorithm=algo, maxit=int(maxit), cnvgtol=float(cnvgtol),
                           cnvgtest=int(cnvgtest), single_inner=1 if single_inner else 0,
                           integrator=self._integrator)
        h = C.c_void_p()
        check(lib().svl_nm_create(C.byref(self._md), C.byref(self._ld), C.byref(opts), C.byref(h)))
        self._h = h
        self.ntotal = model.ntotal

    def Initialize(self, U0=None, V0=None, A0=None):
        arrs = [None if a is None else capi.as_f64(a) for a in (U0, V0, A0)]
        check(lib().svl_nm_set_initial(self._h, *(ptr(a, C.c_double) for a in arrs)))

    def ComputeNewStep(self, k: int) -> bool:
        """One step k; returns True on failure (the reference's `stop`)."""
        return lib().svl_nm_run(self._h, int(k), 1, ptr(None, C.c_double)) != capi.SVL_OK

    def GetDisplacements(self) -> np.ndarray:
        return self._get(0)

    def GetVelocities(self) -> np.ndarray:
        return self._get(1)

    def GetAccelerations(self) -> np.ndarray:
        return self._get(2)

    def ComputeProgressiveForce(self, k: int) -> np.ndarray:
        """Fext(k) + Fbar (ComputeProgressiveForce of the reference's
        integrators, e.g. CentralDifference.cpp:174-186): the stage force Fbar
        of earlier stages is zero in a single-stage run."""
        return self.loads.external_force(self.ntotal, int(k))

    def element_response(self, response: str, elems) -> np.ndarray:
        """ELEMENT recorder values after the last step (as CentralDifference)."""
        return _element_response(lib().svl_nm_element_response, self._h, self.model, response, elems)

    def ComputeReactionForce(self, k: int) -> np.ndarray:
        """Reaction forces after step k (NewmarkBeta::ComputeReactionForce):
        total-dof vector, zeros off the fixed nodes."""
        R = np.zeros(self.ntotal)
        check(lib().svl_nm_reaction(self._h, int(k), ptr(R, C.c_double)))
        return R

    def run(self, k_first: int, nsteps: int, history: bool = False):
        hist = np.zeros((nsteps, self.ntotal)) if history else None
        check(lib().svl_nm_run(self._h, int(k_first), int(nsteps), ptr(hist, C.c_double)))
        return hist

    def run_timed(self, k_first: int, nsteps: int) -> float:
        ms = C.c_float()
        check(lib().svl_nm_run_timed(self._h, int(k_first), int(nsteps), C.byref(ms)))
        return float(ms.value)

    # -- learned preconditioner (lattice models) ---------------------------
    def train_preconditioner(self, k_first: int, solve_steps: int = 0, record_every: int = 4,
                             n_synthetic: int = 300, iters: int = 1500, batch: int = 8, lr: float = 2e-3,
                             seed: int = 0, max_sweeps: int = 0, crop: int = 0) -> float:
        """Optionally advance solve_steps steps with Jacobi-PCG recording CG
        iterates, add synthetic pairs (K_eff e for random e with 0..max_sweeps
        smoothing sweeps), train the network in segments keeping the weights
        whose trial flexible-CG solve of step k_first + solve_steps needs the
        fewest iterations, and switch to the learned preconditioner.  crop > 0
        trains on random crop^3 windows of the pairs instead of the whole
        lattice.  Returns the training loss (mean relative squared error) of
        the kept weights."""
        o = capi.NnTrainOpts(solve_steps=solve_steps, record_every=record_every, n_synthetic=n_synthetic,
                             iters=iters, batch=batch, lr=lr, seed=seed, max_sweeps=max_sweeps, crop=crop)
        loss = C.c_float()
        check(lib().svl_nm_train_preconditioner(self._h, int(k_first), C.byref(o), C.byref(loss)))
        return float(loss.value)

    def set_preconditioner(self, precond: int):
        check(lib().svl_nm_set_preconditioner(self._h, int(precond)))

    def nn_weights(self, new=None) -> np.ndarray:
        n = lib().svl_nn_num_weights()
        out = np.zeros(n, np.float32)
        w_in = None if new is None else np.ascontiguousarray(new, dtype=np.float32)
        check(lib().svl_nm_preconditioner_weights(self._h, ptr(out, C.c_float), ptr(w_in, C.c_float)))
        return out

    def precond_stats(self):
        """(solves with the learned preconditioner, fallbacks to Jacobi, last Jacobi iteration count)."""
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().svl_nm_precond_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return int(a.value), int(b.value), int(c.value)

    def lattice(self):
        d = np.zeros(3, np.int32)
        check(lib().svl_nm_lattice(self._h, ptr(d, C.c_int32)))
        return tuple(int(v) for v in d)

    def nn_loss_grad(self, x, t):
        """Device loss and weight gradient of one sample (grids [3][nz][ny][nx])."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1, np.float32)
        grad = np.zeros(lib().svl_nn_num_weights(), np.float32)
        check(lib().svl_nm_nn_loss_grad(self._h, ptr(x, C.c_float), ptr(t, C.c_float), ptr(loss, C.c_float),
                                        ptr(grad, C.c_float)))
        return float(loss[0]), grad

    def nn_forward(self, x, path: int = 1):
        """Network output y for an r_hat grid x ([3][nz][ny][nx]); path 0 = FP32
        CUDA cores, 1 = BF16 tensor cores."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros_like(x)
        check(lib().svl_nm_nn_forward(self._h, ptr(x, C.c_float), ptr(y, C.c_float), int(path)))
        return y

    def nn_set_path(self, path: int):
        check(lib().svl_nm_nn_set_path(self._h, int(path)))

    def nn_grids(self):
        nx, ny, nz = self.lattice()
        rho = np.zeros((3, nz, ny, nx), np.float32)
        mask = np.zeros((3, nz, ny, nx), np.float32)
        check(lib().svl_nm_nn_grids(self._h, ptr(rho, C.c_float), ptr(mask, C.c_float)))
        return rho, mask

    def stats(self):
        """(CG iterations over all solves, of the last solve, last true relative residual)."""
        a, b, r = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().svl_nm_stats(self._h, C.byref(a), C.byref(b), C.byref(r)))
        return int(a.value), int(b.value), float(r.value)

    def newton_stats(self):
        """(Newton iterations over all steps, of the last step, last convergence-test value)."""
        a, b, r = C.c_int64(), C.c_int64(), C.c_double()
        check(lib().svl_nm_newton_stats(self._h, C.byref(a), C.byref(b), C.byref(r)))
        return int(a.value), int(b.value), float(r.value)

    def launches(self) -> int:
        n = C.c_int64()
        check(lib().svl_nm_launch_count(self._h, C.byref(n)))
        return int(n.value)

    def _get(self, which):
        out = np.zeros(self.ntotal)
        check(lib().svl_nm_get(self._h, which, ptr(out, C.c_double)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().svl_nm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _cd_nondiagonal(model: Model) -> bool:
    """True when K = M/dt^2 + C/2dt of CentralDifference (CentralDifference.cpp:70)
    has off-diagonal entries: a consistent mass or ak != 0 on some element."""
    if not model.lumped:
        return True
    ray = getattr(model, "rayleigh", None)
    return ray is not None and bool(np.any(np.asarray(ray)[:, 1] != 0.0))


class CentralDifferenceSolve(NewmarkBeta):
    """CentralDifference whose effective stiffness K = M/dt^2 + C/2dt is not
    diagonal (CentralDifference.cpp:64-70 with a consistent mass, massform
    CONSISTENT, or stiffness-proportional Rayleigh damping): each step solves
    T^T K T du = Feff (CentralDifference.cpp:204-231) by the matrix-free
    Jacobi-PCG of svl_nm in its central-difference mode to a true relative
    residual of `pcg_tol`, where the reference factorises K once.  Elastic
    and J2 materials, EQUAL constraints, support motion and dashpots; same
    step methods as CentralDifference; reaction forces are not covered."""

    _integrator = capi.SVL_NM_CENTRAL_DIFFERENCE

    def __init__(self, model: Model, loads: Loads | None, dt: float, ftol: float = 1e-12,
                 mtol: float = 1e-12, check_every: int = 0, pcg_tol: float = 1e-12, pcg_maxit: int = 20000):
        super().__init__(model, loads, dt, pcg_tol=pcg_tol, pcg_maxit=pcg_maxit, ftol=ftol, mtol=mtol,
                         single_inner=False)


class StructuredEnsemble(StructuredCentralDifference):
    """Instances of uneven lin3DHexa8 grids (same element size) advanced by
    one fused tensor-core kernel per step (svl_cdx_create_ensemble): each
    instance is embedded in the bounding grid and only the tiles that meet its
    own nodes are scheduled.  `grids` lists (ne, origin) per instance."""

    def __init__(self, grids, h, instances, dt: float, mtol: float = 1e-12):
        self.dt = float(dt)
        self.ninst = len(instances)
        specs = (capi.GridSpec * self.ninst)()
        for b, (ne, origin) in enumerate(grids):
            specs[b].ndim = 3
            for i in range(3):
                specs[b].ne[i] = int(ne[i])
                specs[b].h[i] = float(h[i])
                specs[b].origin[i] = float(origin[i])
        self._spec = specs
        md = (capi.ModelDesc * self.ninst)()
        ld = (capi.LoadDesc * self.ninst)()
        self._keep = []
        for i, (m, L) in enumerate(instances):
            md[i] = m.desc()
            self._keep.append(m)
            L = L or Loads()
            ld[i] = L.desc()
            self._keep.append(L)
        self._md, self._ld = md, ld
        opts = capi.CdOpts(dt=self.dt, ftol=0.0, mtol=mtol, precision=capi.SVL_PREC_MIXED, check_every=0)
        hnd = C.c_void_p()
        check(lib().svl_cdx_create_ensemble(specs, self.ninst, md, ld, C.byref(opts), C.byref(hnd)))
        self._h = hnd
        self.ntotals = [int(m.ntotal) for m, _ in instances]
        self.offsets = np.concatenate([[0], np.cumsum(self.ntotals)])

    def run(self, k_first: int, nsteps: int, history: bool = False, out=None):
        """Steps of every instance; history (or `out`, float64 [nsteps,
        sum of the instances' total dofs]) receives all displacements, the
        instances one after the other (see split)."""
        n = int(self.offsets[-1])
        hist = out if out is not None else (np.zeros((nsteps, n)) if history else None)
        if hist is not None:
            assert hist.shape == (nsteps, n) and hist.dtype == np.float64 and hist.flags["C_CONTIGUOUS"]
        check(lib().svl_cdx_run(self._h, int(k_first), int(nsteps), ptr(hist, C.c_double)))
        return hist

    def split(self, hist):
        """Per-instance views [nsteps, ntotal_b] of a history."""
        return [hist[:, self.offsets[b]:self.offsets[b + 1]] for b in range(self.ninst)]

    def get(self, inst: int, which: int = 0) -> np.ndarray:
        out = np.zeros(self.ntotals[inst])
        check(lib().svl_cdx_get(self._h, int(inst), int(which), ptr(out, C.c_double)))
        return out


ELEMENT_RESPONSES = {"STRAIN": 0, "STRESS": 1, "INTERNALFORCE": 2, "STRAINRATE": 3}


def _element_response(fn, h, model: Model, response: str, elems) -> np.ndarray:
    code = ELEMENT_RESPONSES[response.upper()]
    el = capi.as_i32(np.asarray(elems, dtype=np.int32).ravel())
    nen = model.conn.shape[1]
    ngp = 4 if model.ndim == 2 else 8
    shape = (el.size, nen * model.ndim) if code == 2 else (el.size, ngp, 3 if model.ndim == 2 else 6)
    out = np.zeros(shape)
    check(fn(h, code, int(el.size), ptr(el, C.c_int32), ptr(out, C.c_double)))
    return out


def _central_difference_pml(model, loads, dt, ftol=1e-12, mtol=1e-12, check_every=0):
    """CentralDifference on a model with PML layers: the explicit staggered
    scheme of the PML-capable handle."""
    return ExtendedNewmarkBeta(model, loads, dt, ftol=ftol, mtol=mtol, integrator="centraldifference")


def _newmark_pml(model: Model, loads: Loads | None, dt: float, pcg_tol: float = 1e-8, pcg_maxit: int = 20000,
                 ftol: float = 1e-12, mtol: float = 1e-12, precond: int = 0, algorithm: str = "linear",
                 maxit: int = 50, cnvgtol: float = 1e-6, cnvgtest: int = 4, single_inner: bool = True):
    if precond != capi.SVL_PRECOND_JACOBI:
        raise capi.SvlError(capi.SVL_ERR_UNSUPPORTED, "the learned preconditioner does not cover PML models")
    return ExtendedNewmarkBeta(model, loads, dt, tol=pcg_tol, solver_maxit=int(pcg_maxit), ftol=ftol,
                               mtol=mtol, algorithm=algorithm, maxit=maxit, cnvgtol=cnvgtol, cnvgtest=cnvgtest,
                               integrator="newmark")
