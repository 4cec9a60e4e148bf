"""ctypes binding of the CPU oracle (oracle/svl_oracle.cpp).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline arm, as the checker -- never by the svl_gb300 product.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ORACLE_LIB = Path(__file__).resolve().parent / "_build" / "libsvl_oracle.so"
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError("oracle library missing (%s); run __graft_entry__.build()" % ORACLE_LIB)
        L = C.CDLL(str(ORACLE_LIB))
        vp = C.c_void_p
        f64p = C.POINTER(C.c_double)
        L.oracle_cd_run.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                    f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p]
        L.oracle_newmark_run.argtypes = [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                         C.c_int, C.c_double, f64p, C.POINTER(C.c_long), C.POINTER(C.c_int)]
        L.oracle_element_fint.argtypes = [vp, f64p, f64p]
        L.oracle_element_matrices.argtypes = [vp, C.c_int, f64p, f64p, f64p]
        L.oracle_body_force.argtypes = [vp, C.c_int, f64p, f64p]
        L.oracle_lumped_mass.argtypes = [vp, C.c_double, f64p]
        L.oracle_j2_path.argtypes = [C.c_int, f64p, C.c_int, f64p, f64p]
        L.oracle_pml_matrices.argtypes = [C.c_int, f64p, C.c_double, C.c_double, C.c_double, C.c_double, f64p,
                                          f64p, f64p, f64p, f64p]
        L.oracle_reaction_run.argtypes = [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                          f64p]
        L.oracle_xnewmark_run.argtypes = [vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_int, f64p, f64p, f64p, f64p, f64p, C.POINTER(C.c_int),
                                          C.POINTER(C.c_double)]
        L.oracle_xnewmark_matrices.argtypes = [vp, f64p, f64p, f64p, f64p]
        L.oracle_cdpml_run.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                       f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p, f64p]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return C.cast(None, C.POINTER(C.c_double))
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def cd_run(model, loads, dt, nsteps, k_first=1, ftol=1e-12, mtol=1e-12, mode=0, history=True,
           U0=None, V0=None, A0=None, timing=None):
    """Central difference on the CPU; returns (hist [nsteps, ntotal] or None, U, V, A).
    If `timing` is a dict, timing['seconds'] receives the step-loop wall time."""
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    nt = model.ntotal
    hist = np.zeros((nsteps, nt)) if history else None
    U, V, A = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (U0, V0, A0)]
    secs = np.zeros(1)
    st = lib().oracle_cd_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, ftol, mtol,
                             k_first, nsteps, mode, _p(keep[0]), _p(keep[1]), _p(keep[2]),
                             _p(hist) if hist is not None else _p(None),
                             U.ctypes.data_as(C.POINTER(C.c_double)), V.ctypes.data_as(C.POINTER(C.c_double)),
                             A.ctypes.data_as(C.POINTER(C.c_double)), secs.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise RuntimeError("oracle_cd_run failed with status %d" % st)
    if timing is not None:
        timing["seconds"] = float(secs[0])
    return hist, U, V, A


def newmark_run(model, loads, dt, nsteps, k_first=1, algo=0, maxit=50, cnvgtol=1e-6, solver=0, pcg_tol=1e-12,
                step_iters=None):
    """algo 0 Linear, 1 Newton with test 5, 2 Newton with test 4, 10 + t
    Newton with test t (1..8); solver 0
    dense LDL^T, 1 Jacobi-PCG.  step_iters (int32 [nsteps]) receives the
    Newton iterations of every step."""
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    hist = np.zeros((nsteps, model.ntotal))
    it = C.c_long(0)
    si = None if step_iters is None else step_iters.ctypes.data_as(C.POINTER(C.c_int))
    st = lib().oracle_newmark_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, k_first,
                                  nsteps, algo, maxit, cnvgtol, solver, pcg_tol,
                                  hist.ctypes.data_as(C.POINTER(C.c_double)), C.byref(it), si)
    if st != 0:
        raise RuntimeError("oracle_newmark_run failed with status %d" % st)
    return hist, it.value


def element_fint(model, U):
    nc = model.conn.shape[1] * model.ndim
    out = np.zeros((model.nelem, nc))
    md = model.desc()
    Ua = np.ascontiguousarray(U, dtype=np.float64)
    st = lib().oracle_element_fint(C.addressof(md), Ua.ctypes.data_as(C.POINTER(C.c_double)),
                                   out.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    return out


def element_matrices(model, e):
    nc = model.conn.shape[1] * model.ndim
    K, Ml, Mc = np.zeros((nc, nc)), np.zeros((nc, nc)), np.zeros((nc, nc))
    md = model.desc()
    st = lib().oracle_element_matrices(C.addressof(md), e, K.ctypes.data_as(C.POINTER(C.c_double)),
                                       Ml.ctypes.data_as(C.POINTER(C.c_double)),
                                       Mc.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    return K, Ml, Mc


def body_force(model, e, q):
    nc = model.conn.shape[1] * model.ndim
    fe = np.zeros(nc)
    md = model.desc()
    qa = np.ascontiguousarray(q, dtype=np.float64)
    st = lib().oracle_body_force(C.addressof(md), e, qa.ctypes.data_as(C.POINTER(C.c_double)),
                                 fe.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    return fe


def lumped_mass(model, mtol=1e-12):
    M = np.zeros(model.ntotal)
    md = model.desc()
    st = lib().oracle_lumped_mass(C.addressof(md), mtol, M.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    return M


def j2_path(mat_type, param, strains):
    strains = np.ascontiguousarray(strains, dtype=np.float64)
    out = np.zeros_like(strains)
    p = np.ascontiguousarray(param, dtype=np.float64)
    st = lib().oracle_j2_path(mat_type, p.ctypes.data_as(C.POINTER(C.c_double)), strains.shape[0],
                              strains.ctypes.data_as(C.POINTER(C.c_double)), out.ctypes.data_as(C.POINTER(C.c_double)))
    assert st == 0
    return out


def num_threads():
    lib().oracle_num_threads.restype = C.c_int
    return lib().oracle_num_threads()


def pml_matrices(ndim, X, E, nu, rho, par, t=1.0):
    """(M, C, K, G) of one PML2DQuad4 / PML3DHexa8 element."""
    nc = 20 if ndim == 2 else 72
    out = [np.zeros((nc, nc)) for _ in range(4)]
    Xa = np.ascontiguousarray(X, dtype=np.float64)
    pa = np.ascontiguousarray(par, dtype=np.float64)
    f64 = C.POINTER(C.c_double)
    st = lib().oracle_pml_matrices(int(ndim), Xa.ctypes.data_as(f64), float(E), float(nu), float(rho), float(t),
                                   pa.ctypes.data_as(f64), *[o.ctypes.data_as(f64) for o in out])
    assert st == 0
    return out


def xnewmark_run(model, loads, dt, nsteps, k_first=1, algo=0, maxit=50, cnvgtol=1e-6, step_iters=None,
                 newmark=False, last_res=None):
    """ExtendedNewmarkBeta (or, newmark=True, NewmarkBeta) on models with PML
    elements (dense LDL^T); algo 0 Linear, 1 Newton with test 5, 2 Newton
    with test 4, 10 + t Newton with test t (Algorithm.cpp:122-188).  Returns
    (history of U [nsteps, ntotal], final U, V, A, Ubar); step_iters (int32
    [nsteps]) receives the iterations of every step, last_res (float64 [1])
    the last step's final convergence-test value."""
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    nt = model.ntotal
    hist = np.zeros((nsteps, nt))
    U, V, A, Ub = (np.zeros(nt) for _ in range(4))
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    si = None if step_iters is None else step_iters.ctypes.data_as(C.POINTER(C.c_int))
    st = lib().oracle_xnewmark_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, k_first,
                                   nsteps, algo, maxit, cnvgtol, int(bool(newmark)), f(hist), f(U), f(V), f(A),
                                   f(Ub), si, None if last_res is None else f(last_res))
    if st != 0:
        raise RuntimeError("oracle_xnewmark_run failed with status %d" % st)
    return hist, U, V, A, Ub


def cdpml_run(model, loads, dt, nsteps, k_first=1, ftol=1e-12, mtol=1e-12, history=True, timing=None):
    """Explicit central difference on a model with PML layers (the staggered
    scheme of CDPml in svl_oracle.cpp).  Returns (history of the total-dof
    vector [nsteps, ntotal] or None, U, V, A, Ubar); on PML nodes the stress
    dofs hold S at the half step after U's time.  timing['seconds'] receives
    the step-loop wall time when `timing` is a dict."""
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    nt = model.ntotal
    hist = np.zeros((nsteps, nt)) if history else None
    U, V, A, Ub = (np.zeros(nt) for _ in range(4))
    secs = np.zeros(1)
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    st = lib().oracle_cdpml_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, ftol, mtol,
                                k_first, nsteps, _p(None), _p(None), _p(None), f(hist) if hist is not None else _p(None),
                                f(U), f(V), f(A), f(Ub), f(secs))
    if st != 0:
        raise RuntimeError("oracle_cdpml_run failed with status %d" % st)
    if timing is not None:
        timing["seconds"] = float(secs[0])
    return hist, U, V, A, Ub


def reaction_run(model, loads, dt, nsteps, k_first=1, integrator="cd", algo=0, maxit=50, cnvgtol=1e-6):
    """Reaction forces (total dofs; zeros off the fixed nodes) after nsteps of
    central difference ("cd"), NewmarkBeta ("newmark"), ExtendedNewmarkBeta
    ("xnewmark") or the PML model's NewmarkBeta mode ("xnewmark_nm"); algo as
    newmark_run."""
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    R = np.zeros(model.ntotal)
    st = lib().oracle_reaction_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, k_first, nsteps,
                                   {"cd": 0, "newmark": 1, "xnewmark": 2, "xnewmark_nm": 3}.get(integrator, 1),
                                   algo, maxit, cnvgtol,
                                   R.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise RuntimeError("oracle_reaction_run failed with status %d" % st)
    return R


def element_response_run(model, loads, dt, nsteps, response, elems, k_first=1, integrator="cd", algo=0, maxit=50,
                         cnvgtol=1e-6):
    """ELEMENT recorder values (STRAIN, STRESS, INTERNALFORCE, STRAINRATE) of
    the element positions `elems` after nsteps of central difference or
    NewmarkBeta; [n, ngp, 3|6] or [n, NC]."""
    code = {"STRAIN": 0, "STRESS": 1, "INTERNALFORCE": 2, "STRAINRATE": 3}[response.upper()]
    md = model.desc()
    ld = loads.desc() if loads is not None else None
    el = np.ascontiguousarray(np.asarray(elems, dtype=np.int32).ravel())
    nen = model.conn.shape[1]
    ngp = 4 if model.ndim == 2 else 8
    shape = (el.size, nen * model.ndim) if code == 2 else (el.size, ngp, 3 if model.ndim == 2 else 6)
    out = np.zeros(shape)
    L = lib()
    L.oracle_element_response_run.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int),
                                              C.POINTER(C.c_double)]
    st = L.oracle_element_response_run(C.addressof(md), C.addressof(ld) if ld is not None else None, dt, k_first,
                                       nsteps, 0 if integrator == "cd" else 1, algo, maxit, cnvgtol, code, int(el.size),
                                       el.ctypes.data_as(C.POINTER(C.c_int)), out.ctypes.data_as(C.POINTER(C.c_double)))
    if st != 0:
        raise RuntimeError("oracle_element_response_run failed with status %d" % st)
    return out


def xnewmark_matrices(model):
    """Dense total-dof K, M, C, G of an ExtendedNewmark model (small models)."""
    nt = model.ntotal
    out = [np.zeros((nt, nt)) for _ in range(4)]
    md = model.desc()
    st = lib().oracle_xnewmark_matrices(C.addressof(md), *(o.ctypes.data_as(C.POINTER(C.c_double)) for o in out))
    if st != 0:
        raise RuntimeError("oracle_xnewmark_matrices failed with status %d" % st)
    return out
