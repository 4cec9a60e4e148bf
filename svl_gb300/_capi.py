"""ctypes view of include/svl_gb300.h.

This is the Python-side binding of the C ABI (the same binding a reference
maintainer would add with ctypes).  The library must have been built in-tree
(`__graft_entry__.build()`); loading fails loudly otherwise -- there is no CPU
fallback in the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsvl_gb300.so"

SVL_OK = 0
SVL_ERR_INVALID = 1
SVL_ERR_CUDA = 2
SVL_ERR_NONFINITE = 3
SVL_ERR_MAXITER = 4
SVL_ERR_BREAKDOWN = 5
SVL_ERR_UNSUPPORTED = 6
SVL_ERR_NOMEM = 7
SVL_ERR_NODEVICE = 8

SVL_ELEM_LIN2DQUAD4 = 1
SVL_ELEM_LIN3DHEXA8 = 2

SVL_MAT_ELASTIC2DPLANESTRAIN = 1
SVL_MAT_ELASTIC3DLINEAR = 2
SVL_MAT_PLASTICPLANESTRAINJ2 = 3
SVL_MAT_PLASTIC3DJ2 = 4
SVL_MAT_NPARAM = 8

SVL_NOALLOC_SCRATCH_BYTES = 8 << 20

SVL_PREC_FP64 = 0
SVL_PREC_MIXED = 1

SVL_PRECOND_JACOBI = 0
SVL_PRECOND_LEARNED = 1

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


class ModelDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("nnode", C.c_int32), ("ndof", C.c_int32),
        ("coords", f64p), ("totaldof", i32p), ("freedof", i32p),
        ("ntotal", C.c_int32), ("nfree", C.c_int32),
        ("nconstraint", C.c_int32), ("con_slave", i32p), ("con_ptr", i32p),
        ("con_master", i32p), ("con_factor", f64p),
        ("elem_type", C.c_int32), ("nelem", C.c_int32), ("conn", i32p),
        ("elem_mat", i32p), ("elem_thickness", f64p),
        ("nmat", C.c_int32), ("mat_type", i32p), ("mat_param", f64p),
        ("lumped", C.c_int32), ("node_mass", f64p), ("elem_rayleigh", f64p),
        ("node_ndof", i32p), ("elem_pml", i32p), ("elem_pml_param", f64p),
        ("ndashpot", C.c_int32), ("dashpot_dof", i32p), ("dashpot_eta", f64p),
    ]


class LoadDesc(C.Structure):
    _fields_ = [
        ("nseries", C.c_int32), ("series_ptr", i32p), ("series_val", f64p),
        ("nforce", C.c_int32), ("force_dof", i32p), ("force_series", i32p), ("force_coef", f64p),
        ("nsupport", C.c_int32), ("sm_dof", i32p), ("sm_series", i32p), ("sm_factor", f64p),
        ("ndrm", C.c_int32), ("drm_elem", i32p), ("drm_factor", f64p), ("drm_nt", C.c_int32),
        ("drm_node_row", i32p), ("drm_node_ext", i32p), ("drm_motion", f64p),
    ]


class GridSpec(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("ne", C.c_int32 * 3), ("h", C.c_double * 3),
        ("origin", C.c_double * 3), ("fix_mask", C.c_int32 * 6), ("periodic_x", C.c_int32),
    ]


class CdOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("ftol", C.c_double), ("mtol", C.c_double),
                ("precision", C.c_int32), ("check_every", C.c_int32)]


SVL_ALGO_LINEAR = 0
SVL_ALGO_NEWTON = 1


class NmOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("ftol", C.c_double), ("mtol", C.c_double), ("pcg_tol", C.c_double),
                ("pcg_maxit", C.c_int32), ("precond", C.c_int32), ("algorithm", C.c_int32), ("maxit", C.c_int32),
                ("cnvgtol", C.c_double), ("cnvgtest", C.c_int32), ("single_inner", C.c_int32),
                ("integrator", C.c_int32)]


SVL_NM_NEWMARK = 0
SVL_NM_CENTRAL_DIFFERENCE = 1


class XnmOpts(C.Structure):
    _fields_ = [("dt", C.c_double), ("ftol", C.c_double), ("mtol", C.c_double), ("tol", C.c_double),
                ("maxit", C.c_int32), ("algorithm", C.c_int32), ("newton_maxit", C.c_int32),
                ("cnvgtest", C.c_int32), ("cnvgtol", C.c_double), ("integrator", C.c_int32),
                ("single_inner", C.c_int32)]


SVL_XNM_EXTENDED_NEWMARK = 0
SVL_XNM_NEWMARK = 1
SVL_XNM_CENTRAL_DIFFERENCE = 2


class NnTrainOpts(C.Structure):
    _fields_ = [("solve_steps", C.c_int32), ("record_every", C.c_int32), ("n_synthetic", C.c_int32),
                ("iters", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("seed", C.c_uint64),
                ("max_sweeps", C.c_int32), ("crop", C.c_int32)]


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (None -> NULL)."""
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


_lib = None


class SvlError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("svl status %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libsvl_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError("libsvl_gb300.so is missing (%s); run __graft_entry__.build()" % LIB_PATH)
    L = C.CDLL(str(LIB_PATH))
    L.svl_version.restype = C.c_char_p
    L.svl_last_error.restype = C.c_char_p
    L.svl_device_info.argtypes = [C.POINTER(C.c_int)] * 4
    L.svl_set_device.argtypes = [C.c_int]
    L.svl_grid_sizes.argtypes = [C.POINTER(GridSpec)] + [C.POINTER(C.c_int32)] * 5
    L.svl_grid_build.argtypes = [C.POINTER(GridSpec), f64p, i32p, i32p, i32p, i32p, i32p, i32p, f64p]
    L.svl_element_body_force.argtypes = [C.POINTER(ModelDesc), C.c_int32, f64p, f64p]
    L.svl_lumped_mass.argtypes = [C.POINTER(ModelDesc), C.c_double, f64p]
    L.svl_cd_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(LoadDesc), C.POINTER(CdOpts), C.POINTER(C.c_void_p)]
    L.svl_cd_set_initial.argtypes = [C.c_void_p, f64p, f64p, f64p]
    L.svl_cd_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_cd_get.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_cd_reaction.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_cd_device_ptr.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]
    L.svl_cd_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.svl_cd_sync.argtypes = [C.c_void_p]
    L.svl_cd_run_timed.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    L.svl_cd_profile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_cdx_create.argtypes = [C.POINTER(GridSpec), C.c_int32, C.POINTER(ModelDesc), C.POINTER(LoadDesc),
                                 C.POINTER(CdOpts), C.POINTER(C.c_void_p)]
    L.svl_cdx_create_ensemble.argtypes = [C.POINTER(GridSpec), C.c_int32, C.POINTER(ModelDesc), C.POINTER(LoadDesc),
                                          C.POINTER(CdOpts), C.POINTER(C.c_void_p)]
    L.svl_cdx_set_initial.argtypes = [C.c_void_p, C.c_int32, f64p, f64p, f64p]
    L.svl_cdx_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_cdx_run_timed.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    L.svl_cdx_get.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_cdx_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.svl_cdx_set_ctas.argtypes = [C.c_void_p, C.c_int32]
    L.svl_cdx_profile.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_cdx_get_ctas.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
    L.svl_cdx_set_schedule.argtypes = [C.c_void_p, i32p]
    L.svl_cdx_get_schedule.argtypes = [C.c_void_p, i32p]
    L.svl_cdx_tune.argtypes = [C.c_void_p, C.c_int32, C.c_int32, i32p, C.POINTER(C.c_float)]
    L.svl_cdx_destroy.argtypes = [C.c_void_p]
    L.svl_cdx_destroy.restype = None
    L.svl_cd_run_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
    L.svl_cd_destroy.argtypes = [C.c_void_p]
    L.svl_cd_destroy.restype = None
    L.svl_host_alloc.argtypes = [C.c_size_t]
    L.svl_host_alloc.restype = C.c_void_p
    L.svl_host_free.argtypes = [C.c_void_p]
    L.svl_host_free.restype = None
    L.svl_xnm_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(LoadDesc), C.POINTER(XnmOpts), C.POINTER(C.c_void_p)]
    L.svl_xnm_set_initial.argtypes = [C.c_void_p, f64p, f64p, f64p, f64p]
    L.svl_xnm_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_xnm_get.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_xnm_reaction.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_cd_element_response.argtypes = [C.c_void_p, C.c_int32, C.c_int32, i32p, f64p]
    L.svl_nm_element_response.argtypes = [C.c_void_p, C.c_int32, C.c_int32, i32p, f64p]
    L.svl_xnm_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.svl_xnm_newton_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.svl_xnm_destroy.argtypes = [C.c_void_p]
    L.svl_xnm_destroy.restype = None
    L.svl_nm_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(LoadDesc), C.POINTER(NmOpts), C.POINTER(C.c_void_p)]
    L.svl_nm_set_initial.argtypes = [C.c_void_p, f64p, f64p, f64p]
    L.svl_nm_run.argtypes = [C.c_void_p, C.c_int32, C.c_int32, f64p]
    L.svl_nm_run_timed.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_float)]
    L.svl_nm_get.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_nm_reaction.argtypes = [C.c_void_p, C.c_int32, f64p]
    L.svl_nm_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.svl_nm_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.svl_nm_newton_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.svl_nm_sync.argtypes = [C.c_void_p]
    f32p = C.POINTER(C.c_float)
    L.svl_nm_train_preconditioner.argtypes = [C.c_void_p, C.c_int32, C.POINTER(NnTrainOpts), f32p]
    L.svl_nm_set_preconditioner.argtypes = [C.c_void_p, C.c_int32]
    L.svl_nm_preconditioner_weights.argtypes = [C.c_void_p, f32p, f32p]
    L.svl_nm_precond_stats.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 3
    L.svl_nm_lattice.argtypes = [C.c_void_p, i32p]
    L.svl_nm_nn_loss_grad.argtypes = [C.c_void_p, f32p, f32p, f32p, f32p]
    L.svl_nm_nn_grids.argtypes = [C.c_void_p, f32p, f32p]
    L.svl_nm_nn_forward.argtypes = [C.c_void_p, f32p, f32p, C.c_int32]
    L.svl_nm_nn_set_path.argtypes = [C.c_void_p, C.c_int32]
    L.svl_pml_element_action.argtypes = [C.c_int32, C.c_int32, f64p, f64p, f64p, f64p, f64p, f64p, f64p]
    L.svl_nm_destroy.argtypes = [C.c_void_p]
    L.svl_nm_destroy.restype = None
    _lib = L
    return L


def check(code):
    if code != SVL_OK:
        raise SvlError(code, lib().svl_last_error().decode())
    return code


def exported_symbols():
    """Names declared in include/svl_gb300.h (for the export test)."""
    import re
    hdr = Path(__file__).resolve().parent.parent / "include" / "svl_gb300.h"
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(svl_[a-z0-9_]+)\s*\(",
                       hdr.read_text(), flags=re.M)
    return sorted(set(names))


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def as_i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class _Pinned:
    def __init__(self, nbytes):
        self.p = lib().svl_host_alloc(nbytes)
        if not self.p:
            raise SvlError(SVL_ERR_NOMEM, lib().svl_last_error().decode())

    def __del__(self):
        try:
            lib().svl_host_free(self.p)
        except Exception:
            pass


def pinned_empty(shape, dtype=np.float64):
    """numpy array in page-locked host memory (svl_host_alloc); the memory is
    released when the array and its views are gone."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    owner = _Pinned(max(n, 1))
    buf = (C.c_char * max(n, 1)).from_address(owner.p)
    buf._owner = owner
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
