"""GPU element action of PML2DQuad4 / PML3DHexa8 (svl_pml_element_action)
against the oracle's assembled element matrices: y = cM M u0 + cC C u1 +
cK K u2 + cG G u3, relative error <= 1e-12 per element."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import _capi as capi
from tests.test_pml_oracle import PAR2, PAR3, hexa, quad

pytestmark = pytest.mark.gpu


def _gpu_action(ndim, X, mat, thick, par, coef, u):
    lib = capi.lib()
    y = np.zeros(u.shape[1:])
    f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    X, mat, thick, par, coef, u = map(f, (X, mat, thick, par, coef, u))
    capi.check(lib.svl_pml_element_action(ndim, X.shape[0], capi.ptr(X, C.c_double), capi.ptr(mat, C.c_double),
                                          capi.ptr(thick, C.c_double), capi.ptr(par, C.c_double),
                                          capi.ptr(coef, C.c_double), capi.ptr(u, C.c_double), capi.ptr(y, C.c_double)))
    return y


@pytest.mark.parametrize("ndim", [2, 3])
def test_pml_action_matches_oracle_matrices(gpu, ndim):
    rng = np.random.default_rng(ndim)
    ne = 37
    nc = 20 if ndim == 2 else 72
    shift = np.array([0.0, -8.0]) if ndim == 2 else np.array([0.0, 0.0, -8.0])
    X = np.stack([(quad(jitter=0.15, seed=i) if ndim == 2 else hexa(jitter=0.15, seed=i)) + shift * (1 + 0.1 * i % 3)
                  for i in range(ne)])
    mat = np.stack([[2.0e8 * (1 + 0.5 * rng.uniform()), 0.2 + 0.15 * rng.uniform(), 1800 + 400 * rng.uniform()]
                    for _ in range(ne)])
    thick = 1.0 + 0.2 * rng.uniform(size=ne) if ndim == 2 else None
    par = np.tile(PAR2 if ndim == 2 else PAR3, (ne, 1))
    coef = np.array([0.7, -1.3, 2.1, 0.4 if ndim == 3 else 0.0])
    u = rng.standard_normal((4, ne, nc))
    y = _gpu_action(ndim, X, mat, thick, par, coef, u)
    for e in range(ne):
        mats = O.pml_matrices(ndim, X[e], *mat[e], par[e], t=(thick[e] if thick is not None else 1.0))
        ref = sum(coef[i] * mats[i] @ u[i, e] for i in range(4))
        assert np.linalg.norm(y[e] - ref) <= 1e-12 * np.linalg.norm(ref), e


def test_pml_internal_force_is_k_times_u(gpu):
    X = hexa(jitter=0.1)[None] + np.array([0.0, 0.0, -8.0])
    mat = np.array([[3.0e8, 0.25, 2100.0]])
    u = np.zeros((4, 1, 72))
    u[2] = np.random.default_rng(9).standard_normal((1, 72))
    y = _gpu_action(3, X, mat, None, PAR3[None], np.array([0.0, 0.0, 1.0, 0.0]), u)
    K = O.pml_matrices(3, X[0], *mat[0], PAR3)[2]
    assert np.linalg.norm(y[0] - K @ u[2, 0]) <= 1e-12 * np.linalg.norm(K @ u[2, 0])
