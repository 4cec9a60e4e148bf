"""The tensor-core step stores the lin3DHexa8 stiffness patterns of a cube
as integers: K = lambda K_lambda + mu K_mu with K_lambda, K_mu integer
matrices times h/72 (|entries| <= 32), exact in TF32, h/72 folded into
lambda and mu.  Pinned here against the oracle's element stiffness
(lin3DHexa8.cpp:289-318 with the 15-digit Gauss abscissa): two materials
give K_lambda and K_mu entry by entry, and both are integers times h/72 up
to the abscissa's rounding."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300 import _capi as capi
from svl_gb300.model import Model, elastic_params


def _cube_k(h, E, nu):
    m = Model.grid(3, (1, 1, 1), (h, h, h), fix_mask=(0, 0, 0, 0, 0, 0),
                   mat_type=np.array([capi.SVL_MAT_ELASTIC3DLINEAR], np.int32),
                   mat_param=elastic_params(3, E, nu, 2000.0)[None, :])
    K, _, _ = O.element_matrices(m, 0)
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    return K, lam, mu


@pytest.mark.parametrize("h", [2.0, 0.5, 3.0])
def test_cube_stiffness_patterns_are_integers_times_h_over_72(h):
    K1, l1, m1 = _cube_k(h, 2.0e8, 0.25)
    K2, l2, m2 = _cube_k(h, 3.0e8, 0.35)
    det = l1 * m2 - l2 * m1
    Kl = (K1 * m2 - K2 * m1) / det
    Km = (l1 * K2 - l2 * K1) / det
    for P in (Kl, Km):
        v = P * 72.0 / h
        r = np.round(v)
        assert np.abs(v - r).max() <= 1e-6 * max(1.0, np.abs(v).max())
        assert np.abs(r).max() <= 32 and np.abs(r).max() >= 1
    # the reconstruction is the element's matrix
    assert np.allclose(l1 * Kl + m1 * Km, K1, rtol=1e-12, atol=1e-9 * np.abs(K1).max())
