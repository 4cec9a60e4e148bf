"""The oracle's ExtendedNewmarkBeta with PML elements (XNewmark in
oracle/svl_oracle.cpp): assembled operators, reduction to NewmarkBeta without
PML, the support-motion step index, and absorption by the layers."""
import numpy as np
import pytest

from oracle import oracle as O
from svl_gb300.model import Loads
from tests.helpers import h8_box, pml_box, q4_box, q4_j2_columns, rel_l2


@pytest.mark.parametrize("ndim", [2, 3])
def test_pml_model_operators(ndim):
    m, L, dt = pml_box(ndim, (4, 3) if ndim == 2 else (2, 2, 2), npml=2)
    assert m.elem_pml.sum() > 0 and m.ntotal > m.nnode * ndim
    K, M, Cm, G = O.xnewmark_matrices(m)
    for A in (K, M, Cm, G):
        assert np.allclose(A, A.T, rtol=0, atol=1e-12 * max(np.abs(A).max(), 1.0))
    stress = np.zeros(m.ntotal, bool)
    for n in range(m.nnode):
        stress[m.totaldof[n, ndim:m.node_ndof[n]]] = True
    d = np.diag(M)
    assert np.all(d[stress] < 0) and np.all(d[~stress] > 0)
    assert (np.abs(G).max() == 0.0) == (ndim == 2)          # PML2DQuad4 has no history matrix
    assert np.count_nonzero(K[np.ix_(~stress, stress)]) > 0


def test_without_pml_equals_newmark_linear():
    for m, L, dt in (q4_box(8, 5, nt=40), h8_box(3, 3, 2, nt=40)):
        m.rayleigh = np.tile([1.5, 1.0e-3], (m.nelem, 1))
        h0, _ = O.newmark_run(m, L, 4 * dt, 30, solver=0)
        h1, *_ = O.xnewmark_run(m, L, 4 * dt, 30)
        assert np.abs(h0).max() > 0
        assert rel_l2(h1, h0) <= 1e-12


def test_support_motion_index_is_the_current_step():
    """ExtendedNewmarkBeta takes the increment of step k (ExtendedNewmarkBeta.cpp:196),
    NewmarkBeta that of step k - 1 (NewmarkBeta.cpp:187): with the series shifted
    by one the two runs coincide."""
    m, L, dt = q4_j2_columns(ncol=1, width=3, heights=(6,), nt=60)
    E_nu = np.zeros_like(m.mat_param)
    G, K, rho = m.mat_param[:, 1], m.mat_param[:, 0], m.mat_param[:, 2]
    E_nu[:, 0] = 9 * K * G / (3 * K + G)
    E_nu[:, 1] = (3 * K - 2 * G) / (2 * (3 * K + G))
    E_nu[:, 2] = rho
    m.mat_param = E_nu
    from svl_gb300 import _capi as capi
    m.mat_type = np.full_like(m.mat_type, capi.SVL_MAT_ELASTIC2DPLANESTRAIN)
    assert L.series[0][0] == 0.0
    Ls = Loads()
    Ls.series = [np.concatenate([s[1:], s[-1:]]) for s in L.series]
    Ls.sm_dof, Ls.sm_series, Ls.sm_factor = list(L.sm_dof), list(L.sm_series), list(L.sm_factor)
    hx, *_ = O.xnewmark_run(m, L, 2 * dt, 40)
    hn, _ = O.newmark_run(m, Ls, 2 * dt, 40, solver=0)
    assert np.abs(hx).max() > 0
    assert rel_l2(hx, hn) <= 1e-12


def test_layers_absorb_the_outgoing_wave():
    m, L, dt = pml_box(2, (12, 6), npml=3, nt=260, f0=10.0, dt_factor=1.0)
    h, U, V, A, Ub = O.xnewmark_run(m, L, dt, 250)
    interior = m.totaldof[m.node_ndof == 2][:, :2].ravel()
    e = (h[:, interior] ** 2).sum(axis=1)
    assert np.all(np.isfinite(h)) and np.abs(Ub).max() > 0
    assert e[-1] < 1e-4 * e.max()
