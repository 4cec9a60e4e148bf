"""ELEMENT recorder values of the oracle (Sim::element_response) against
restatements: the internal force of an elastic element is K_e u_e with the
oracle's element stiffness and the run's final displacement, the stress is
C eps of the recorded strain, and the strain rate of these materials is zero
(Elastic2DPlaneStrain.cpp:103-109)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import h8_box, q4_box


@pytest.mark.parametrize("builder", ["q4", "h8"])
def test_elastic_element_responses(builder):
    if builder == "q4":
        m, L, dt = q4_box(8, 5, nt=60)
    else:
        m, L, dt = h8_box(3, 3, 2, nt=60)
    n = 40
    els = [0, m.nelem // 2, m.nelem - 1]
    _, U, _, _ = O.cd_run(m, L, dt, n)[:4]
    F = O.element_response_run(m, L, dt, n, "INTERNALFORCE", els)
    E = O.element_response_run(m, L, dt, n, "STRAIN", els)
    S = O.element_response_run(m, L, dt, n, "STRESS", els)
    R = O.element_response_run(m, L, dt, n, "STRAINRATE", els)
    assert not np.any(R)
    assert np.abs(S).max() > 0
    for i, e in enumerate(els):
        Em, nu = m.mat_param[m.elem_mat[e]][:2]
        c1 = Em * (1 - nu) / ((1 - 2 * nu) * (1 + nu))
        c2 = Em * nu / ((1 - 2 * nu) * (1 + nu))
        c3 = Em / (2 * (1 + nu))
        if m.ndim == 2:
            C = np.array([[c1, c2, 0], [c2, c1, 0], [0, 0, c3]])
        else:
            C = np.zeros((6, 6))
            C[:3, :3] = c2
            np.fill_diagonal(C[:3, :3], c1)
            C[3:, 3:] = np.eye(3) * c3
        assert np.allclose(S[i], E[i] @ C.T, rtol=1e-12, atol=1e-12 * np.abs(S).max())
    for i, e in enumerate(els):
        Ke, _, _ = O.element_matrices(m, e)
        ue = U[m.totaldof[m.conn[e]].reshape(-1)]
        assert np.allclose(F[i], Ke @ ue, rtol=1e-10, atol=1e-10 * np.abs(F).max())
