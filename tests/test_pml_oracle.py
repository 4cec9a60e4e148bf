"""CPU checks of the PML element matrices in the oracle (PML2DQuad4,
PML3DHexa8): symmetry, the structure the reference's formulas give (no
displacement-stress coupling in M, rho-weighted displacement block), and
the limits R -> 1 (no stretching: a = 1, b = 0)."""
import numpy as np

from oracle import oracle as O


def hexa(h=2.0, jitter=0.0, seed=0):
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    return (base + jitter * rng.uniform(-1, 1, base.shape)) * h


def quad(h=1.0, jitter=0.0, seed=0):
    rng = np.random.default_rng(seed)
    base = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    return (base + jitter * rng.uniform(-1, 1, base.shape)) * h


PAR3 = np.array([2.0, 10.0, 1e-3, -5.0, -5.0, -5.0, 0.0, 0.0, -1.0])   # bottom layer, n = (0, 0, -1)
PAR2 = np.array([2.0, 10.0, 1e-3, 0.0, 5.0, 0.0, -1.0])                 # n = (0, -1)


def _pml3(jit=0.1):
    X = hexa(jitter=jit) + np.array([0.0, 0.0, -8.0])     # inside the layer: z below z0
    return O.pml_matrices(3, X, 2.0e8, 0.3, 2000.0, PAR3)


def test_pml3d_matrices_are_symmetric_and_structured():
    M, Cm, K, G = _pml3()
    for A in (M, Cm, K, G):
        assert np.allclose(A, A.T, rtol=0, atol=1e-12 * np.abs(A).max())
    disp = np.array([d % 9 < 3 for d in range(72)])
    assert np.count_nonzero(M[np.ix_(disp, ~disp)]) == 0          # no coupling in M
    assert np.count_nonzero(K[np.ix_(disp, ~disp)]) > 0
    assert np.all(np.diag(M)[disp] > 0) and np.all(np.diag(M)[~disp] < 0)
    # displacement block of M sums to rho * integral of ax ay az >= rho * volume per direction
    Mu = O.pml_matrices(3, hexa() + np.array([0.0, 0.0, -8.0]), 2.0e8, 0.3, 2000.0, PAR3)[0]
    assert Mu[np.ix_(disp, disp)].sum() > 3 * 2000.0 * 8.0


def test_pml_without_stretching_reduces_to_plain_blocks():
    par = PAR3.copy()
    par[2] = 1.0                       # R = 1: a = 1, b = 0 everywhere
    X = hexa(jitter=0.0)
    M, Cm, K, G = O.pml_matrices(3, X, 2.0e8, 0.3, 2000.0, par)
    assert np.abs(K).max() == 0.0 and np.abs(G).max() == 0.0
    disp = np.array([d % 9 < 3 for d in range(72)])
    # consistent mass of the unit-stretch element: rho * V per direction
    assert np.isclose(M[np.ix_(disp, disp)].sum(), 3 * 2000.0 * 8.0)
    M2, C2, K2, G2 = O.pml_matrices(2, quad(), 2.0e8, 0.3, 2000.0, np.array([2.0, 10.0, 1.0, 0, 0, 0, 1.0]), t=1.0)
    assert np.abs(K2).max() == 0.0 and np.abs(G2).max() == 0.0


def test_pml2d_matrices_are_symmetric():
    X = quad(jitter=0.1) + np.array([0.0, -8.0])
    M, Cm, K, G = O.pml_matrices(2, X, 2.0e8, 0.25, 2000.0, PAR2, t=1.0)
    for A in (M, Cm, K):
        assert np.allclose(A, A.T, rtol=0, atol=1e-12 * np.abs(A).max())
    assert np.abs(G).max() == 0.0
