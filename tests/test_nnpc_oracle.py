"""CPU checks of the learned preconditioner's network oracle: tap convention
and the analytic weight gradient against central finite differences."""
import numpy as np

from oracle import nnpc_oracle as N


def test_conv_tap_convention():
    # out[v] = sum W[t] in[v + s_t]: a unit input at node u reaches output v = u - s_t
    nz, ny, nx = 3, 4, 5
    x = np.zeros((1, nz, ny, nx))
    x[0, 1, 2, 3] = 1.0
    W = np.zeros((1, 1, 27))
    t = 9 * (1 + 1) + 3 * (-1 + 1) + (0 + 1)       # dz=+1, dy=-1, dx=0
    W[0, 0, t] = 2.0
    out = N.conv(x, W)
    assert out[0, 0, 3, 3] == 2.0 and np.count_nonzero(out) == 1


def test_weight_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nz, ny, nx = 3, 4, 5
    w = rng.standard_normal(N.num_weights()) * 0.2
    x = rng.standard_normal((3, nz, ny, nx))
    t = rng.standard_normal((3, nz, ny, nx))
    rho = rng.uniform(0.1, 1.0, (3, nz, ny, nx))
    mask = (rng.uniform(size=(3, nz, ny, nx)) > 0.2).astype(float)
    x *= mask
    t *= mask
    loss, g = N.loss_grad(w, x, t, rho, mask)
    assert np.isfinite(loss) and loss > 0
    idx = rng.choice(w.size, 40, replace=False)
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (N.loss_grad(wp, x, t, rho, mask)[0] - N.loss_grad(wm, x, t, rho, mask)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_zero_last_layer_is_jacobi():
    rng = np.random.default_rng(1)
    w = rng.standard_normal(N.num_weights())
    w[-16 * 3 * 27:] = 0.0
    r = rng.standard_normal((3, 2, 3, 4))
    mask = np.ones_like(r)
    assert np.array_equal(N.apply(w, r, np.ones_like(r), mask), r)
