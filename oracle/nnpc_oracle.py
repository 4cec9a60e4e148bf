"""CPU oracle of the learned preconditioner's network (test infrastructure).

A numpy restatement, in float64, of the 4-layer 3x3x3 convolutional network
the library trains and applies on the node lattice: the forward pass, the
training loss and its weight gradient.  The GPU kernels' gradients are checked
against it, and it is checked against central finite differences.  The
network has no counterpart in the reference; its conventions are those of
include/svl_gb300.h (svl_nm_train_preconditioner):

  grids     [C][nz][ny][nx], node index x + nx (y + ny z)
  weights   layer by layer, [cout][cin][27], tap t = 9 (dz+1) + 3 (dy+1) + (dx+1),
            out[co][v] = sum_{ci,t} W[co][ci][t] in[ci][v + (dx, dy, dz)]  (zero outside)
  layers    6 -> 16 (relu) -> 16 (relu) -> 16 (relu) -> 3
  features  [x ; rho * x]
  loss      sum(((x + y - t) * mask)^2)
"""
from __future__ import annotations

import numpy as np

LAYERS = [(6, 16), (16, 16), (16, 16), (16, 3)]
TAPS = 27


def num_weights():
    return sum(ci * co * TAPS for ci, co in LAYERS)


def split(w):
    out, off = [], 0
    for ci, co in LAYERS:
        n = ci * co * TAPS
        out.append(np.asarray(w[off:off + n], dtype=np.float64).reshape(co, ci, TAPS))
        off += n
    return out


def _taps():
    for t in range(TAPS):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def conv(x, W):
    """x [cin, nz, ny, nx], W [cout, cin, 27] -> [cout, nz, ny, nx]."""
    cin, nz, ny, nx = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    out = np.zeros((W.shape[0], nz, ny, nx))
    for t, dz, dy, dx in _taps():
        sh = xp[:, 1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
        out += np.tensordot(W[:, :, t], sh, axes=(1, 0))
    return out


def conv_grads(x, W, g):
    """Weight and input gradients of conv(x, W) for output gradient g."""
    cin, nz, ny, nx = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    dW = np.zeros_like(W)
    dxp = np.zeros_like(xp)
    for t, dz, dy, dx in _taps():
        sl = (slice(None), slice(1 + dz, 1 + dz + nz), slice(1 + dy, 1 + dy + ny), slice(1 + dx, 1 + dx + nx))
        dW[:, :, t] = np.tensordot(g, xp[sl], axes=([1, 2, 3], [1, 2, 3]))
        dxp[sl] += np.tensordot(W[:, :, t].T, g, axes=(1, 0))
    return dW, dxp[:, 1:-1, 1:-1, 1:-1]


def forward(w, x, rho):
    Ws = split(w)
    a = [np.concatenate([x, rho * x], 0)]
    for i, W in enumerate(Ws):
        z = conv(a[-1], W)
        a.append(np.maximum(z, 0.0) if i < 3 else z)
    return a          # a[0] features, a[1..3] hidden, a[4] = y


def loss_grad(w, x, t, rho, mask):
    """(loss, dloss/dw) of one sample."""
    Ws = split(w)
    a = forward(w, x, rho)
    d = (x + a[4] - t) * mask
    loss = float(np.sum(d * d))
    g = 2.0 * d * mask
    grads = [None] * 4
    for i in range(3, -1, -1):
        dW, gin = conv_grads(a[i], Ws[i], g)
        grads[i] = dW
        if i > 0:
            g = gin * (a[i] > 0)
    return loss, np.concatenate([gw.ravel() for gw in grads])


def apply(w, r_hat, rho, mask):
    """z_hat = (r_hat + net(r_hat)) * mask."""
    return (r_hat + forward(w, r_hat, rho)[4]) * mask
