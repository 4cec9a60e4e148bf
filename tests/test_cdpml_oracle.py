"""The oracle of the explicit central difference with PML layers (the
library's staggered scheme; CDPml in oracle/svl_oracle.cpp), on the CPU.

* Without PML elements it is the plain central difference: bitwise equal to
  the central-difference oracle (the reference's CentralDifference).
* It absorbs: a Ricker pulse in a box with PML layers on the sides and the
  bottom leaves the interior (displacements down by more than 1e3 from
  their peak), while the same box with fixed faces keeps ringing.
* It is stable at half the lumped-mass step limit over thousands of steps,
  in 2D (PML2DQuad4) and 3D (PML3DHexa8).
"""
import numpy as np

from oracle import oracle as O
from svl_gb300 import _capi as capi
from svl_gb300.model import Model
from tests.helpers import h8_box, pml_box, q4_box


def _interior_udofs(m):
    pn = np.zeros(m.nnode, bool)
    pn[m.conn[m.elem_pml == 1].ravel()] = True
    return m.totaldof[~pn, :m.ndim].ravel()


def test_without_pml_it_is_the_plain_central_difference():
    for m, L, dt in (q4_box(16, 8, nt=150), h8_box(6, 5, 4, nt=150)):
        h0, U0, V0, A0 = O.cd_run(m, L, dt, 150, mode=0)
        h1, U1, V1, A1, _ = O.cdpml_run(m, L, dt, 150)
        assert np.abs(h0).max() > 0
        assert np.array_equal(h0, h1) and np.array_equal(V0, V1) and np.array_equal(A0, A1)


def _fixed_box(m):
    """The same mesh with every element solid and the outer faces fixed."""
    X = m.coords
    nd = m.ndim
    vert = nd - 1
    ext = X.max(axis=0)
    outer = np.zeros(m.nnode, bool)
    for d in range(nd):
        outer |= np.isclose(X[:, d], 0.0) if d == vert else (np.isclose(X[:, d], 0.0) | np.isclose(X[:, d], ext[d]))
    tdof = np.arange(m.nnode * nd, dtype=np.int32).reshape(m.nnode, nd)
    fdof = -np.ones((m.nnode, nd), np.int32)
    f = 0
    for n in range(m.nnode):
        for j in range(nd):
            if not outer[n]:
                fdof[n, j] = f
                f += 1
    return Model(ndim=nd, coords=X, totaldof=tdof, freedof=fdof, conn=m.conn, elem_type=m.elem_type,
                 elem_mat=m.elem_mat, mat_type=m.mat_type, mat_param=m.mat_param, lumped=True)


def test_pml_absorbs_in_2d_and_the_fixed_box_does_not():
    nt = 3000
    m, L, dt = pml_box(2, (30, 20), npml=6, nt=nt, dt_factor=0.5)
    h, *_ = O.cdpml_run(m, L, dt, nt)
    assert np.isfinite(h).all()
    ud = _interior_udofs(m)
    amp = np.abs(h[:, ud]).max(axis=1)
    peak = amp.max()
    assert amp[-300:].max() < 1e-3 * peak
    # the same pulse in the fixed box
    mf = _fixed_box(m)
    c = L.force_dof[0]
    node = int(np.flatnonzero(m.totaldof == c)[0] // m.totaldof.shape[1])
    from svl_gb300.model import Loads
    Lf = Loads()
    s = Lf.add_series(L.series[0])
    Lf.add_point_load(mf, node, (0.0, -L.force_coef[0]), s)
    hf, *_ = O.cd_run(mf, Lf, dt, nt, mode=1)
    pn = np.zeros(m.nnode, bool)
    pn[m.conn[m.elem_pml == 1].ravel()] = True
    udf = mf.totaldof[~pn].ravel()
    ampf = np.abs(hf[:, udf]).max(axis=1)
    assert ampf[-300:].max() > 0.05 * ampf.max()


def test_pml_absorbs_in_3d():
    nt = 300
    m, L, dt = pml_box(3, (6, 6, 5), npml=3, nt=nt, dt_factor=0.5, f0=10.0)
    h, U, V, A, Ub = O.cdpml_run(m, L, dt, nt)
    assert np.isfinite(h).all()
    ud = _interior_udofs(m)
    amp = np.abs(h[:, ud]).max(axis=1)
    assert amp[-30:].max() < 2e-2 * amp.max()
    # stress dofs carry the outgoing wave, the history integral is filled
    sd = np.array([m.totaldof[n, j] for n in range(m.nnode) for j in range(3, m.node_ndof[n])])
    assert np.abs(h[:, sd]).max() > 0 and np.abs(Ub[sd]).max() > 0
