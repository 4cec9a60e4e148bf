"""GPU tests of the learned preconditioner (svl_nm_train_preconditioner and
the flexible-CG solve): the device gradient against the numpy oracle, the
gain over Jacobi-PCG after training, and the Jacobi fallback."""
import numpy as np
import pytest

from oracle import nnpc_oracle as N
from svl_gb300 import NewmarkBeta, workloads
from svl_gb300 import _capi as capi
from tests.helpers import h8_box, rel_l2

pytestmark = pytest.mark.gpu


def test_device_gradient_matches_oracle(gpu):
    m, L, dt = h8_box(5, 4, 3, seed=2, nt=10)
    nm = NewmarkBeta(m, L, 10 * dt)
    assert nm.lattice() == (6, 5, 4)
    rho, mask = nm.nn_grids()
    rng = np.random.default_rng(0)
    w = (rng.standard_normal(N.num_weights()) * 0.15).astype(np.float32)
    nm.nn_weights(w)
    x = (rng.standard_normal(mask.shape) * mask).astype(np.float32)
    t = (rng.standard_normal(mask.shape) * mask).astype(np.float32)
    loss, g = nm.nn_loss_grad(x, t)
    nm.close()
    lo, go = N.loss_grad(w.astype(np.float64), x.astype(np.float64), t.astype(np.float64),
                         rho.astype(np.float64), mask.astype(np.float64))
    assert abs(loss - lo) <= 1e-5 * lo
    assert rel_l2(g, go) <= 1e-4


def test_tensor_core_forward_matches_fp32_and_oracle(gpu):
    # 10 x 18 x 11 node lattice: ragged 8 x 16 x 8 tiles on every axis
    m, L, dt = h8_box(9, 17, 10, seed=4, nt=10)
    nm = NewmarkBeta(m, L, 10 * dt)
    rho, mask = nm.nn_grids()
    rng = np.random.default_rng(5)
    w = (rng.standard_normal(N.num_weights()) * 0.2).astype(np.float32)
    nm.nn_weights(w)
    x = (rng.standard_normal(mask.shape) * mask).astype(np.float32)
    y32 = nm.nn_forward(x, path=0)
    ytc = nm.nn_forward(x, path=1)
    nm.close()
    yo = N.forward(w.astype(np.float64), x.astype(np.float64), rho.astype(np.float64))[4]
    assert np.abs(yo).max() > 0
    assert rel_l2(y32, yo) <= 1e-5
    assert rel_l2(ytc, yo) <= 3e-2        # BF16 operands, FP32 accumulation


def test_trained_preconditioner_cuts_iterations(gpu):
    m, L, dt = workloads.config4(16, 16, 16, nt=80)
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-8, precond=capi.SVL_PRECOND_JACOBI)
    b = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    a.Initialize()
    b.Initialize()
    a.run(1, 10)                      # Jacobi-PCG steps (the fallback reference count)
    b.run(1, 10)
    loss = a.train_preconditioner(11, solve_steps=0, n_synthetic=200, iters=800, batch=4, seed=1)
    assert np.isfinite(loss) and loss < 0.2
    it_a0, _, _ = a.stats()
    it_b0, _, _ = b.stats()
    ha = a.run(11, 10, history=True)
    hb = b.run(11, 10, history=True)
    it_a = a.stats()[0] - it_a0
    it_b = b.stats()[0] - it_b0
    solves, fallbacks, jref = a.precond_stats()
    _, _, res = a.stats()
    a.close()
    b.close()
    assert solves == 10 and fallbacks == 0
    assert res <= 1e-8
    assert it_a < 0.6 * it_b, (it_a, it_b)
    assert rel_l2(ha, hb) <= 1e-5


def test_training_on_crops_cuts_iterations(gpu):
    """Training on random 13^3 windows of the pairs (loss masked inside window
    faces interior to the lattice) gives a preconditioner that still cuts the
    iterations against Jacobi-PCG and solves to the same tolerance."""
    m, L, dt = workloads.config4(24, 24, 24, nt=60)
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    b = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    a.Initialize()
    b.Initialize()
    a.run(1, 8)
    b.run(1, 8)
    loss = a.train_preconditioner(9, solve_steps=0, n_synthetic=200, iters=600, batch=8, seed=1, crop=13)
    assert np.isfinite(loss)
    it_a0, it_b0 = a.stats()[0], b.stats()[0]
    ha = a.run(9, 8, history=True)
    hb = b.run(9, 8, history=True)
    it_a, it_b = a.stats()[0] - it_a0, b.stats()[0] - it_b0
    solves, fallbacks, _ = a.precond_stats()
    res = a.stats()[2]
    a.close()
    b.close()
    assert solves == 8 and res <= 1e-8
    assert it_a < 0.75 * it_b, (it_a, it_b)
    assert rel_l2(ha, hb) <= 1e-5


def test_cuda_core_and_tensor_core_paths_both_converge(gpu):
    m, L, dt = workloads.config4(12, 12, 12, nt=40)
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    a.Initialize()
    a.run(1, 5)
    a.train_preconditioner(6, solve_steps=0, n_synthetic=100, iters=300, batch=4, seed=3)
    U0 = [a.GetDisplacements(), a.GetVelocities(), a.GetAccelerations()]
    its = []
    res = []
    for path in (0, 1):
        a.Initialize(*U0)
        a.nn_set_path(path)
        i0 = a.stats()[0]
        a.run(6, 5)
        its.append(a.stats()[0] - i0)
        res.append(a.stats()[2])
    a.close()
    assert max(res) <= 1e-8
    assert abs(its[1] - its[0]) <= 0.25 * its[0] + 2, its


def test_training_from_solve_iterates_runs(gpu):
    """Pairs from the CG iterates of the first steps (e_k = x* - x_k) feed the
    same training; the steps they come from advance the state."""
    m, L, dt = workloads.config4(10, 10, 10, nt=40)
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    b = NewmarkBeta(m, L, dt, pcg_tol=1e-8)
    a.Initialize()
    b.Initialize()
    loss = a.train_preconditioner(1, solve_steps=4, record_every=3, n_synthetic=20, iters=100, batch=2, seed=2)
    b.run(1, 4)
    assert np.isfinite(loss)
    assert rel_l2(a.GetDisplacements(), b.GetDisplacements()) == 0.0     # same Jacobi solves
    ha = a.run(5, 3, history=True)
    hb = b.run(5, 3, history=True)
    a.close()
    b.close()
    assert rel_l2(ha, hb) <= 1e-6


def test_bad_network_falls_back_to_jacobi(gpu):
    m, L, dt = workloads.config4(10, 9, 8, nt=40)
    a = NewmarkBeta(m, L, dt, pcg_tol=1e-9)
    b = NewmarkBeta(m, L, dt, pcg_tol=1e-9)
    a.Initialize()
    b.Initialize()
    a.run(1, 3)                       # sets the Jacobi reference count
    b.run(1, 3)
    rng = np.random.default_rng(3)
    a.nn_weights(rng.standard_normal(N.num_weights()).astype(np.float32) * 3.0)
    a.set_preconditioner(capi.SVL_PRECOND_LEARNED)
    ha = a.run(4, 5, history=True)
    hb = b.run(4, 5, history=True)
    solves, fallbacks, _ = a.precond_stats()
    _, _, res = a.stats()
    a.close()
    b.close()
    assert solves == 5 and fallbacks >= 1
    assert res <= 1e-9
    assert rel_l2(ha, hb) <= 1e-6
