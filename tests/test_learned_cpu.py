"""CPU checks of the learned path: the float64 reference gradient itself."""
import numpy as np

from cl_forward_gb300 import learned


def _data(n=64, seed=1):
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.normal(0, 1, (n, learned.N_IN))
    y = (rng.random(n) < 0.3).astype(np.float64)
    t = np.abs(rng.normal(0.1, 0.05, n)) * y
    return x, y, t


def test_reference_gradient_matches_finite_differences():
    w = learned.init_weights(3).astype(np.float64)
    x, y, t = _data()
    loss, g = learned.reference_loss_and_grad(w, x, y, t)
    rng = np.random.Generator(np.random.PCG64(0))
    for i in rng.choice(learned.N_PARAMS, 60, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        num = (learned.reference_loss_and_grad(wp, x, y, t)[0] - learned.reference_loss_and_grad(wm, x, y, t)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(num), (i, num, g[i])


def test_forward_shapes_and_layout():
    w = learned.init_weights(0)
    assert w.shape == (learned.N_PARAMS,) and w.dtype == np.float32
    out = learned.forward_np(w, np.zeros((5, learned.N_IN)))
    assert out.shape == (5, 2)
    A, a, B, b, C, c = learned.unpack(w)
    assert A.shape == (32, 10) and B.shape == (32, 32) and C.shape == (2, 32)
