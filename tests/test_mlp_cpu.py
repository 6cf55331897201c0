"""CPU checks of the FP64 surrogate oracle: analytic gradients against
central finite differences (plain float64 network)."""
import numpy as np

from oracle import mlp_oracle as mo
from phd_gb300.surrogate import he_init


def test_oracle_gradients_match_finite_differences():
    rng = np.random.Generator(np.random.PCG64(3))
    W, b = he_init(5)
    W = [w.astype(np.float64) * 0.5 for w in W]
    b = [x.astype(np.float64) + 0.01 * rng.standard_normal(x.shape) for x in b]
    x = rng.standard_normal((8, 12))
    t = rng.standard_normal((8, 10))
    loss, gW, gb = mo.loss_and_grads(W, b, x, t, rounding=False)
    eps = 1e-6
    for l, (i, j) in [(0, (3, 7)), (1, (10, 20)), (2, (100, 5)), (3, (255, 200)), (4, (17, 9))]:
        Wp = [w.copy() for w in W]; Wp[l][i, j] += eps
        Wm = [w.copy() for w in W]; Wm[l][i, j] -= eps
        fp = float(((mo.forward(Wp, b, x, False)[0] - t) ** 2).mean())
        fm = float(((mo.forward(Wm, b, x, False)[0] - t) ** 2).mean())
        fd = (fp - fm) / (2 * eps)
        assert abs(fd - gW[l][i, j]) <= 1e-6 * max(1.0, abs(fd)), (l, fd, gW[l][i, j])
    for l, j in [(0, 11), (3, 128), (4, 2)]:
        bp = [v.copy() for v in b]; bp[l][j] += eps
        bm = [v.copy() for v in b]; bm[l][j] -= eps
        fd = (float(((mo.forward(W, bp, x, False)[0] - t) ** 2).mean()) -
              float(((mo.forward(W, bm, x, False)[0] - t) ** 2).mean())) / (2 * eps)
        assert abs(fd - gb[l][j]) <= 1e-6 * max(1.0, abs(fd))


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159], dtype=np.float32)
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
