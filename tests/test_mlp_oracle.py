"""The CPU statement of the surrogate network (oracle/mlp_oracle.py), the
checker of the GPU training kernels: its backward pass against central finite
differences of its forward pass in FP64, on a few parameters of every block."""
import numpy as np

import mlp_oracle as M


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(7)
    flat = rng.normal(0.0, 0.08, M.NUM_PARAMS)
    x = rng.normal(0.0, 0.5, (16, M.N_IN))
    t = rng.normal(0.0, 0.1, (16, M.N_USED))
    loss, g = M.loss_grad(flat, x, t, rb=False)
    assert loss > 0
    off = 0
    for name, shape in M.SHAPES:
        n = int(np.prod(shape))
        for k in rng.choice(n, 3, replace=False):
            i = off + int(k)
            h = 1e-6
            fp = flat.copy()
            fp[i] += h
            fm = flat.copy()
            fm[i] -= h
            num = (M.loss_grad(fp, x, t, rb=False)[0] - M.loss_grad(fm, x, t, rb=False)[0]) / (2 * h)
            assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(num)) + 1e-9, (name, k, num, g[i])
        off += n


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], dtype=np.float32)
    got = M.bf16(v)
    assert got[0] == 1.0 and got[1] == 1.0  # halfway rounds to even
    assert got[2] == 1.0 + 2 ** -7
    assert got[3] == -2.5
    assert abs(got[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8
