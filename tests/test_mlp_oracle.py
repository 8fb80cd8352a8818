"""The MLP oracle's back-propagation against central finite differences (FP64, no BF16
rounding), and the BF16 rounding helper against exact round-to-nearest-even."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import mlp_ref as M  # noqa: E402


def random_params(rng):
    p = rng.normal(0, 0.3, M.NPARAM)
    d = M.unpack(p)
    d["scale"] = np.abs(d["scale"]) + 0.5
    d["oscale"] = np.abs(d["oscale"]) + 0.5
    return M.pack(d)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = random_params(rng)
    X = rng.normal(0, 1, (37, M.IN))
    T = rng.normal(0, 1, (37, M.OUT))
    _, loss, g = M.forward_backward(p, X, T, rounding=False)
    assert g.shape == (M.NW,)
    idx = rng.choice(M.NW, 300, replace=False)
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.forward_backward(pp, X, T, rounding=False)[1] - M.forward_backward(pm, X, T, rounding=False)[1]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.14159, 1e-3], np.float32)
    r = M.bf16(x)
    # representable values stay, halfway cases go to the even mantissa
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0 + 4 * 2 ** -8) and r[3] == 1.0 and r[4] == -2.5
    for v, q in zip(x, r):
        assert abs(float(q) - float(v)) <= abs(float(v)) * 2 ** -8
        assert (np.float32(q).view(np.uint32) & 0xFFFF) == 0
