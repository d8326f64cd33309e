"""The CPU restatement of the warm-start MLP: its backward pass against central
finite differences of its own float64 forward (no BF16 rounding)."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo


def _case(seed=0, P=7, slots=(0, 3, 7)):
    rng = np.random.default_rng(seed)
    p = mo.init_params(seed, film_scale=0.2).astype(np.float64)
    xy = rng.uniform(0, 1, (P, 2))
    cond = rng.uniform(-1, 1, (len(slots) - 1, 2))
    target = rng.uniform(-1, 1, (P, 3))
    return p, xy, np.array(slots), cond, target


def test_layout_size():
    _, total = mo.offsets()
    assert total == 4 * (256 * 7) + 256 * 64 + 3 * 256 * 256 + 3 * 256 + 3


def test_backward_matches_finite_differences():
    p, xy, sp, cond, target = _case()
    _, g = mo.loss_grad(p, xy, sp, cond, target, use_bf16=False)
    off, _ = mo.offsets()
    rng = np.random.default_rng(1)
    h = 1e-6
    for key, (o, size) in off.items():
        for idx in rng.choice(size, size=min(size, 3), replace=False):
            e = o + idx
            pp, pm = p.copy(), p.copy()
            pp[e] += h
            pm[e] -= h
            lp, _ = mo.loss_grad(pp, xy, sp, cond, target, use_bf16=False)
            lm, _ = mo.loss_grad(pm, xy, sp, cond, target, use_bf16=False)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[e]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (key, idx, fd, g[e])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 1e-30])
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125   # ties to even, then round up
    assert abs(r[3] + 3.140625) < 1e-12 and r[4] == 0.0
