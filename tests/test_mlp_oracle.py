"""CPU checks of the learned-MTS network oracle: the backward pass is the exact
gradient of the loss (central finite differences in FP64), and the bfloat16
rounding helper rounds to nearest even."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_nearest_even():
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert mo.bf16(1.0 + 2.0 ** -8) == 1.0
    # 1 + 3*2^-8 is halfway between 1+2^-7 and 1+2^-6: ties go to 1+2^-6
    assert mo.bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6
    assert mo.bf16(-2.5) == -2.5
    x = np.random.default_rng(0).normal(size=1000)
    r = mo.bf16(x)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8 + 1e-300)


def test_pack_roundtrip():
    p = mo.initial_params(3)
    assert p.size == mo.NPARAM == 51 * 128 + 128 + 128 * 128 + 128 + 128 * 3 + 3
    assert np.array_equal(mo.pack(mo.unpack(p)), p)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(11)
    x = rng.normal(size=(24, mo.NIN))
    t = rng.normal(size=(24, 3)) * 0.3
    p = mo.initial_params(5, out_gain=1.0)
    p[mo.NIN * mo.NH: mo.NIN * mo.NH + mo.NH] = rng.normal(size=mo.NH) * 0.1  # non-zero b1
    loss, g, _ = mo.loss_and_grad(x, t, p, bf16_points=False)
    idx = np.concatenate([rng.choice(mo.NPARAM, 60, replace=False), np.arange(mo.NPARAM - 3, mo.NPARAM)])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp = mo.loss_and_grad(x, t, pp, bf16_points=False)[0]
        lm = mo.loss_and_grad(x, t, pm, bf16_points=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-7 * max(1.0, abs(g[k])) + 1e-9, (k, fd, g[k])
    assert loss > 0


def test_bf16_points_change_little():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(64, mo.NIN))
    t = rng.normal(size=(64, 3))
    p = mo.initial_params(1, out_gain=1.0)
    _, g64, y64 = mo.loss_and_grad(x, t, p, bf16_points=False)
    _, gb, yb = mo.loss_and_grad(x, t, p, bf16_points=True)
    assert np.linalg.norm(yb - y64) <= 0.05 * np.linalg.norm(y64)
    assert np.dot(gb, g64) / (np.linalg.norm(gb) * np.linalg.norm(g64)) > 0.99
