"""Learned multiple-time-step form on the GPU.

- the training kernel's forward, loss and gradients match the CPU oracle
  (oracle/mlp_oracle.py, FP64 with the same bfloat16 rounding points);
- the tensor-core inference kernel matches the oracle forward;
- an online-trained MTS run (impulse split: coarse-grid force plus the network's
  correction on the inner steps) matches the reciprocal force better than the
  coarse-grid force alone and than the previous full step's force held fixed,
  the ablations;
- the check falls back to plain SPME when the bound cannot be met.
"""
import numpy as np
import pytest

from dlpoly_gb300 import systems
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _data(nb, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(nb, mo.NIN)).astype(np.float32)
    t = (0.3 * rng.normal(size=(nb, 3))).astype(np.float32)
    p = mo.initial_params(seed, out_gain=1.0).astype(np.float32)
    p[mo.NIN * mo.NH: mo.NIN * mo.NH + mo.NH] = 0.1 * rng.normal(size=mo.NH)  # non-zero b1
    return x, t, p


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.fixture()
def ctx(gpu_lib):
    gpu_lib.init(systems.nacl_melt(16), precision=1)
    return gpu_lib


def test_param_count(ctx):
    assert ctx.mlp_param_count() == mo.NPARAM


@pytest.mark.parametrize("nb", [1, 37, 2048])
def test_training_gradients_match_oracle(ctx, nb):
    x, t, p = _data(nb, 3 + nb)
    loss, grad, y = ctx.mlp_train_eval(x, t, p)
    lo, go, yo = mo.loss_and_grad(x, t, p.astype(np.float64), bf16_points=True)
    assert loss == pytest.approx(lo, rel=2e-3)
    assert _rel(y, yo) <= 1e-3
    assert _rel(grad, go) <= 2e-3
    # every block of the parameter vector, not only the dominant one
    o = 0
    for name, shape in mo.SHAPES:
        n = int(np.prod(shape))
        assert _rel(grad[o:o + n], go[o:o + n]) <= 5e-3, name
        o += n


def test_training_is_deterministic(ctx):
    x, t, p = _data(1000, 9)
    a = ctx.mlp_train_eval(x, t, p)
    b = ctx.mlp_train_eval(x, t, p)
    assert a[0] == b[0] and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("nb", [1, 63, 64, 65, 5000])
def test_inference_matches_oracle(ctx, nb):
    x, _, p = _data(nb, 100 + nb)
    y = ctx.mlp_infer_eval(x, p)
    yo, _ = mo.forward(x, p.astype(np.float64), bf16_points=True)
    assert _rel(y, yo) <= 1e-3


def _mts_run(lib, s, k, train, steps, no_network):
    lib.init(s, precision=1)
    lib.start()
    lib.mts_ablation(no_network)
    lib.mts_config(k, 1.0, train)  # a loose bound: measure the error, never fall back
    st = lib.md_vv(steps)
    ms = lib.mts_stats()
    lib.mts_ablation(False)
    return st, ms


def test_mts_ablation(gpu_lib):
    """Every check measures the same step three ways against full SPME: the inner
    steps' force S (coarse grid plus the network's correction), the coarse-grid
    force alone, and the previous full step's force held unchanged.  The network
    must beat both ablations."""
    s = systems.nacl_melt(16)
    k, train, steps = 4, 400, 600
    st, ms = _mts_run(gpu_lib, s, k, train, steps, no_network=False)
    # schedule: SPME every step while training, then every k-th step
    full = [x.mts_full for x in st]
    assert all(full[:train])
    assert sum(full[train:]) == (steps - train) // k
    assert ms["n_inner"] == (steps - train) - (steps - train) // k
    assert ms["opt_steps"] > 0
    assert ms["n_checked"] >= 10
    assert ms["err_no_network"] < 0.1 * ms["err_stale"], ms
    assert ms["last_err"] < ms["err_no_network"], ms
    # the same schedule with the network switched off
    st0, ms0 = _mts_run(gpu_lib, s, k, train, steps, no_network=True)
    assert ms0["opt_steps"] == 0
    assert ms0["last_err"] == pytest.approx(ms0["err_no_network"], rel=1e-6)


def test_mts_fallback_when_bound_missed(gpu_lib):
    """A bound no surrogate meets keeps plain SPME on every step after training."""
    s = systems.nacl_melt(16)
    gpu_lib.init(s, precision=1)
    gpu_lib.start()
    gpu_lib.mts_config(4, 1e-12, 20)
    st = gpu_lib.md_vv(60)
    ms = gpu_lib.mts_stats()
    assert ms["in_fallback"] == 1.0 and ms["n_fallback"] >= 1
    # after the first check every step runs SPME
    assert ms["n_inner"] <= 3
    assert all(x.mts_full for x in st[24:])


def test_mts_requires_mixed(gpu_lib):
    from dlpoly_gb300.binding import PathError

    gpu_lib.init(systems.nacl_melt(16), precision=0)
    with pytest.raises(PathError):
        gpu_lib.mts_config(4, 1e-4, 10)


@pytest.mark.parametrize("nb", [1, 127, 128, 129, 70000])
def test_tcgen05_inference_matches_mma_sync_kernel(ctx, monkeypatch, nb):
    """The tcgen05 inference kernel (operands in shared memory, FP32 accumulators in tensor
    memory) against the mma.sync kernel on the same inputs and weights: both round the
    same hidden activations to BF16 and accumulate in FP32, so they agree to the order of
    the FP32 sums (a BF16 rounding flip of a hidden value at most), and both against the
    oracle forward."""
    x, _, p = _data(nb, 300 + nb)
    monkeypatch.setenv("GB_MLP_TC", "0")
    y_sync = ctx.mlp_infer_eval(x, p)
    monkeypatch.delenv("GB_MLP_TC", raising=False)
    y_tc = ctx.mlp_infer_eval(x, p)
    yo, _ = mo.forward(x, p.astype(np.float64), bf16_points=True)
    assert _rel(y_tc, yo) <= 1e-3
    assert _rel(y_tc, y_sync) <= 1e-3


@pytest.mark.parametrize("nb", [1, 129, 8192])
def test_tcgen05_training_matches_cuda_core_kernel(ctx, monkeypatch, nb):
    """The tcgen05 training kernel (the three forward and five backward products of a
    128-atom tile on the tensor cores, FP32 accumulators in tensor memory) against the
    CUDA-core training kernel (GB_MLP_TC=0) on the same batch: the same BF16 rounding
    points and FP32 accumulation, so loss, outputs and every gradient block agree to the
    order of the FP32 sums, and both against the FP64 oracle; the tensor-core step is
    deterministic."""
    x, t, p = _data(nb, 500 + nb)
    monkeypatch.setenv("GB_MLP_TC", "0")
    lc, gc, yc = ctx.mlp_train_eval(x, t, p)
    monkeypatch.delenv("GB_MLP_TC", raising=False)
    lt, gt, yt = ctx.mlp_train_eval(x, t, p)
    lo, go, yo = mo.loss_and_grad(x, t, p.astype(np.float64), bf16_points=True)
    assert lt == pytest.approx(lo, rel=2e-3) and lt == pytest.approx(lc, rel=2e-3)
    assert _rel(yt, yo) <= 1e-3 and _rel(yt, yc) <= 1e-3
    assert _rel(gt, go) <= 2e-3 and _rel(gt, gc) <= 2e-3
    o = 0
    for name, shape in mo.SHAPES:
        n = int(np.prod(shape))
        assert _rel(gt[o:o + n], go[o:o + n]) <= 5e-3, name
        o += n
    again = ctx.mlp_train_eval(x, t, p)
    assert again[0] == lt and np.array_equal(again[1], gt)
