"""The learned part's MLP: CPU oracle pinned by finite differences, GPU
forward / gradient against the oracle, training on the GPU.

Tolerances: the oracle rounds at the same points as the kernels (BF16
inputs, weights and stored activations, FP32 accumulation), so outputs agree
to FP32 summation order -- except where a different order flips a BF16
rounding of an activation (one BF16 ulp, 2^-8 relative, on that element).
Outputs are compared at 1e-3 and gradients at 5e-3 relative in norm.
"""
import numpy as np
import pytest

from oracle import mlp_ref as R


def _data(rows, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((rows, R.IN)).astype(np.float32)
    x[:, 9:] = 0.0
    t = rng.standard_normal((rows, R.OUT)).astype(np.float32)
    w = rng.uniform(0.0, 1.0, (rows, R.OUT)).astype(np.float32)
    return x, t, w


def test_oracle_gradient_matches_finite_differences():
    p = R.init_params(1).astype(np.float64)
    x, t, w = _data(40, 2)
    _, g = R.loss_grad(p, x, t, w, exact=True)
    rng = np.random.default_rng(3)
    idx = np.concatenate([rng.choice(np.arange(R.OFF_W1, R.OFF_B1), 6), rng.choice(np.arange(R.OFF_B1, R.OFF_W2), 3),
                          rng.choice(np.arange(R.OFF_W2, R.OFF_B2), 6), rng.choice(np.arange(R.OFF_W3, R.OFF_B3), 4),
                          np.arange(R.OFF_B3, R.OFF_MEAN)])
    h = 1e-6
    for j in idx:
        pp, pm = p.copy(), p.copy()
        pp[j] += h
        pm[j] -= h
        fd = (R.loss_grad(pp, x, t, w, exact=True)[0] - R.loss_grad(pm, x, t, w, exact=True)[0]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-6 * max(1.0, abs(fd)), (j, fd, g[j])


def test_oracle_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    v = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-8, 8, 10000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.005859375, 65504.0]]).astype(np.float32)
    ref = torch.from_numpy(v).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(R.bf16(v), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [1000, 37, 4096 + 5])
def test_gpu_forward_matches_oracle(rows):
    torch = pytest.importorskip("torch")
    from help_gb300 import learned

    x, _, _ = _data(rows, 7)
    p = R.init_params(4)
    p[R.OFF_B1:R.OFF_W2] = 0.1
    with_model = learned.Mlp(0, p)
    xb = torch.from_numpy(learned.bf16_bits(x).view(np.int16)).cuda()
    out = with_model.forward(xb, rows).cpu().numpy()
    ref, _, _ = R.forward(p, x)
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 1e-3, err
    with_model.close()


@pytest.mark.gpu
def test_gpu_inference_forward_matches_training_forward():
    """The inference forward (tcgen05, TMEM accumulators, several 128-row
    tiles per CTA and a ragged last tile) against the oracle element-wise and
    against the training forward (mma.sync) through the loss both give."""
    torch = pytest.importorskip("torch")
    from help_gb300 import learned

    rows = 300_001
    x, t, w = _data(rows, 12)
    p = R.init_params(13)
    m = learned.Mlp(0, p)
    xb = torch.from_numpy(learned.bf16_bits(x).view(np.int16)).cuda()
    out = m.forward(xb, rows).cpu().numpy().astype(np.float64)
    ref = R.forward(p, x)[0]
    assert np.isfinite(out).all()
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-3
    assert np.abs(out - ref).max() < 2e-2 * np.abs(ref).max()
    loss_train, _ = m.loss_grad(xb, torch.from_numpy(t).cuda(), torch.from_numpy(w).cuda(), rows)
    loss_inf = float(np.sum(w * (out - t) ** 2) / np.sum(w))
    assert abs(loss_inf - loss_train) <= 1e-5 * abs(loss_train), (loss_inf, loss_train)
    m.close()


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [640, 37])
def test_gpu_gradient_matches_oracle(rows):
    torch = pytest.importorskip("torch")
    from help_gb300 import learned

    x, t, w = _data(rows, 8)
    p = R.init_params(5)
    m = learned.Mlp(0, p)
    xb = torch.from_numpy(learned.bf16_bits(x).view(np.int16)).cuda()
    loss, g = m.loss_grad(xb, torch.from_numpy(t).cuda(), torch.from_numpy(w).cuda(), rows)
    lref, gref = R.loss_grad(p, x, t, w)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    for a, b in ((R.OFF_W1, R.OFF_B1), (R.OFF_B1, R.OFF_W2), (R.OFF_W2, R.OFF_B2), (R.OFF_B2, R.OFF_W3),
                 (R.OFF_W3, R.OFF_B3), (R.OFF_B3, R.OFF_MEAN)):
        err = np.linalg.norm(g[a:b] - gref[a:b]) / max(np.linalg.norm(gref[a:b]), 1e-30)
        assert err < 5e-3, (a, b, err)
    m.close()


@pytest.mark.gpu
def test_gpu_training_fits_a_teacher():
    """Adam with the library's kernels fits targets made by another MLP."""
    torch = pytest.importorskip("torch")
    from help_gb300 import learned

    rows = 8192
    x, _, _ = _data(rows, 9)
    teacher = R.init_params(10)
    t = R.forward(teacher, x)[0].astype(np.float32)
    w = np.ones_like(t)
    m = learned.Mlp(0, R.init_params(11))
    xb = torch.from_numpy(learned.bf16_bits(x).view(np.int16)).cuda()
    tt, ww = torch.from_numpy(t).cuda(), torch.from_numpy(w).cuda()
    first = m.train_step(xb, tt, ww, rows, 3e-3)
    for _ in range(300):
        last = m.train_step(xb, tt, ww, rows, 3e-3)
    assert last < 0.1 * first, (first, last)
    # the parameters read back give the same loss in the oracle
    lref, _ = R.loss_grad(m.get_params(), x, t, w)
    l2, _ = m.loss_grad(xb, tt, ww, rows)
    assert abs(lref - l2) <= 1e-3 * abs(lref) + 1e-7
    m.close()
