"""Host side of the learned part: the training targets' properties, the
feature normalisation's BF16 rounding (no GPU)."""
import numpy as np
import pytest

from help_gb300 import learned


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, 3 * n))
    return a @ a.T / n + 0.1 * np.eye(n)


def test_energy_scale_target_is_one_for_a_scaled_copy():
    # x_now = a * x_prev: the best per-row scale is the common scalar, i.e. 1 after dividing it out
    G = _spd(40, 1)
    xp = np.random.default_rng(2).standard_normal(40)
    s = learned.energy_scale_target(G, xp, 3.7 * xp, ridge=1e-6)
    assert np.allclose(s, 1.0, atol=1e-6)


def test_energy_scale_target_reduces_the_g_norm_error():
    G = _spd(30, 3)
    rng = np.random.default_rng(4)
    xp, xc = rng.standard_normal(30), rng.standard_normal(30)
    gn = lambda e: float(e @ G @ e)
    a = float(xc @ G @ xp) / float(xp @ G @ xp)
    for ridge in (0.1, 10.0, 100.0):
        s = learned.energy_scale_target(G, xp, xc, ridge=ridge)
        assert gn(a * s * xp - xc) <= gn(a * xp - xc) + 1e-12   # never worse than the single scalar
    # a heavier ridge keeps the scales closer to 1
    d1 = np.abs(learned.energy_scale_target(G, xp, xc, ridge=0.1) - 1).mean()
    d2 = np.abs(learned.energy_scale_target(G, xp, xc, ridge=100.0) - 1).mean()
    assert d2 < d1


def test_equilibration_makes_scaled_rows_unit_norm():
    S = _spd(25, 5)
    t = learned.equilibrated_log_ratio(S, iters=30)
    e = np.diag(S) * np.exp(t)
    Z = S / np.sqrt(np.outer(e, e))
    assert np.allclose(np.linalg.norm(Z, axis=1), 1.0, atol=1e-3)


def test_feature_bits_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(6).standard_normal((100, 16)).astype(np.float32) * 7
    mean = np.linspace(-1, 1, 16).astype(np.float32)
    scale = np.linspace(0.5, 2, 16).astype(np.float32)
    bits = learned.normalise_bits(x, mean, scale)
    z = (x - mean) * scale
    z[:, learned.FEATURES:] = 0
    ref = torch.from_numpy(z).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(bits, ref)


def test_sparse_warm_start_target_equals_dense():
    """The warm-start head's target from sparse products of A equals the one
    from the dense G = A D^-1 A^T (1e-6 relative: the sparse one is an
    iterative solve to 1e-8)."""
    from scipy.sparse import csr_matrix

    from help_gb300 import learned, lp as L

    lp = L.generate(L.spec_mcf(8, 3, 2), 4)
    rp, ci, v = lp.csr()
    A = csr_matrix((v, ci, rp), shape=(lp.m, lp.n))
    rng = np.random.default_rng(0)
    d = np.exp(rng.uniform(-3, 3, lp.n))
    xp = rng.standard_normal(lp.m)
    xc = xp * (1 + 0.1 * rng.standard_normal(lp.m))
    Ad = learned._dense(lp)
    t_dense = learned.energy_scale_target((Ad / d) @ Ad.T, xp, xc)
    t_sparse = learned.energy_scale_target_sparse(A, d, xp, xc)
    assert np.max(np.abs(t_dense - t_sparse)) <= 1e-6 * np.max(np.abs(t_dense))
