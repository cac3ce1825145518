"""The FP64 network oracle (oracle/mlp_ref.py) pinned on the CPU: its BF16 rounding
against PyTorch's, and its analytic gradients against central finite differences."""
import numpy as np
import pytest

from oracle import mlp_ref as R


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(size=4096) * 10.0 ** rng.integers(-30, 30, size=4096),
                        [0.0, -0.0, 1.0, 1.00390625, 1.005859375, 65504.0, 3.3895e38]]).astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(R.bf16_round(x), want)


def _tiny(seed=5, dims=(6, 16, 12, 5), rows=9):
    rng = np.random.default_rng(seed)
    n = sum(dims[l] * dims[l + 1] + dims[l + 1] for l in range(len(dims) - 1))
    p = rng.normal(size=n) * 0.5
    x = rng.uniform(-1, 1, size=(rows, dims[0]))
    y = rng.normal(size=(rows, dims[-1]))
    return p, list(dims), x, y


def test_exact_gradients_match_finite_differences():
    p, dims, x, y = _tiny()
    g = R.exact_gradients(p, dims, x, y)
    idx = np.arange(0, p.size, 7)
    num = R.numeric_gradients(p, dims, x, y, idx)
    np.testing.assert_allclose(g[idx], num, rtol=1e-6, atol=1e-9)


def test_unrounded_mode_is_the_exact_network_on_bf16_values():
    p, dims, x, y = _tiny(seed=11)
    pb, xb = R.bf16_round(p), R.bf16_round(x)
    g, loss = R.gradients(pb, dims, xb, y, emulate=False)
    np.testing.assert_allclose(g, R.exact_gradients(pb, dims, xb, y), rtol=1e-12, atol=1e-15)
    z, _ = R.forward(pb, dims, xb, emulate=False)
    assert loss == pytest.approx(float(np.mean((z - y) ** 2)), rel=1e-12)


def test_pack_unpack_roundtrip():
    p, dims, _, _ = _tiny()
    np.testing.assert_array_equal(R.pack(R.unpack(p, dims)), p)
