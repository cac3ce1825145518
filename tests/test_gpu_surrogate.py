"""The surrogate's GPU parts: the per-step monitor, the BF16 MLP kernels against the FP64
network oracle, training, and the screened sweep against the solver alone."""
import numpy as np
import pytest

from mfree_iwf_gb300 import scenarios as S
from oracle import mlp_ref as R

pytestmark = pytest.mark.gpu

DIMS = [6, 256, 256, 256, 66]


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


# ---------------------------------------------------------------- monitor
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_monitor_matches_state(lib, precision):
    import mfree_iwf_gb300 as M
    sc = S.c1_rings(dx=4e-3, two_bodies=True)
    sim = M.from_scenario(sc, precision=precision)
    sim.set_monitor(8)
    sim.step(11)
    mon = sim.monitor()
    assert mon.shape == (8, 2, 4)
    rows = {}
    for b in range(2):
        st = sim.get_state(b, ("vx", "vy", "rho", "Sxx", "Sxy", "Syy", "fcx", "fcy"))
        p = sc.c0 ** 2 * (st["rho"] - sc.rho0)  # the workload's EOS: p = c0^2 (rho - rho0)
        sxx, syy, sxy = st["Sxx"] - p, st["Syy"] - p, st["Sxy"]
        vm = np.sqrt(np.maximum(sxx * sxx - sxx * syy + syy * syy + 3 * sxy * sxy, 0)).max()
        rows[b] = [st["vx"].mean(), st["vy"].mean(), vm, np.hypot(st["fcx"], st["fcy"]).sum()]
    sim.close()
    last = (11 - 1) % 8  # ring row of the last step
    for b in range(2):
        np.testing.assert_allclose(mon[last, b, :3], rows[b][:3], rtol=2e-6, atol=1e-6 * abs(sc.bodies[0].arrays["vx"]).max())
        np.testing.assert_allclose(mon[last, b, 3], rows[b][3], rtol=2e-6, atol=1e-9)


# ---------------------------------------------------------------- MLP kernels
@pytest.fixture(scope="module")
def mlp(lib):
    from mfree_iwf_gb300.surrogate import Mlp
    m = Mlp(DIMS, members=5, max_batch=256, seed=123)
    yield m
    m.close()


def _batch(seed, members, rows):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=(members, rows, DIMS[0])).astype(np.float32)
    y = rng.normal(size=(members, rows, DIMS[-1])).astype(np.float32)
    return x, y


@pytest.mark.parametrize("rows", [256, 77])
def test_mlp_gradients_match_oracle(mlp, rows):
    x, y = _batch(rows, mlp.members, rows)
    g, loss = mlp.gradients(x, y)
    for z in range(mlp.members):
        p = mlp.get_params(z).astype(np.float64)
        ge, le = R.gradients(p, DIMS, x[z], y[z], emulate=True)
        gx, lx = R.gradients(p, DIMS, x[z], y[z], emulate=False)
        # BF16 at the same points as the kernels: only the FP32 accumulation differs
        assert _rel(g[z], ge) < 5e-3, (z, _rel(g[z], ge))
        assert abs(loss[z] - le) <= 1e-3 * le
        # against the unrounded network the BF16 activations cost ~1e-2
        assert _rel(g[z], gx) < 4e-2, (z, _rel(g[z], gx))
        assert abs(loss[z] - lx) <= 2e-2 * lx
        # layer by layer too (the first layer's 6 inputs and the biases are small blocks)
        o = 0
        for l in range(len(DIMS) - 1):
            for n in (DIMS[l] * DIMS[l + 1], DIMS[l + 1]):
                assert _rel(g[z][o:o + n], ge[o:o + n]) < 1e-2, (z, l, n)
                o += n


def test_mlp_predict_matches_oracle(mlp):
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, size=(1000, DIMS[0])).astype(np.float32)  # 4 chunks, the last ragged
    y = mlp.predict(x)
    assert y.shape == (mlp.members, 1000, DIMS[-1])
    for z in range(mlp.members):
        ye, _ = R.forward(mlp.get_params(z).astype(np.float64), DIMS, x, emulate=True)
        assert _rel(y[z], ye) < 3e-3


def test_mlp_params_roundtrip_and_errors(lib):
    from mfree_iwf_gb300 import MfError
    from mfree_iwf_gb300.surrogate import Mlp
    m = Mlp([3, 20, 2], members=2, max_batch=16, seed=5)
    p = np.random.default_rng(1).normal(size=m.num_params).astype(np.float32)
    assert m.num_params == 3 * 20 + 20 + 20 * 2 + 2
    m.set_params(1, p)
    np.testing.assert_array_equal(m.get_params(1), p)
    with pytest.raises(MfError):
        m.train(10, 1e-3, 1e-4)  # no data yet
    with pytest.raises(MfError):
        m.gradients(np.zeros((2, 17, 3), np.float32), np.zeros((2, 17, 2), np.float32))  # > max_batch
    m.close()


def test_mlp_training_fits_a_smooth_map(lib):
    from mfree_iwf_gb300.surrogate import Mlp
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, size=(4096, 6)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], x[:, 2] ** 2 - x[:, 3] * x[:, 4], np.cos(x[:, 5] + x[:, 0])], axis=1)
    y = np.concatenate([t, np.tile(t[:, :1], (1, 63))], axis=1).astype(np.float32)
    m = Mlp(DIMS, members=5, max_batch=256, seed=2)
    m.set_data(x, y)
    before = m.launch_count()
    hist = m.train(3000, 2e-3, 2e-5)
    assert m.launch_count() > before  # replays of the captured training step
    assert np.all(np.isfinite(hist))
    assert hist[-50:].mean() < 0.02 * hist[:10].mean()
    xt = rng.uniform(-1, 1, size=(512, 6)).astype(np.float32)
    tt = np.stack([np.sin(2 * xt[:, 0]) * xt[:, 1], xt[:, 2] ** 2 - xt[:, 3] * xt[:, 4], np.cos(xt[:, 5] + xt[:, 0])],
                  axis=1)
    pred = m.predict(xt).mean(axis=0)[:, :3]
    assert np.sqrt(np.mean((pred - tt) ** 2)) < 0.05
    m.close()


# ---------------------------------------------------------------- the screen
def test_dimensionless_outputs_are_self_similar(lib):
    """Instances that share nu, v / c0 and r_in / r_out give the same dimensionless
    outputs whatever their size, stiffness and density: the property the surrogate's
    inputs rest on."""
    from mfree_iwf_gb300 import surrogate as SG
    base = np.array([4e7, 0.35, 1200.0, 8.0, 0.7 * 0.04, 0.04])
    rows = [base]
    for sr, se, sv in ((1.25, 1.0, 1.0), (0.8, 1.4, 1.0), (1.0, 2.0, np.sqrt(2.0))):
        r = base.copy()
        r[5] *= sr
        r[4] = 0.7 * r[5]
        r[0] *= se
        r[2] *= se           # E and rho together: c0 unchanged
        if sv != 1.0:
            r[0] *= sv * sv  # E x2, v x sqrt(2): v / c0 unchanged
            r[3] *= sv
        rows.append(r)
    p = np.array(rows)
    run = SG.simulate(p, steps=64 * 20)
    d = SG.dimensionless(p, run.targets)
    for k in range(1, len(p)):
        assert abs(d[k, 0] - d[0, 0]) <= 2e-3 * abs(d[0, 0]), (k, d[:, 0])
        assert abs(d[k, 1] - d[0, 1]) <= 2e-3, (k, d[:, 1])
        assert _rel(d[k, 2:], d[0, 2:]) < 1e-2, k



def test_screened_sweep_beats_the_solver(lib):
    """Train on instances the batched solver simulates, then answer a new sweep: the
    network takes the instances its members agree on and the solver the rest.  The
    rebound velocity of the accepted instances stays within 2 % (95th percentile) and
    the sweep finishes faster than the solver alone."""
    from mfree_iwf_gb300 import surrogate as SG
    train_p = SG.sample_params(1792, seed=1001)
    test_p = SG.sample_params(256, seed=2002)
    run = SG.simulate(np.concatenate([train_p, test_p]))
    assert run.valid.mean() > 0.98 and not run.failed.any()
    train_t, test_t = run.targets[:1792], run.targets[1792:]
    truth = SG.simulate(test_p)  # the solver-only sweep, timed
    np.testing.assert_array_equal(truth.targets, test_t)  # batch composition does not change an instance
    fit = np.nonzero(run.valid[:1536])[0]
    val = 1536 + np.nonzero(run.valid[1536:1792])[0]
    sur = SG.Surrogate(seed=7)
    hist = sur.fit(train_p[fit], train_t[fit], steps=4000)
    assert hist[-100:].mean() < 0.05 * hist[:10].mean()
    thr = sur.calibrate(train_p[val], train_t[val])
    assert thr > 0
    res = sur.screen(test_p)
    acc = res.accepted & truth.valid
    err = np.abs(res.targets[:, 0] - test_t[:, 0]) / np.abs(test_t[:, 0])
    assert res.accepted.mean() >= 0.5, res.accepted.mean()
    assert np.quantile(err[acc], 0.95) <= 0.03, np.quantile(err[acc], 0.95)
    fb = ~res.accepted
    np.testing.assert_array_equal(res.targets[fb], test_t[fb])  # fallbacks are the solver's own answer
    t_screened = res.seconds_network + res.seconds_solver
    assert t_screened < truth.seconds + truth.setup_seconds


# ------------------------------------------------------- tcgen05 GEMM
@pytest.mark.parametrize("rows", [300, 4096])
def test_tcgen05_forward_matches_mma_sync(lib, rows):
    """Inference on tcgen05 -- the fused whole-network kernel (the default) and the
    per-layer GEMM (option fused 0: TMEM accumulators, TMA-staged 128-byte-swizzled
    operands for the products with K a multiple of 64) -- against the mma.sync kernels on
    the same parameters and inputs: all accumulate the same BF16 products in FP32 in
    different orders, so the FP32 outputs agree to within the BF16 rounding of the hidden
    activations they pass between layers (relative L2 <= 5e-3 per member; in practice
    ~1e-3).  300 rows: one partial tile per member; 4096 rows: several tiles per
    persistent CTA, both accumulators."""
    from mfree_iwf_gb300.surrogate import Mlp
    mlp = Mlp(DIMS, members=5, max_batch=rows, seed=11)
    assert mlp.get_option("tcgen05") == 1  # the default on a GB300
    assert mlp.get_option("fused") == 1
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, size=(rows, DIMS[0])).astype(np.float32)
    y_fz = mlp.predict(x)
    mlp.set_option("fused", 0)
    assert mlp.get_option("fused") == 0
    y_tc = mlp.predict(x)
    mlp.set_option("tcgen05", 0)
    y_ref = mlp.predict(x)
    mlp.set_option("tcgen05", 1)
    y_tc2 = mlp.predict(x)
    mlp.set_option("fused", 1)
    y_fz2 = mlp.predict(x)
    mlp.close()
    assert y_tc.shape == y_fz.shape == (5, rows, DIMS[-1])
    np.testing.assert_array_equal(y_tc, y_tc2)  # deterministic
    np.testing.assert_array_equal(y_fz, y_fz2)
    for z in range(5):
        e, ef = _rel(y_tc[z], y_ref[z]), _rel(y_fz[z], y_ref[z])
        print(f"member {z}: relative L2 per-layer {e:.2e} fused {ef:.2e}")
        assert e <= 5e-3 and ef <= 5e-3, (z, e, ef)


@pytest.mark.parametrize("dims", [[6, 100, 40, 66], [3, 64, 2], [70, 256, 130, 8], [6, 64, 200]])
def test_fused_predict_on_padded_widths(lib, dims):
    """The fused kernel on widths that are not multiples of 64 (the hidden activations
    zero padded to the next layer's K, outputs fewer than 32 or more than 128 -- two
    blocks of the transposed output layer --, an input wider than 64) against the FP64
    network oracle with BF16 rounding at the same points, and against the mma.sync
    kernels."""
    from mfree_iwf_gb300.surrogate import Mlp
    mlp = Mlp(dims, members=3, max_batch=300, seed=7)
    assert mlp.get_option("fused") == 1
    rng = np.random.default_rng(8)
    for z in range(3):  # non-zero biases too
        p = mlp.get_params(z)
        mlp.set_params(z, p + rng.normal(scale=0.1, size=p.shape).astype(np.float32))
    x = rng.uniform(-1, 1, size=(700, dims[0])).astype(np.float32)  # 3 chunks, the last ragged
    y = mlp.predict(x)
    mlp.set_option("tcgen05", 0)
    y_ref = mlp.predict(x)
    for z in range(3):
        ye, _ = R.forward(mlp.get_params(z).astype(np.float64), dims, x, emulate=True)
        e, er = _rel(y[z], ye), _rel(y[z], y_ref[z])
        print(dims, z, f"oracle {e:.2e} mma.sync {er:.2e}")
        assert e < 3e-3 and er < 5e-3, (z, e, er)
    mlp.close()


def test_fused_predict_not_taken_past_256_wide(lib):
    """A layer wider than 256 leaves inference on the per-layer kernels."""
    from mfree_iwf_gb300.surrogate import Mlp
    mlp = Mlp([6, 300, 4], members=2, max_batch=64, seed=3)
    assert mlp.get_option("tcgen05") == 1 and mlp.get_option("fused") == 0
    x = np.random.default_rng(2).uniform(-1, 1, size=(50, 6)).astype(np.float32)
    y = mlp.predict(x)
    for z in range(2):
        ye, _ = R.forward(mlp.get_params(z).astype(np.float64), [6, 300, 4], x, emulate=True)
        assert _rel(y[z], ye) < 3e-3
    mlp.close()


def test_fused_predict_device_buffers_one_launch(lib):
    """With device-resident inputs and outputs the fused path runs every row in one
    launch, straight into the caller's [members][n][out] buffer, and equals the chunked
    host-buffer path bit for bit (rows are independent of the tiling); new parameters
    are re-packed before the next inference."""
    import ctypes
    import torch
    from mfree_iwf_gb300.surrogate import Mlp
    mlp = Mlp(DIMS, members=4, max_batch=512, seed=21)
    rng = np.random.default_rng(6)
    n = 3000
    x = rng.uniform(-1, 1, size=(n, DIMS[0])).astype(np.float32)
    y_host = mlp.predict(x)  # 6 chunks of 512 rows through host staging
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty((4, n, DIMS[-1]), device="cuda", dtype=torch.float32)
    fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))
    before = mlp.launch_count()
    mlp._check(mlp._lib.mf_mlp_predict(mlp._h, fp(xd), n, fp(yd)), "mf_mlp_predict")
    assert mlp.launch_count() - before == 1
    np.testing.assert_array_equal(yd.cpu().numpy(), y_host)
    p = mlp.get_params(2) * 0.5
    mlp.set_params(2, p)
    mlp._check(mlp._lib.mf_mlp_predict(mlp._h, fp(xd), n, fp(yd)), "mf_mlp_predict")
    ye, _ = R.forward(p.astype(np.float64), DIMS, x, emulate=True)
    assert _rel(yd[2].cpu().numpy(), ye) < 3e-3
    np.testing.assert_array_equal(yd[0].cpu().numpy(), y_host[0])
    mlp.close()


def test_tcgen05_training_matches_mma_sync(lib):
    """A short training run (captured step graph) with the forward products on tcgen05
    follows the mma.sync run: the loss histories agree within 2 % and both fall."""
    from mfree_iwf_gb300.surrogate import Mlp
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, size=(2048, DIMS[0])).astype(np.float32)
    y = np.tanh(x @ rng.normal(size=(DIMS[0], DIMS[-1])).astype(np.float32))
    hist = {}
    for tc in (1, 0):
        mlp = Mlp(DIMS, members=3, max_batch=512, seed=2)
        mlp.set_option("tcgen05", tc)
        mlp.set_data(x, y)
        hist[tc] = mlp.train(60, 1e-3, 1e-4)
        mlp.close()
    for tc in (1, 0):
        assert hist[tc][-5:].mean() < 0.5 * hist[tc][:5].mean(), tc
    e = _rel(hist[1][-10:], hist[0][-10:])
    print(f"loss histories: relative L2 {e:.2e}")
    assert e <= 2e-2
