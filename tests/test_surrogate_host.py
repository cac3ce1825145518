"""Host-side logic of the surrogate screen (no GPU): sampling, instance geometry,
scalings, monitor reduction and threshold calibration."""
import numpy as np
import pytest

from mfree_iwf_gb300 import surrogate as SG


def test_sampling_is_seeded_and_in_range():
    a, b = SG.sample_params(500, 3), SG.sample_params(500, 3)
    np.testing.assert_array_equal(a, b)
    for j, k in enumerate(("E", "nu", "rho", "v")):
        lo, hi = SG.RANGES[k]
        assert a[:, j].min() >= lo and a[:, j].max() <= hi
    q = a[:, 4] / a[:, 5]
    assert q.min() >= SG.RANGES["q"][0] - 1e-12 and q.max() <= SG.RANGES["q"][1] + 1e-12
    f = SG.features(a)
    assert f.dtype == np.float32 and f.min() >= -1 and f.max() <= 1


def test_instance_geometry():
    p = np.array([3e7, 0.35, 1200.0, 8.0, 0.028, 0.04])
    sc = SG.impact_instance(p)
    dx = 0.04 / SG.NR
    assert len(sc.bodies) == 2 and sc.contact == 1
    left, right = sc.bodies
    assert len(left.hull) > 0 and len(right.hull) > 0
    gap = right.arrays["x"].min() - left.arrays["x"].max()
    assert gap == pytest.approx(3 * dx, rel=1e-9)  # centres at -+(r_out + dx/2); the lattice keeps r < r_out
    assert sc.dt == pytest.approx(0.3 * 1.3 * dx / SG.wave_speed(p[None])[0], rel=1e-12)
    assert np.all(left.arrays["vx"] == 8.0) and np.all(right.arrays["vx"] == -8.0)
    r = np.hypot(left.arrays["x"] - left.arrays["x"].mean(), left.arrays["y"])
    assert r.max() <= 0.04 + 1e-12 and r.min() >= 0.028 - 1e-12


def test_batch_scenario_groups():
    p = SG.sample_params(3, 9)
    ens, groups = SG.batch_scenario(p)
    assert groups == [0, 0, 1, 1, 2, 2]
    assert len(ens.bodies) == 6
    for k in range(3):
        assert ens.bodies[2 * k].params["E"] == p[k, 0]


def test_scalings_roundtrip():
    p = SG.sample_params(50, 4)
    rng = np.random.default_rng(0)
    t = np.concatenate([-rng.uniform(1, 8, (50, 1)), rng.uniform(1e5, 1e7, (50, 1)), rng.uniform(0, 1e4, (50, 64))],
                       axis=1)
    np.testing.assert_allclose(SG.physical(p, SG.dimensionless(p, t)), t, rtol=1e-12)


def test_targets_from_monitor():
    n, steps = 3, 128
    mon = np.zeros((steps, 2 * n, 4), np.float32)
    mon[:, :, 0] = np.arange(steps)[:, None]
    mon[5, 1, 2] = 7.0   # instance 0, right ring
    mon[9, 4, 2] = 3.0   # instance 2, left ring
    mon[:, 2, 3] = np.repeat(np.arange(64), 2)[:, None].ravel()  # instance 1, left ring force
    t = SG.targets_from_monitor(mon, n)
    assert t.shape == (n, SG.N_OUT)
    assert np.all(t[:, 0] == steps - 1)
    assert t[0, 1] == 7.0 and t[2, 1] == 3.0 and t[1, 1] == 0.0
    np.testing.assert_array_equal(t[1, 2:], np.arange(64))


def test_calibration_picks_the_largest_safe_threshold(monkeypatch):
    sur = SG.Surrogate.__new__(SG.Surrogate)
    n = 200
    spread = np.linspace(0.001, 0.2, n)
    truth = np.zeros((n, SG.N_OUT))
    truth[:, 0] = -5.0
    pred = truth.copy()
    pred[:, 0] = -5.0 * (1 + 0.5 * spread)  # error = spread / 2
    monkeypatch.setattr(sur, "predict", lambda params: (pred, spread), raising=False)
    thr = sur.calibrate(np.zeros((n, 6)), truth, max_error=0.02, quantile=1.0)
    assert thr == pytest.approx(spread[spread / 2 <= 0.02 + 1e-15].max())
