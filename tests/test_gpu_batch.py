"""Batched ensembles, CUDA-graph replay and the autotuner.

* A batch of independent bodies in one context gives every body exactly (bit for
  bit) what it gets when simulated alone: each body has its own cell grid, and the
  cell-ordered summation order does not depend on the other bodies.
* Replaying a captured step graph, and running with the launch shapes the autotuner
  picked, give bit-identical states (per-row arithmetic does not depend on the launch
  shape; the autotuner restores the state it trialled on).
"""
import numpy as np
import pytest

from mfree_iwf_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy")


def states(sim, nb):
    return [sim.get_state(b, FIELDS) for b in range(nb)]


def small_ensemble(k=6):
    # coarse instances (dx drawn in 2.5-4 mm) so the test stays small
    return S.c4_ensemble(k, dx_range=(2.5e-3, 4e-3))


@pytest.mark.parametrize("precision", ["fp64_strict", "mixed"])
def test_batch_equals_instances_alone(lib, precision):
    import mfree_iwf_gb300 as M
    ens = small_ensemble()
    sim = M.from_scenario(ens, precision=precision)
    sim.step(20)
    batched = states(sim, len(ens.bodies))
    sim.close()
    for k, b in enumerate(ens.bodies):
        one = S.Scenario(method=ens.method, bodies=[b], actions=ens.actions, dt=b.params["dt"], nu=b.params["nu"],
                         E=b.params["E"], rho0=b.params["rho0"], wdeltap=b.params["wdeltap"], corr_exp=ens.corr_exp,
                         mghn_eps=ens.mghn_eps, alpha=ens.alpha, beta=ens.beta, eta=ens.eta, xsph_eps=ens.xsph_eps,
                         nbh_eps=ens.nbh_eps)
        s1 = M.from_scenario(one, precision=precision)
        s1.step(20)
        alone = s1.get_state(0, FIELDS)
        s1.close()
        for f in FIELDS:
            assert np.array_equal(alone[f], batched[k][f]), (k, f)


@pytest.mark.parametrize("kind", ["ul", "tl"])
def test_graph_and_autotune_do_not_change_results(lib, kind):
    import mfree_iwf_gb300 as M
    sc = small_ensemble() if kind == "ul" else S.c2_rings_tl(dx=2e-3)
    nb = len(sc.bodies)
    a = M.from_scenario(sc, precision="mixed")
    a.step(12)
    want = states(a, nb)
    a.close()
    b = M.from_scenario(sc, precision="mixed", graph=True)
    b.step(1)
    report = b.autotune(2)
    assert "->" in report or "cached" in report
    b.step(11)
    got = states(b, nb)
    b.close()
    for k in range(nb):
        for f in FIELDS:
            assert np.array_equal(got[k][f], want[k][f]), (kind, k, f)


@pytest.mark.parametrize("precision", ["fp64_strict", "mixed"])
def test_all_bodies_state_io_equals_per_body(lib, precision):
    """get_state_all / set_state_all move every body's rows in one call per field; they
    read and write exactly what the per-body calls do (densities of bodies with
    different rho0 included)."""
    import mfree_iwf_gb300 as M
    ens = small_ensemble()
    sims = [M.from_scenario(ens, precision=precision) for _ in range(2)]
    for s in sims:
        s.step(7)
    n = sum(b.n for b in ens.bodies)
    allst = {f: np.empty(n) for f in FIELDS}
    sims[0].get_state_all_into(allst)
    per = states(sims[0], len(ens.bodies))
    offs = np.cumsum([0] + [b.n for b in ens.bodies])
    for k in range(len(ens.bodies)):
        for f in FIELDS:
            np.testing.assert_array_equal(allst[f][offs[k]:offs[k + 1]], per[k][f])
    # write back: all at once into one context, per body into the other, then step on
    perturbed = {f: v * (1 + 1e-9) if f in ("vx", "vy") else v for f, v in allst.items()}
    sims[0].set_state_all(perturbed)
    for k in range(len(ens.bodies)):
        sims[1].set_state(k, {f: perturbed[f][offs[k]:offs[k + 1]] for f in FIELDS})
    for s in sims:
        s.step(3)
    a, b = states(sims[0], len(ens.bodies)), states(sims[1], len(ens.bodies))
    for k in range(len(ens.bodies)):
        for f in FIELDS:
            np.testing.assert_array_equal(a[k][f], b[k][f])
    for s in sims:
        s.close()


def instance_alone(ens, k):
    b = ens.bodies[k]
    return S.Scenario(method=ens.method, bodies=[b], actions=ens.actions, dt=b.params["dt"], nu=b.params["nu"],
                      E=b.params["E"], rho0=b.params["rho0"], wdeltap=b.params["wdeltap"], corr_exp=ens.corr_exp,
                      mghn_eps=ens.mghn_eps, alpha=ens.alpha, beta=ens.beta, eta=ens.eta, xsph_eps=ens.xsph_eps,
                      nbh_eps=ens.nbh_eps)


@pytest.mark.parametrize("precision", ["fp64_strict", "mixed"])
def test_failed_instance_is_masked(lib, precision):
    """Per-body failure masking ("mask_failed"): a NaN planted from the host into one
    of six instances after 5 steps fails that instance alone -- mf_step reports
    MF_ERR_BODY_FAILED, the failure word names it, and its state stays frozen -- while
    the other five step on bit for bit as they do alone (20 steps)."""
    import mfree_iwf_gb300 as M
    ens = small_ensemble()
    nb = len(ens.bodies)
    sim = M.from_scenario(ens, precision=precision)
    sim.set_option("mask_failed", 1)
    assert sim.get_option("mask_failed") == 1
    sim.step(5)
    bad = 2
    st = sim.get_state(bad, FIELDS)
    st["vx"][len(st["vx"]) // 2] = np.nan
    sim.set_state(bad, st)
    with pytest.raises(M.BodyFailed) as ei:
        sim.step(15)
    assert ei.value.status == M.ERR_BODY_FAILED
    failed = sim.failed()
    assert list(np.nonzero(failed)[0]) == [bad], failed
    assert failed[bad] & (4 | 8), failed  # a grid error or a non-finite state
    got = states(sim, nb)
    frozen = got[bad]
    with pytest.raises(M.BodyFailed):  # the failed body stays frozen, the others go on
        sim.step(1)
    again = sim.get_state(bad, FIELDS)
    for f in FIELDS:
        np.testing.assert_array_equal(again[f], frozen[f], err_msg=f)
    sim.close()
    for k in range(nb):
        if k == bad:
            continue
        s1 = M.from_scenario(instance_alone(ens, k), precision=precision)
        s1.step(20)
        alone = s1.get_state(0, FIELDS)
        s1.close()
        for f in FIELDS:
            assert np.array_equal(alone[f], got[k][f]), (k, f)


@pytest.mark.parametrize("masked", [False, True])
def test_async_steps_report_at_synchronize(lib, masked):
    """Option async_steps: mf_step queues the steps and returns at once; a NaN planted
    from the host surfaces at the next mf_synchronize -- as a non-finite state, or with
    mask_failed as the failed body -- instead of at the step."""
    import mfree_iwf_gb300 as M
    ens = small_ensemble()
    sim = M.from_scenario(ens, precision="mixed")
    if masked:
        sim.set_option("mask_failed", 1)
    sim.set_option("async_steps", 1)
    assert sim.get_option("async_steps") == 1
    sim.step(3)
    sim.synchronize()
    st = sim.get_state(1, FIELDS)
    st["vx"][len(st["vx"]) // 2] = np.nan
    sim.set_state(1, st)
    sim.step(5)  # no error here: nothing read the status yet
    with pytest.raises(M.MfError) as ei:
        sim.synchronize()
    assert isinstance(ei.value, M.BodyFailed) == masked, ei.value
    sim.close()


def test_without_masking_a_failure_fails_the_step(lib):
    """Without the option a NaN in one instance fails mf_step as a whole (the
    reference's behaviour is an abort)."""
    import mfree_iwf_gb300 as M
    ens = small_ensemble()
    sim = M.from_scenario(ens, precision="fp64_strict")
    sim.step(2)
    st = sim.get_state(1, FIELDS)
    st["x"][0] = np.nan
    sim.set_state(1, st)
    with pytest.raises(M.MfError) as ei:
        sim.step(3)
    assert not isinstance(ei.value, M.BodyFailed)
    assert ei.value.status in (-4, -7)  # non-finite state / grid
    sim.close()


@pytest.mark.parametrize("method,precision", [("ul", "fp64_strict"), ("ul", "mixed"), ("tl", "mixed"), ("tl", "fp64")])
def test_async_state_transfers_equal_sync(lib, method, precision):
    """The stream-ordered transfers (per-field copies on two copy streams, each set
    waiting for the earlier get of its field) give exactly what the synchronous calls
    give: a loop of set / step / get on the same pinned host arrays ends in the same
    bits, and the state read back equals the per-body reads."""
    import torch
    import mfree_iwf_gb300 as M
    sc = small_ensemble() if method == "ul" else S.c2_rings_tl(dx=2e-3)
    nb = len(sc.bodies)
    n = sum(b.n for b in sc.bodies)
    out = {}
    for mode in ("sync", "async"):
        sim = M.from_scenario(sc, precision=precision)
        sim.step(2)
        host = {f: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for f in FIELDS}
        sim.get_state_all_into(host)
        for _ in range(6):
            if mode == "sync":
                sim.set_state_all(host)
                sim.step(1)
                sim.get_state_all_into(host)
            else:
                sim.set_state_all_async(host)
                sim.step(1)
                sim.get_state_all_async_into(host)
        sim.synchronize()
        out[mode] = {f: host[f].copy() for f in FIELDS}
        if mode == "async":
            per = states(sim, nb)
            offs = np.cumsum([0] + [b.n for b in sc.bodies])
            for k in range(nb):
                for f in FIELDS:
                    np.testing.assert_array_equal(out[mode][f][offs[k]:offs[k + 1]], per[k][f], err_msg=f)
        sim.close()
    for f in FIELDS:
        np.testing.assert_array_equal(out["async"][f], out["sync"][f], err_msg=f)
