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
