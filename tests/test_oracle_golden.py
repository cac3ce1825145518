"""The CPU oracle restatement against golden vectors produced by the reference itself
(its own scenario builders and step loop, compiled from its unmodified sources).
Expected: bit-for-bit equality of every dumped field and of the neighbour lists."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mfree_iwf_gb300 import scenarios as S

CASES = ["rings_monaghan", "rings_monaghan_contact", "rings_tl_contact", "tensile_tl", "tensile_tl_weak",
         "c1_rings_dx4mm", "c2_rings_tl_dx4mm", "rings_corot_contact", "tensile_corot", "rotation_corot",
         "rings_godunov", "rings_godunov_contact", "rotation_godunov", "rings_potential_contact", "tensile_potential",
         "rotation_potential", "tensile_godunov", "tensile_monaghan", "rotation_monaghan", "rotation_tl",
         "tensile_ul_weak", "rotation_ul_weak", "rings_ul_weak_contact", "tensile_tl_fem", "rotation_tl_fem",
         "rings_tl_fem_contact", "rotation_tl_weak", "rings_tl_weak_contact", "tensile_ul_fem", "rotation_ul_fem",
         "rings_ul_fem_contact"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_bitwise(name, oracle_bin, tmp_path):
    import oracle
    case = os.path.join(GOLDEN, f"{name}.case")
    out = str(tmp_path / "o.out")
    assert oracle.run_case_file(case, out, oracle_bin) == 0
    got = S.read_result(out)
    ref = S.read_result(os.path.join(GOLDEN, f"{name}.ref.out"))
    assert got.ok and ref.ok
    assert len(got.dumps) == len(ref.dumps)
    for dg, dr in zip(got.dumps, ref.dumps):
        assert dg["step"] == dr["step"]
        assert dg["time"] == dr["time"]
        for bg, br in zip(dg["bodies"], dr["bodies"]):
            for k in S.OUT_NAMES:
                assert np.array_equal(bg[k].view(np.uint64), br[k].view(np.uint64)), (name, k)
    for lg, lr in zip(got.neighbors, ref.neighbors):
        assert all(np.array_equal(a, b) for a, b in zip(lg, lr))


def test_golden_cases_exercise_contact_and_pull():
    r = S.read_result(os.path.join(GOLDEN, "rings_monaghan_contact.ref.out"))
    assert any(np.count_nonzero(b["fcx"]) > 0 for b in r.dumps[-1]["bodies"])
    for name in ("rings_tl_contact", "rings_corot_contact", "rings_godunov_contact", "rings_potential_contact",
                 "rings_ul_weak_contact"):
        r = S.read_result(os.path.join(GOLDEN, f"{name}.ref.out"))
        assert any(np.count_nonzero(b["fcx"]) > 0 for b in r.dumps[-1]["bodies"]), name
    c = S.read_case(os.path.join(GOLDEN, "tensile_tl.case"))
    r = S.read_result(os.path.join(GOLDEN, "tensile_tl.ref.out"))
    left = c.bodies[0].bcs[0].idx
    assert np.all(r.dumps[-1]["bodies"][0]["vx"][left] == -10.0)


def test_oracle_reports_neighbour_overflow(oracle_bin, tmp_path):
    """A neighbour list reaching MAX_NBH = 200 is the reference's assert (grid.h:167)."""
    import oracle
    sc = S.rings_monaghan(40)
    sc.bodies[0].arrays["h"] *= 6.0  # h = 10 dx: several hundred particles inside 2h
    res = oracle.run(sc, 1)
    assert not res.ok
