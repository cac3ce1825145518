"""State output: the VTK writer against the reference's own vtk_writer_write output
(golden files made by tests/golden/make_golden.py), asynchronous dumps while the
simulation steps on, and exact checkpoint/restart."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mfree_iwf_gb300 import scenarios as S

VTK_CASES = ["tensile_tl", "rings_tl_contact"]
FIELDS = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy")


def _vtk_bodies(sc, state_bodies):
    return [dict(x=s["x"], y=s["y"], h=b.arrays["h"], rho=s["rho"], Sxx=s["Sxx"], Sxy=s["Sxy"], Syy=s["Syy"],
                 vx=s["vx"], vy=s["vy"]) for b, s in zip(sc.bodies, state_bodies)]


@pytest.mark.parametrize("name", VTK_CASES)
def test_vtk_writer_matches_the_reference_writer(lib, name, tmp_path):
    """The host writer, given the reference's final state, writes the reference's file byte for byte."""
    import mfree_iwf_gb300 as M
    sc = S.read_case(os.path.join(GOLDEN, f"{name}.case"))
    ref = S.read_result(os.path.join(GOLDEN, f"{name}.ref.out")).dumps[-1]["bodies"]
    out = str(tmp_path / "o.vtk")
    M.write_vtk_arrays(out, _vtk_bodies(sc, ref))
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, f"{name}.vtk"), "rb").read()


def test_vtk_writer_ragged_bodies(lib, tmp_path):
    import mfree_iwf_gb300 as M
    rng = np.random.default_rng(2)
    bodies = []
    for n in (3, 0, 5):
        bodies.append({f: rng.normal(size=n) for f in ("x", "y", "h", "rho", "Sxx", "Sxy", "Syy", "vx", "vy")})
    out = str(tmp_path / "o.vtk")
    M.write_vtk_arrays(out, bodies)
    text = open(out).read().split("\n")
    assert "POINTS 8 float" in text and "CELLS 8 16" in text and "CELL_TYPES 8" in text and "POINT_DATA 8" in text
    i = text.index("VECTORS velocity float")
    vel = np.array([list(map(float, t.split())) for t in text[i + 1:i + 9]])
    want = np.concatenate([b["vx"] for b in bodies])
    np.testing.assert_allclose(vel[:, 0], want, atol=5e-7)


# ---------------------------------------------------------------- on the GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", VTK_CASES)
def test_gpu_vtk_equals_the_reference_writer(lib, name, tmp_path):
    """The TL path is bit-identical to the reference, so its VTK file is the reference's."""
    import mfree_iwf_gb300 as M
    sc = S.read_case(os.path.join(GOLDEN, f"{name}.case"))
    steps = S.read_result(os.path.join(GOLDEN, f"{name}.ref.out")).dumps[-1]["step"]
    sim = M.from_scenario(sc, precision="fp64_strict")
    sim.step(steps)
    out = str(tmp_path / "o.vtk")
    sim.write_vtk(out)
    sim.close()
    assert open(out, "rb").read() == open(os.path.join(GOLDEN, f"{name}.vtk"), "rb").read()


@pytest.mark.gpu
def test_gpu_async_dump_is_the_state_at_the_dump(lib, tmp_path):
    """A dump issued after step 5 holds the step-5 state although 20 more steps are
    issued before it is waited for."""
    import mfree_iwf_gb300 as M
    sc = S.c1_rings(dx=4e-3, two_bodies=True)
    sim = M.from_scenario(sc, precision="mixed")
    sim.step(5)
    want = [sim.get_state(b) for b in range(2)]
    sim.dump_async(str(tmp_path / "async.vtk"))
    sim.step(20)
    sim.dump_wait()
    sim.close()
    M.write_vtk_arrays(str(tmp_path / "want.vtk"), _vtk_bodies(sc, want))
    assert open(tmp_path / "async.vtk", "rb").read() == open(tmp_path / "want.vtk", "rb").read()


@pytest.mark.gpu
@pytest.mark.parametrize("case,precision", [("ul_contact", "fp64_strict"), ("ul_contact", "mixed"),
                                            ("tl_contact", "mixed"), ("tl_pull", "fp64")])
def test_gpu_checkpoint_restart_is_exact(lib, tmp_path, case, precision):
    """10 steps straight equal 5 steps, a checkpoint, a new context loading it, and 5
    more steps -- bit for bit, contact forces and clocks included."""
    import mfree_iwf_gb300 as M
    if case == "ul_contact":
        sc = S.rings_monaghan_contact(20)
    elif case == "tl_contact":
        sc = S.c2_rings_tl(dx=4e-3, nbh_eps=1e-6)
    else:
        sc = S.tensile_tl(11)
    nb = len(sc.bodies)
    fields = FIELDS + ("fcx", "fcy")
    a = M.from_scenario(sc, precision=precision)
    a.step(10)
    want = [a.get_state(b, fields) for b in range(nb)]
    t_want = [a.time(b) for b in range(nb)]
    a.close()
    b_ = M.from_scenario(sc, precision=precision)
    b_.step(5)
    ck = str(tmp_path / "c.ckpt")
    b_.checkpoint_save(ck)
    b_.close()
    c = M.from_scenario(sc, precision=precision)
    c.checkpoint_load(ck)
    c.step(5)
    for k in range(nb):
        got = c.get_state(k, fields)
        for f in fields:
            np.testing.assert_array_equal(got[f], want[k][f], err_msg=f"{case} {precision} {f}")
        assert c.time(k) == t_want[k]
    # a checkpoint of another context's shape is refused
    other = M.from_scenario(S.rings_monaghan(20), precision=precision)
    with pytest.raises(M.MfError):
        other.checkpoint_load(ck)
    other.close()
    c.close()
