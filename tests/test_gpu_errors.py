"""Error behaviour of the CUDA path: the reference's asserts and floating-point traps
become status codes (no GPU fault, no trap -- the kernels set a status word)."""
import numpy as np
import pytest

from mfree_iwf_gb300 import scenarios as S

pytestmark = pytest.mark.gpu


def test_neighbour_overflow_is_reported(lib):
    import mfree_iwf_gb300 as M
    sc = S.rings_monaghan(40)
    sc.bodies[0].arrays["h"] *= 6.0
    sim = M.from_scenario(sc)
    with pytest.raises(M.MfError) as e:
        sim.step(1)
    assert e.value.name == "MF_ERR_NBH_OVERFLOW"


def test_action_order_is_validated(lib):
    import mfree_iwf_gb300 as M
    sc = S.rings_monaghan(20)
    sc.actions = list(reversed(sc.actions))
    sim = M.from_scenario(sc)
    with pytest.raises(M.MfError) as e:
        sim.step(1)
    assert e.value.name == "MF_ERR_PIPELINE"


def test_nonfinite_state_is_reported(lib):
    import mfree_iwf_gb300 as M
    sc = S.rings_monaghan(20)
    sc.bodies[0].arrays["vx"][5] = np.nan
    sim = M.from_scenario(sc)
    with pytest.raises(M.MfError) as e:
        sim.step(1)
    assert e.value.name == "MF_ERR_NONFINITE"


def test_tl_overflow_is_reported(lib):
    import mfree_iwf_gb300 as M
    sc = S.tensile_tl(21)
    sc.nbh_h *= 5.0
    sim = M.from_scenario(sc)
    with pytest.raises(M.MfError) as e:
        sim.step(1)
    assert e.value.name == "MF_ERR_NBH_OVERFLOW"
