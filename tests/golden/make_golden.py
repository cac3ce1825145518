"""Generates the golden fixtures of this directory from the reference itself.

Runs the reference's own scenario builders and step loop -- compiled out of tree
from its unmodified sources by oracle/build_ref.sh -- and stores, per case, the
initial state it built (NAME.case) and the state it reached (NAME.ref.out).  Also
runs workload-constant cases built by mfree_iwf_gb300.scenarios through the
reference's body/action machinery, and writes the final state of the VTK cases with
the reference's own vtk_writer_write (NAME.vtk).  Needs the reference sources (not on
GPU machines).

Usage: python tests/golden/make_golden.py [--vtk-only] [NAME ...]
(with names: only those reference cases)
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mfree_iwf_gb300 import scenarios as S  # noqa: E402

# (reference scenario function, nbox, steps): small enough to keep every file tiny,
# long enough that the ring contacts engage (rings_*_contact) and the pulls act.
REFERENCE_CASES = [
    ("rings_monaghan", 20, 12),
    ("rings_monaghan_contact", 20, 30),
    ("rings_tl_contact", 20, 375),
    ("tensile_tl", 11, 25),
    ("tensile_tl_weak", 7, 6),
    ("rings_corot_contact", 20, 480),
    ("tensile_corot", 11, 25),
    ("rotation_corot", 15, 400),
    ("rings_godunov", 20, 30),
    ("rings_godunov_contact", 20, 560),
    ("rotation_godunov", 15, 100),
    ("rings_potential_contact", 20, 5975),
    ("tensile_potential", 11, 25),
    ("rotation_potential", 15, 200),
    ("tensile_godunov", 11, 25),
    ("tensile_monaghan", 11, 25),
    ("rotation_monaghan", 15, 20),
    ("rotation_tl", 15, 100),
    ("tensile_ul_weak", 11, 25),
    ("rotation_ul_weak", 21, 50),
    ("rings_ul_weak_contact", 20, 450),
    ("tensile_tl_fem", 11, 25),
    ("rotation_tl_fem", 15, 50),
    ("rotation_tl_weak", 15, 50),
    ("rings_tl_fem_contact", 20, 450),
    ("rings_tl_weak_contact", 20, 450),
    ("tensile_ul_fem", 11, 25),
    ("rotation_ul_fem", 15, 50),
    ("rings_ul_fem_contact", 20, 450),
]


# cases whose final state is also stored as the reference's VTK output
VTK_CASES = ["tensile_tl", "rings_tl_contact"]


def write_vtk_goldens(ref):
    for name in VTK_CASES:
        with tempfile.TemporaryDirectory() as d:
            os.makedirs(os.path.join(d, "results"))
            subprocess.run([ref, "run", os.path.join(HERE, f"{name}.case"), os.path.join(d, "o.out"), d], check=True)
            (vtk,) = os.listdir(os.path.join(d, "results"))
            shutil.copy(os.path.join(d, "results", vtk), os.path.join(HERE, f"{name}.vtk"))
            print("wrote", name + ".vtk", "from", vtk)


def main():
    ref = oracle.build_ref(force=True)
    if ref is None:
        raise SystemExit("reference sources not present")
    if "--vtk-only" in sys.argv:
        write_vtk_goldens(ref)
        return
    only = [a for a in sys.argv[1:] if not a.startswith("--")]
    for name, nbox, steps in REFERENCE_CASES:
        if only and name not in only:
            continue
        case = os.path.join(HERE, f"{name}.case")
        out = os.path.join(HERE, f"{name}.ref.out")
        subprocess.run([ref, "scenario", name, str(nbox), str(steps), case, out], check=True)
        print("wrote", case, out)
    if only:
        return
    # workload constants (rho 1200, +-10 m/s, h = 1.3 dx, CFL dt) at dx = 4 mm
    sc = S.c1_rings(dx=4e-3, nbh_eps=1e-6)  # the reference predicate has a fixed 1e-6
    case = os.path.join(HERE, "c1_rings_dx4mm.case")
    S.write_case(case, sc, 30)
    subprocess.run([ref, "run", case, os.path.join(HERE, "c1_rings_dx4mm.ref.out")], check=True)
    sc = S.c2_rings_tl(dx=4e-3, nbh_eps=1e-6)
    case = os.path.join(HERE, "c2_rings_tl_dx4mm.case")
    S.write_case(case, sc, 30)
    subprocess.run([ref, "run", case, os.path.join(HERE, "c2_rings_tl_dx4mm.ref.out")], check=True)
    write_vtk_goldens(ref)
    print("done")


if __name__ == "__main__":
    main()
