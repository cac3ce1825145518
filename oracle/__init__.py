"""ORACLE -- test infrastructure only (tests, smoke check, CPU-baseline leg of the bench).

Builds and runs the CPU restatement of the reference's time step (oracle/mfo.cpp) and,
where the reference sources are present, the reference itself compiled out of tree
(oracle/build_ref.sh -> oracle/_ref/ref_harness).  The product never imports this."""
from __future__ import annotations

import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
MFO = os.path.join(HERE, "mfo_run")
REF = os.path.join(HERE, "_ref", "ref_harness")


def build_oracle(force: bool = False) -> str:
    """Compile the restatement (g++, -ffp-contract=off so x86-64 and aarch64 agree)."""
    src = [os.path.join(HERE, f) for f in ("mfo.cpp", "mfcase.h")] + [os.path.join(HERE, "glm_subset", "glm", "glm.hpp")]
    if not force and os.path.exists(MFO) and all(os.path.getmtime(s) <= os.path.getmtime(MFO) for s in src):
        return MFO
    cmd = ["g++", "-std=c++14", "-O3", "-ffp-contract=off", "-I", os.path.join(HERE, "glm_subset"),
           "-o", MFO, os.path.join(HERE, "mfo.cpp")]
    subprocess.run(cmd, check=True)
    return MFO


def build_ref(force: bool = False, root: str | None = None) -> str | None:
    """Compile the reference (only where its sources are present).  The sources' root
    is `root`, else the environment variable MF_REFERENCE_ROOT, else the default of
    build_ref.sh; returns None when no sources are found there."""
    if os.path.exists(REF) and not force:
        return REF
    root = root or os.environ.get("MF_REFERENCE_ROOT")
    cmd = [os.path.join(HERE, "build_ref.sh")] + ([root] if root else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode == 3:  # no reference sources on this machine
        return None
    if r.returncode != 0:
        raise RuntimeError(f"building the reference failed:\n{r.stdout}{r.stderr}")
    return REF


def run_case_file(case_path: str, out_path: str, binary: str = MFO, timeout: float = 3600) -> int:
    return subprocess.run([binary, case_path, out_path], capture_output=True, timeout=timeout).returncode


def run(scenario, nsteps: int, dump_every: int = 0, binary: str | None = None):
    """Run a Scenario through the oracle and return its Result."""
    from mfree_iwf_gb300 import scenarios as S

    binary = binary or build_oracle()
    with tempfile.TemporaryDirectory() as d:
        cp, op = os.path.join(d, "c.case"), os.path.join(d, "o.out")
        S.write_case(cp, scenario, nsteps, dump_every)
        if binary == REF:
            rc = subprocess.run([binary, "run", cp, op], capture_output=True).returncode
        else:
            rc = run_case_file(cp, op, binary)
        res = S.read_result(op)
        if rc != 0:
            res.ok = False
        return res
