"""Builds the CUDA extension: libmfree_gb300.so, in-tree next to this file.

Every kernel translation unit is compiled twice -- namespace mf_strict with
--fmad=false (the FP64 parity form: no a*b+c contraction) and namespace mf_fast
with contraction allowed -- for sm_103a only, in parallel, then linked with the
host-side C ABI (csrc/mf_api.cu) into one shared library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfree_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
KERNEL_TUS = ["mf_ul.cu", "mf_tl.cu", "mf_contact.cu", "mf_weak.cu", "mf_corot.cu", "mf_ulweak.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def _newer(out: str, deps) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "mfree_gb300.h"))
    base = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
            "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for tu in KERNEL_TUS:
        for ns, fmad in (("mf_strict", "false"), ("mf_fast", "true")):
            src = os.path.join(CSRC, tu)
            obj = os.path.join(BUILD, f"{tu[:-3]}_{ns}.o")
            strict = "1" if ns == "mf_strict" else "0"
            jobs.append((src, obj, base + [f"-DMF_NS={ns}", f"-DMF_STRICT_FORM={strict}", f"--fmad={fmad}", src, "-o", obj]))
    for host_tu in ("mf_api.cu", "mf_noalloc.cu", "mf_mlp.cu"):
        src = os.path.join(CSRC, host_tu)
        obj = os.path.join(BUILD, host_tu[:-3] + ".o")
        jobs.append((src, obj, base + [src, "-o", obj]))

    def run(job):
        s, o, cmd = job
        if not force and _newer(o, [s] + headers):
            return o, 0, ""
        r = subprocess.run(cmd, capture_output=True, text=True)
        return o, r.returncode, r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=min(len(jobs), max(2, os.cpu_count() or 2))) as ex:
        results = list(ex.map(run, jobs))
    for o, rc, log in results:
        if rc != 0:
            raise RuntimeError(f"nvcc failed for {o}:\n{log}")
        if verbose and log:
            print(log)
    objs = [o for o, _, _ in results]
    if force or not _newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
