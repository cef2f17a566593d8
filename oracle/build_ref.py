"""Build recipe for oracle/_ref: the reference's own hot-path headers, compiled
from where they lie (<reference tree>/src), wrapped by
oracle/ref_harness{2d,3d}.cpp.  Test infrastructure only.

Compiled with g++ -O2 -ffp-contract=off (FMA contraction off, the setting under
which the restatement in oracle/pfast_oracle.cpp is bit-identical).  The 2D and
3D headers define the same helper symbols (swap, notin, readmod, ...), so each
goes into its own shared object.  Nothing is copied out of the reference tree;
outputs go only to oracle/_ref/.  Exits quietly (returns None) when the
reference tree is absent.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def ref_root():
    """The reference tree: $PFAST_REF_ROOT, else a `reference` folder beside the checkout."""
    return os.environ.get("PFAST_REF_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build(verbose=False):
    src = os.path.join(ref_root(), "src")
    if not os.path.isfile(os.path.join(src, "T_pfsm3d.h")):
        return None
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for dim in ("2d", "3d"):
        out = os.path.join(OUT, f"libpfast_ref{dim}.so")
        cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-I", src,
               os.path.join(HERE, f"ref_harness{dim}.cpp"), os.path.join(src, "fftn.cpp"),
               "-o", out]
        jobs.append(cmd)
    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    with ThreadPoolExecutor(2) as ex:
        list(ex.map(run, jobs))
    return OUT


if __name__ == "__main__":
    r = build(verbose=True)
    print("built" if r else "reference tree absent: nothing built", r or "")
    sys.exit(0)
