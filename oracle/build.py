"""Build recipe of the CPU oracle (liboracle.so) -- test infrastructure only.

    python oracle/build.py

compiles oracle/nesf_oracle.c with gcc into oracle/_build/liboracle.so, with
OpenMP (the timed CPU baseline uses every host core) and without contraction
of multiply-adds, so the same source gives the same results on x86-64 and
aarch64 hosts. The reference itself is Julia and cannot be compiled here; the
oracle is its C restatement.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = [os.path.join(HERE, "nesf_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "nesf_oracle.h"), os.path.join(os.path.dirname(HERE), "include", "nesf.h"),
              os.path.abspath(__file__)]


def build(force=False):
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in DEPS):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB + ".tmp"
    cmd = [cc, "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-o", tmp, *SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
