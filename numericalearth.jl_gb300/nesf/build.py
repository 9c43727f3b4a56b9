"""In-tree build of libnesf.so (the CUDA kernels + C ABI) for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked with the static CUDA runtime into `nesf/libnesf.so`. Rebuilds only when
a source or header is newer than the library.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libnesf.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# The streaming kernels (interpolation, sea-ice-ocean fluxes, assembly) are HBM-bound:
# without contracted multiply-adds they round exactly like the CPU restatement.
# The interface solves' FP32 arithmetic -- the adaptive solver's FP32 sweep, its FP32 flux
# epilogue, the classify passes' features -- uses the hardware's approximate division,
# square root, logarithm and exponential (FP32 denormals flushed): the sweep's own
# tests of convergence and conditioning decide which FP32 results are kept, and the
# cells they do not keep are polished or replayed in FP64, whose arithmetic these flags
# do not touch (the plain FP64 path, the polish's Newton steps and the replays are
# unchanged). Measured on the 1/8-degree step: 6.70 -> 5.77 ms, the largest error
# against the FP64 oracle 4.3e-6 both ways.
FAST_FP32 = ["--use_fast_math"]
PER_FILE_FLAGS = {"nesf_exchange.cu": ["-fmad=false"], "nesf_ao.cu": FAST_FP32, "nesf_ai.cu": FAST_FP32,
                  "nesf_df.cu": FAST_FP32}
# The solve files instantiate every kernel for FP64 and FP32 storage: each is compiled
# twice, one storage type per object, so the slowest translation unit takes half as long.
SPLIT_BY_STORAGE = ("nesf_ao.cu", "nesf_ai.cu", "nesf_al.cu")
# The two interface solves are split once more: their double-float replay kernels
# (NESF_DF_PART 1) compile apart from the other kernels (NESF_DF_PART 0).
SPLIT_DF_PART = ("nesf_ao.cu", "nesf_ai.cu")


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnesf.so")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, jobs=None):
    """Compile and link libnesf.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    srcs = sources()

    units = []
    for src in srcs:
        base = os.path.basename(src)[:-3]
        if os.path.basename(src) in SPLIT_DF_PART:
            units += [(src, [f"-DNESF_STORAGE={b}", f"-DNESF_DF_PART={d}"], f"{base}.f{b}.p{d}.o")
                      for b in (64, 32) for d in (0, 1)]
        elif os.path.basename(src) in SPLIT_BY_STORAGE:
            units += [(src, [f"-DNESF_STORAGE={b}"], f"{base}.f{b}.o") for b in (64, 32)]
        else:
            units.append((src, [], base + ".o"))

    def compile_one(unit):
        src, defs, name = unit
        obj = os.path.join(BUILD, name)
        cmd = [exe, *ARCH, *NVCC_FLAGS, *PER_FILE_FLAGS.get(os.path.basename(src), []), *defs, "-I", INCLUDE, "-c",
               src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    # slowest first, so the long units start at once when there are fewer cores than units
    units.sort(key=lambda u: (os.path.basename(u[0]) not in SPLIT_BY_STORAGE, "-DNESF_DF_PART=1" not in u[1]))
    with ThreadPoolExecutor(max_workers=jobs or max(1, min(len(units), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
