"""In-tree build of libflowket_gb300.so for sm_103a (nvcc, no cmake).

Every translation unit under csrc/ is compiled in parallel to
_build/*.o (the AR2D machine's twice: BF16 and FP16 tensor-core operands)
and linked into flowket_gb300/libflowket_gb300.so.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflowket_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
         "-I" + CSRC]


def _nvcc():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build flowket_gb300")
    return nvcc


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


# Translation units of the AR2D machine: compiled a second time with
# FK_TC_FP16 (FP16 tensor-core operands, namespace fk16, entry points
# fk_ar2d_*_tc_fp16).
TWO_FORMATS = ("fk_ar2d.cu", "fk_ar2d_pipe.cu", "fk_ar2d_bwd.cu", "fk_ar2d_bwd_tc.cu")


def objects():
    """(source, object, extra flags) of every compilation."""
    out = []
    for src in sources():
        base = os.path.basename(src)[:-3]
        out.append((src, os.path.join(BUILD, base + ".o"), []))
        if os.path.basename(src) in TWO_FORMATS:
            out.append((src, os.path.join(BUILD, base + "_fp16.o"), ["-DFK_TC_FP16"]))
    return out


def build(verbose=False, force=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "flowket_gb300.h"))
    jobs = []
    for src, obj, extra in objects():
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + ARCH + FLAGS + extra + ["-c", src, "-o", obj])
    objs = [obj for _, obj, _ in objects()]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
