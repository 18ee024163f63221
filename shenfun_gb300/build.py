"""Build the in-tree CUDA library ``shenfun_gb300/libshenfun_gb300.so``.

Plain nvcc, one translation unit per ``csrc/*.cu`` compiled in parallel, then
one shared-library link.  Device code is generated for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``).  A stamp of the sources and
flags skips the rebuild when nothing changed.
"""
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshenfun_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + os.path.join(REPO, "include")]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build shenfun_gb300")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def stamp():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)) + ["../../include/shenfun_gb300.h"]:
        p = os.path.join(CSRC, f)
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(verbose=False, force=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    st = stamp() + "|" + " ".join(extra_flags)
    stamp_file = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read() == st:
                return LIB
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src[:-3] + ".o")
        cmd = [exe, "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + FLAGS + list(extra_flags)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [exe, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as fh:
        fh.write(st)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
