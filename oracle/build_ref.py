"""Recipe: compile the reference's own Cython/C++ kernels into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this file or its
outputs.  The compiled modules let ``tests/golden/make_golden.py`` import the
reference package unmodified (with the shims in ``tests/golden/refshim``) to
produce golden fixtures, and let ``bench.py --impl reference`` time the
reference's own compiled solve kernels when they are present.

Sources are read where they lie in the reference checkout (``--src``, default
the ``REFERENCE_ROOT`` environment variable); nothing is copied into the
repository.  Outputs (generated C++ and shared objects) go only to
``oracle/_ref/``, which is git-ignored.

Modules built (the reference's ``setup.py:41-58`` list minus the ones off the
solve path):
  shenfun/optimization/cython/{la,transforms,Matvec,leg2chebm}.pyx  (C++)
  shenfun/legendre/fastgl/fastgl_wrap.pyx + fastgl.cpp    (C++)

The second stage (C++ -> .so) needs only g++, Python and numpy headers, so a
machine without Cython or the reference checkout can still finish a build from
the generated ``.cpp`` files (``--from-cpp``).
"""
import argparse
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

CY_MODULES = {
    # name: (pyx path relative to reference root, extra C++ sources)
    "la": ("shenfun/optimization/cython/la.pyx", []),
    "transforms": ("shenfun/optimization/cython/transforms.pyx", []),
    "Matvec": ("shenfun/optimization/cython/Matvec.pyx", []),
    # needed only because the reference's Legendre space plans a fast DLT
    # object on construction (legendre/bases.py:285, legendre/dlt.py:136)
    "leg2chebm": ("shenfun/optimization/cython/leg2chebm.pyx", []),
    # fastgl_wrap.pxd includes fastgl.cpp textually; only its directory is
    # needed on the include path.
    "fastgl_wrap": ("shenfun/legendre/fastgl/fastgl_wrap.pyx", []),
}


def ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def cythonize(src_root, name):
    pyx, _ = CY_MODULES[name]
    cpp = os.path.join(OUT, name + ".cpp")
    cmd = [sys.executable, "-m", "cython", "-3", "--cplus", "-o", cpp,
           os.path.join(src_root, pyx)]
    subprocess.run(cmd, check=True)
    return cpp


def compile_cpp(src_root, name):
    import numpy
    cpp = os.path.join(OUT, name + ".cpp")
    inc = [sysconfig.get_paths()["include"], numpy.get_include()]
    if src_root:
        inc.append(os.path.join(src_root, os.path.dirname(CY_MODULES[name][0])))
    so = os.path.join(OUT, name + ext_suffix())
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-std=c++14", "-w",
           "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION"]
    cmd += ["-I" + i for i in inc] + [cpp] + ["-o", so, "-lm"]
    subprocess.run(cmd, check=True)
    return so


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=os.environ.get("REFERENCE_ROOT") or os.path.normpath(os.path.join(
        os.path.dirname(os.path.dirname(OUT)), os.pardir, "reference")),
        help="reference checkout (default: REFERENCE_ROOT, else a 'reference' checkout beside the repository)")
    ap.add_argument("--from-cpp", action="store_true",
                    help="skip Cython; compile existing oracle/_ref/*.cpp")
    ap.add_argument("--only", nargs="*", default=None)
    args = ap.parse_args(argv)
    os.makedirs(OUT, exist_ok=True)
    names = args.only or list(CY_MODULES)
    if not args.from_cpp:
        if not os.path.isdir(args.src):
            print(f"reference checkout not found at {args.src}; nothing to build")
            return 1
        with ThreadPoolExecutor(len(names)) as ex:
            list(ex.map(lambda n: cythonize(args.src, n), names))
    with ThreadPoolExecutor(len(names)) as ex:
        list(ex.map(lambda n: compile_cpp(args.src, n), names))
    print("built:", ", ".join(names), "->", OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main())
