"""Import the unmodified reference package (shenfun) in this container.

TEST INFRASTRUCTURE ONLY (fixture generation; never used by the product or on
the GPU machine).  Puts the single-process shims of ``refshim/`` on sys.path,
maps ``shenfun.optimization.cython.*`` and ``shenfun.legendre.fastgl.fastgl_wrap``
onto the reference's own Cython kernels compiled by ``oracle/build_ref.py`` into
``oracle/_ref/``, and imports shenfun from the reference checkout
(``REFERENCE_ROOT``, else a checkout named ``reference`` beside this
repository).
"""
import importlib.abc
import importlib.machinery
import importlib.util
import os
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_ROOT = os.environ.get("REFERENCE_ROOT") or os.path.normpath(os.path.join(REPO, os.pardir, "reference"))
REF_BUILD = os.path.join(REPO, "oracle", "_ref")

_MAP = {
    "shenfun.optimization.cython.la": "la",
    "shenfun.optimization.cython.transforms": "transforms",
    "shenfun.optimization.cython.Matvec": "Matvec",
    "shenfun.optimization.cython.leg2chebm": "leg2chebm",
    "shenfun.legendre.fastgl.fastgl_wrap": "fastgl_wrap",
}


class _CompiledRefFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path=None, target=None):
        short = _MAP.get(fullname)
        if short is None:
            # Cython modules that are off the solve path are not built; let
            # the cython package import fail cleanly for them.
            return None
        so = os.path.join(REF_BUILD, short + sysconfig.get_config_var("EXT_SUFFIX"))
        if not os.path.exists(so):
            return None
        loader = importlib.machinery.ExtensionFileLoader(fullname, so)
        return importlib.util.spec_from_file_location(fullname, so, loader=loader)


class _StubCythonPackage(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    """``shenfun.optimization.cython/__init__.py`` imports every Cython module,
    including ones off the solve path that are not built; replace the package
    init with one that exposes just the built modules' names."""

    def find_spec(self, fullname, path=None, target=None):
        if fullname == "shenfun.optimization.cython":
            spec = importlib.util.spec_from_loader(fullname, self, is_package=True)
            spec.submodule_search_locations = [
                os.path.join(REF_ROOT, "shenfun", "optimization", "cython")]
            return spec
        return None

    def create_module(self, spec):
        return None

    def exec_module(self, module):
        la = importlib.import_module("shenfun.optimization.cython.la")
        mv = importlib.import_module("shenfun.optimization.cython.Matvec")
        tr = importlib.import_module("shenfun.optimization.cython.transforms")
        for mod in (la, mv):
            for k in dir(mod):
                if not k.startswith("_"):
                    setattr(module, k, getattr(mod, k))
        for k in ("evaluate_expansion_all", "scalar_product", "restricted_product",
                  "Lambda", "leg2cheb", "cheb2leg"):
            if hasattr(tr, k):
                setattr(module, k, getattr(tr, k))
        l2c = importlib.import_module("shenfun.optimization.cython.leg2chebm")
        module.Leg2Cheb = l2c.Leg2Cheb
        module.Cheb2Leg = l2c.Cheb2Leg
        module.leg2chebm = l2c
        module.transforms = tr
        module.la = la
        module.Matvec = mv


def import_reference():
    sys.dont_write_bytecode = True
    if "shenfun" in sys.modules:
        return sys.modules["shenfun"]
    shim = os.path.join(HERE, "refshim")
    if shim not in sys.path:
        sys.path.insert(0, shim)
    if REF_ROOT not in sys.path:
        sys.path.insert(1, REF_ROOT)
    sys.meta_path.insert(0, _CompiledRefFinder())
    sys.meta_path.insert(0, _StubCythonPackage())
    os.environ.setdefault("pytest", "True")
    import shenfun  # noqa: E402
    return shenfun


if __name__ == "__main__":
    sf = import_reference()
    print("imported reference shenfun", sf.__version__, sf.__file__)
