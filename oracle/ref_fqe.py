"""Import the reference FQE package (test infrastructure only).

This module is part of the oracle: it lets fixture-generation scripts and the
CPU-only pin tests import the unmodified reference Python package
(``src/fqe`` of OpenFermion-FQE 0.3.0) together with its own C library and
Cython extension, compiled from the reference sources by ``make -C oracle ref``
into ``oracle/_ref/``.  Nothing in the GPU product imports it.

Two things the reference needs are not installed here:

* ``openfermion``, ``cirq`` and ``cirq_google`` are imported at module level
  (``_fqe_control.py:22-27``, ``lib/_fqe_data.pyx:22``).  A meta-path finder
  serves inert stand-in modules for them; ``up_index(i) = 2 i`` and
  ``down_index(i) = 2 i + 1`` follow OpenFermion's spin-orbital convention.
  Tests of the reference that build operators through OpenFermion cannot run
  under the stand-ins; none of them is on the H·psi path.
* ``fqe/lib/__init__.py`` loads ``libfqe.so`` from its own directory, which is
  read-only in the reference tree.  The finder therefore provides the
  ``fqe.lib`` package object itself: it opens ``oracle/_ref/libfqe.so`` and
  searches both the reference's ``lib`` directory (pure-Python wrappers) and
  ``oracle/_ref`` (the compiled ``fqe_data`` extension) for submodules.
"""

import ctypes
import importlib.abc
import importlib.machinery
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
# FQE_REFERENCE_ROOT, else a checkout named `reference` beside the repository
REF_ROOT = os.environ.get("FQE_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
REF_SRC = os.path.join(REF_ROOT, "src")


def available() -> bool:
    """True when both the reference sources and the built natives exist."""
    return (os.path.isdir(os.path.join(REF_SRC, "fqe"))
            and os.path.exists(os.path.join(REF_OUT, "libfqe.so")))


class _Inert(types.ModuleType):
    """Stand-in module: every attribute is a do-nothing class."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        if name == "up_index":
            return lambda i: 2 * i
        if name == "down_index":
            return lambda i: 2 * i + 1
        cls = type(name, (), {
            "__init__": lambda s, *a, **k: None,
            "__call__": lambda s, *a, **k: None,
        })
        setattr(self, name, cls)
        return cls


class _c_double_complex(ctypes.Structure):
    _fields_ = [("real", ctypes.c_double), ("imag", ctypes.c_double)]

    @property
    def value(self):
        return self.real + 1j * self.imag


class _Finder(importlib.abc.MetaPathFinder, importlib.abc.Loader):

    def find_spec(self, fullname, path, target=None):
        top = fullname.split(".")[0]
        if top in ("openfermion", "cirq", "cirq_google"):
            return importlib.machinery.ModuleSpec(fullname, self,
                                                  is_package=True)
        if fullname == "fqe.lib":
            return importlib.machinery.ModuleSpec(fullname, self,
                                                  is_package=True)
        return None

    def create_module(self, spec):
        if spec.name == "fqe.lib":
            mod = types.ModuleType("fqe.lib")
            mod.__path__ = [os.path.join(REF_SRC, "fqe", "lib"), REF_OUT]
            mod.lib_fqe = ctypes.cdll.LoadLibrary(
                os.path.join(REF_OUT, "libfqe.so"))
            mod.c_double_complex = _c_double_complex
            return mod
        mod = _Inert(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        pass


_installed = False


def import_fqe():
    """Return the reference ``fqe`` package (raises if it is unavailable)."""
    global _installed
    if not available():
        raise ImportError("reference FQE or oracle/_ref natives not present")
    if not _installed:
        sys.meta_path.insert(0, _Finder())
        if REF_SRC not in sys.path:
            sys.path.insert(0, REF_SRC)
        _installed = True
    import fqe  # noqa: E402  (the reference package)
    return fqe
