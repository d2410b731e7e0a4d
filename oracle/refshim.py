"""Import the reference's torch-only hot-path modules under import shims
(oracle, test-only; used by tests/golden/make_golden.py in a container where
the reference sources are present — never on the GPU machine).

The reference's third-party dependencies (quimb, symmray, cotengra, mpi4py,
pyblock2, pyinstrument) are not installed.  None of them is on the Slater /
NNBF / Hubbard hot path, so they are replaced by MagicMock modules; autoray is
replaced by a small numpy/torch dispatcher; ``quimb.tensor.edges_2d_square`` is
replaced by the cell-order edge list of ``oracle.lattice.square_edges``.
"""
import importlib
import importlib.abc
import importlib.machinery
import os
import sys
import types
from unittest import mock

import numpy

# the reference checkout to import from: required, no default location
REFERENCE_ROOT = os.environ.get("VMC_REFERENCE_ROOT")
_STUB = ("quimb", "symmray", "cotengra", "mpi4py", "pyblock2", "pyinstrument")


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path, target=None):
        if name.split(".")[0] in _STUB:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = mock.MagicMock(name=spec.name)
        m.__path__ = []
        m.__spec__ = spec
        return m

    def exec_module(self, module):
        pass


_installed = False
# optional packages the reference imports at module level: stubbed only where
# they are not installed (the GPU host ships without them)
_OPTIONAL = ("tqdm",)


def install(root=None):
    """Install the shims and put the reference on sys.path (idempotent).
    root: the directory holding the ``vmc_torch`` package (a checkout, or a
    pip --target install); default VMC_REFERENCE_ROOT."""
    global _installed
    if _installed:
        return
    root = root or REFERENCE_ROOT
    if not root or not os.path.isdir(os.path.join(root, "vmc_torch")):
        raise RuntimeError("give the directory holding the reference's vmc_torch package (argument or "
                           "VMC_REFERENCE_ROOT) to import the reference")
    import torch
    global _STUB
    missing = []
    for name in _OPTIONAL:
        try:
            importlib.import_module(name)
        except ImportError:
            missing.append(name)
    _STUB = _STUB + tuple(missing)

    sys.meta_path.insert(0, _StubFinder())
    ar = types.ModuleType("autoray")
    ar.numpy = numpy

    def do(fn, *a, **k):
        lib = torch if any(isinstance(x, torch.Tensor) for x in a) else numpy
        obj = lib
        for p in fn.split("."):
            obj = getattr(obj, p)
        return obj(*a, **k)

    ar.do = do
    sys.modules["autoray"] = ar
    sys.path.insert(0, root)
    import quimb.tensor as qtn  # the MagicMock stub
    from .lattice import square_edges

    def edges_2d_square(Lx, Ly, cyclic=False, cells=None):
        assert not cyclic
        out = []
        for (i, j) in square_edges(Lx, Ly):
            out.append((divmod(i, Ly), divmod(j, Ly)))
        return out

    qtn.edges_2d_square = edges_2d_square
    _installed = True


def load(modname, root=None):
    install(root)
    return importlib.import_module(modname)
