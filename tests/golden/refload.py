"""Import the PtyLab.py reference in a container that lacks its GUI/HDF5 dependencies.

Test infrastructure only: this module is used by ``make_golden.py`` to run the
reference's own NumPy code path and record golden fixtures.  It is never
imported by the package, by ``bench.py`` or by the GPU tests, and it needs the
reference source tree, which exists only where the fixtures are generated.

The reference imports ``h5py``, ``tables``, ``matplotlib``, ``IPython``,
``skimage``, ``pyqtgraph``, ``cupy`` and ``tensorflow`` at module level, none of
which sit on the numerical path of the engines (ePIE.py, mPIE.py, qNewton.py,
e3PIE.py, BaseEngine.py, Operators.py, utils.py).  They are replaced by inert
stub modules; ``cupy`` is deliberately left missing so that every array module
lookup resolves to NumPy (``PtyLab/utils/gpuUtils.py:8-27``).
"""

from __future__ import annotations

import importlib.abc
import importlib.machinery
import os
import sys
import types

STUB_ROOTS = (
    "h5py",
    "tables",
    "matplotlib",
    "mpl_toolkits",
    "IPython",
    "skimage",
    "pyqtgraph",
    "tensorflow",
    "napari",
    "bokeh",
)


class _Anything:
    """Callable, subscriptable, attribute-rich placeholder."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Anything()

    def __getitem__(self, item):
        return _Anything()

    def __iter__(self):
        return iter(())

    def __bool__(self):
        return False


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Anything


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path=None, target=None):
        if fullname.split(".")[0] in STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        return None


_installed = False


def load_reference(root: str):
    """Put the reference at ``root`` on ``sys.path`` behind the stubs; return the ``PtyLab`` package."""
    global _installed
    os.environ.setdefault("TQDM_DISABLE", "1")
    if not _installed:
        for name in list(sys.modules):
            if name.split(".")[0] in STUB_ROOTS:
                del sys.modules[name]
        sys.meta_path.insert(0, _StubFinder())
        _installed = True
    if root not in sys.path:
        sys.path.insert(0, root)
    import logging

    import PtyLab  # noqa: F401

    logging.disable(logging.WARNING)
    return PtyLab
