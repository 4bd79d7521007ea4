"""cppe_gb300 -- GB300-native induced-dipole path of CPPE.

Drop-in for the reference's ``cppe`` Python package on the polarizable-embedding
hot path (``CppeState``, ``BMatrix``, ``InducedMoments``, ``MultipoleFields``,
``PotfileReader`` ... with the same names and arguments), backed by CUDA kernels
for sm_103a behind the C ABI of ``include/cppe_gpu.h``::

    import cppe_gb300 as cppe
    state = cppe.CppeState({"potfile": "water.pot"}, mol, print)

The native module is built in-tree by ``cppe_gb300._build.build()``.  There is
no CPU fallback: without the built module every public name raises
ImportError, and operations that need the GPU raise RuntimeError when no CUDA
device is present.
"""
import importlib as _importlib
import os as _os

_here = _os.path.dirname(_os.path.abspath(__file__))
__version__ = "0.1.0"
LIBRARY_PATH = _os.path.join(_here, "libcppe_gpu.so")

# The native module (and with it libcppe_gpu.so) loads on the first access to
# one of its names, not at package import: the package's pure-Python modules
# (``synthetic``, the seeded input generators) stay usable without mapping the
# CUDA library.
_PY_SUBMODULES = {"synthetic", "capi", "learned", "shard"}
_native = None
_IMPORT_ERROR = None


def _load_native():
    global _native, _IMPORT_ERROR
    if _native is None:
        try:
            _native = _importlib.import_module(".pycppe", __name__)
        except ImportError as e:  # only before the in-tree build has run
            _IMPORT_ERROR = e
            raise ImportError(
                "cppe_gb300: the native module is not built "
                "(run `python -c 'import __graft_entry__ as g; g.build()'`, needs nvcc)") from e
    return _native


def __getattr__(name):
    if name.startswith("_") and name not in ("__build_type__", "__parallel__"):
        raise AttributeError(name)  # private names and submodules such as _build
    if name in _PY_SUBMODULES:
        raise AttributeError(name)  # let the import system load the submodule
    native = _load_native()
    # the reference package also re-exports its tensors submodule at the top
    # level (src/cppe/__init__.py:3)
    for src in (native, native.tensors):
        if hasattr(src, name):
            value = getattr(src, name)
            break
    else:
        raise AttributeError(f"module 'cppe_gb300' has no attribute '{name}'") from None
    globals()[name] = value
    return value


def __dir__():
    names = set(globals())
    if _native is not None:
        names.update(n for n in dir(_native) if not n.startswith("_"))
        names.update(n for n in dir(_native.tensors) if not n.startswith("_"))
    return sorted(names)


__all__ = ["__build_type__", "__parallel__", "__version__"]
