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
import os as _os

_here = _os.path.dirname(_os.path.abspath(__file__))
__version__ = "0.1.0"
LIBRARY_PATH = _os.path.join(_here, "libcppe_gpu.so")

try:
    from .pycppe import *  # noqa: F401,F403
    from .pycppe import __build_type__, __parallel__  # noqa: F401
    _IMPORT_ERROR = None
except ImportError as _e:  # only before the in-tree build has run
    _IMPORT_ERROR = _e

    def __getattr__(name):
        if name.startswith("_"):  # submodules such as _build stay importable
            raise AttributeError(name)
        raise ImportError(
            f"cppe_gb300.{name}: the native module is not built "
            "(run `python -c 'import __graft_entry__ as g; g.build()'`, needs nvcc)"
        ) from _IMPORT_ERROR

__all__ = ["__build_type__", "__parallel__", "__version__"]
