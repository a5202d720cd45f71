"""GB300-native orbital-free DFT: DFTpy's energy/potential evaluation and
direct density optimisation on hand-written sm_103a CUDA kernels.

The Python classes keep DFTpy's interface (``DirectGrid``, ``DirectField``,
``Functional``, ``TotalFunctional``, ``LocalPseudo``, ``Optimization``); the
work runs in ``libgbofdft.so`` through its C ABI (``include/gbofdft.h``).
There is no CPU fallback: without the library or a CUDA device the calls
raise.
"""
__version__ = "0.1.0"

from . import _lib  # noqa: F401


def __getattr__(name):
    # lazy imports keep `import dftpy_gb300` free of torch/CUDA initialisation
    if name in ("DirectGrid", "ReciprocalGrid"):
        from . import grid
        return getattr(grid, name)
    if name in ("DirectField", "ReciprocalField"):
        from . import field
        return getattr(field, name)
    if name == "Ions":
        from .ions import Ions
        return Ions
    if name == "Optimization":
        from .optimization import Optimization
        return Optimization
    raise AttributeError(name)
