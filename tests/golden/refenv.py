"""Import the reference DFTpy in this container (golden-fixture generation).

Only ``tests/golden/make_golden.py`` uses this.  It puts the two shims
(``_shims/ase`` and the ``dcsrch`` adapter) and the reference sources on
``sys.path``.  The reference tree is not present where the GPU tests run;
nothing there imports this module.
"""
import os
import pathlib
import sys

HERE = pathlib.Path(__file__).resolve().parent
REF_SRC = pathlib.Path(os.environ.get("DFTPY_REFERENCE_SRC", "/root/reference/src"))
REF_DATA = REF_SRC.parent / "examples" / "DATA"


def load():
    os.environ.setdefault("DFTPY_LOGLEVEL", "4")
    os.environ.setdefault("DFTPY_FFTLIB", "numpy")
    shims = str(HERE / "_shims")
    if shims not in sys.path:
        sys.path.insert(0, shims)
    import dcsrch_adapter
    dcsrch_adapter.install()
    if str(REF_SRC) not in sys.path:
        sys.path.insert(1, str(REF_SRC))
    import dftpy  # noqa: F401
    return dftpy
