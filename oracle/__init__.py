"""CPU FP64 oracle for the OF-DFT hot path (test infrastructure only).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` import it.  The product (``dftpy_gb300``) runs on the GPU
and fails loudly when its CUDA library is missing.

``ofdft`` restates, in numpy, each reference function on the path
(DFTpy 2.1.1rc0, ``src/dftpy/...``; every function cites the file:line it
follows).  It is pinned against fixtures generated by running the reference
itself (``tests/golden/make_golden.py``): the reference's own test values
(WT 2.916818700014412, Ewald terms) and full TN solves.
"""
