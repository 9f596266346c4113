"""Oracle package -- TEST INFRASTRUCTURE ONLY.

Holds the CPU checkers for the sparse gate path: a C restatement of the reference's FC
gate algorithm (``sparse``), an independent dense FP64 statevector (``dense``), and the
host emulation of the reference's own kernels (``refemu``, built only where the reference
sources are present). Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg may import this package; the product never does.
"""
