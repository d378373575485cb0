"""FP64 CPU oracle for the sarlab-tdc focus path -- TEST INFRASTRUCTURE ONLY.

Imported by ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
reference arm of ``bench.py`` to check and time against. The product library never
imports, links or calls anything here.
"""
from .oracle import (  # noqa: F401
    Problem,
    Opts,
    focus,
    adjoint_offsets,
    range_window,
    wavelength_center,
    window_is_nonzero,
    skip_row_pri,
    skip_points,
    lib,
    refmath,
)
