"""GB300-native per-cell hot path of the EdynCFD 1-D reacting-flow solver.

The compute lives in ``_lib/libedyn_gb300.so`` (sm_103a CUDA kernels behind
the C ABI of ``include/edyn_gpu.h``); this package is its Python host side.
"""
from .edyn import (GRI30_DIR, Blocks, EdynError, Reactors, Tube, Tubes, lib, lvir_for, mech_compile,  # noqa: F401
                   species_names, tran_compile)

__all__ = ["Tube", "Tubes", "Blocks", "Reactors", "EdynError", "lib", "mech_compile", "tran_compile", "species_names",
           "lvir_for", "GRI30_DIR"]
