"""GB300-native per-cell hot path of the EdynCFD 1-D reacting-flow solver.

The compute lives in ``_lib/libedyn_gb300.so`` (sm_103a CUDA kernels behind
the C ABI of ``include/edyn_gpu.h``); this package is its Python host side.
"""
from .edyn import (GRI30_DIR, OUTPUT_FIELDS, Blocks, EdynError, H5Writer, Reactors, Tube, Tubes, h5_attr,  # noqa: F401
                   h5_attr_names, h5_list, h5_read, lib, lvir_for, mech_compile, output_path, species_names,
                   step_group_name, tran_compile)

__all__ = ["Tube", "Tubes", "Blocks", "Reactors", "EdynError", "lib", "mech_compile", "tran_compile", "species_names",
           "lvir_for", "GRI30_DIR", "OUTPUT_FIELDS", "H5Writer", "h5_list", "h5_read", "h5_attr", "h5_attr_names",
           "output_path", "step_group_name"]
