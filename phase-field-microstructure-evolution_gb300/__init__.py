"""GB300-native semi-implicit spectral phase-field step (drop-in for the time
step of var_diff.x from smjim/phase-field-microstructure-evolution).

The compute path is the CUDA library ``libpfgpu.so`` (``csrc/``, C ABI in
``include/pfgpu.h``); this package holds its build recipe, the ctypes binding
and the host-side mirror of the reference's input/output files.  There is no
CPU fallback: every entry point fails loudly when the library or a GPU is
missing.
"""
from . import build as build_mod
from .pfgpu import (Batch, Config, Diag, PFError, Ran2, Run, load_library, library_path, make_config,
                    ic_noise, ic_voronoi, ic_noise_aos, ic_voronoi_aos, to_aos, from_aos,
                    PF_FP32_FUSED, PF_FP64_PLAIN, PF_MOB_C1MC, PF_MOB_REFERENCE, EXPORTED,
                    PF_OK, PF_EINVAL, PF_ECUDA, PF_ENOMEM, PF_ENONFINITE, PF_EIO,
                    Input, read_input, input_to_config, write_data_save, read_data_save, ic_circle, ic_plane,
                    ic_polycryst, insert_precipitates, format_e, format_summary, format_list_int,
                    format_list_real, driver_path, VoxelCounts, AnalysisOut, analyze_fields, analyze_run,
                    write_vtk, paraview_path, sweep, sweep_path, variant_counts, Server, ServerConfig,
                    RequestTimes, Pool, place_units, pick_device, check_fp64, ErrorReport, PF_EBUSY, PF_REQ_QUEUED, PF_REQ_RUNNING, PF_REQ_DONE, PF_REQ_FAILED)


def build(force: bool = False, verbose: bool = False):
    """Compile libpfgpu.so for sm_103a (in-tree, ``_build/``)."""
    return build_mod.build(force=force, verbose=verbose)
