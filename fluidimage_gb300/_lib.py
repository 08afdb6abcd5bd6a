"""ctypes binding of ``libfluidimage_gb300.so`` (the C ABI in include/fluidimage_gb300.h).

The library is built in-tree by ``fluidimage_gb300.build``; loading fails loudly
when it is missing — there is no fallback implementation.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

FI_OK = 0
FI_U8, FI_U16, FI_F32 = 0, 1, 2

VEC_OK = 0
VEC_PEAK_BOUNDARY = 1
VEC_PEAK_NAN = 2
VEC_WRONG_SUBPIX = 3
VEC_BAD_CROP = 4
VEC_ALL_NAN = 5
VEC_CLOSE_BOUNDARY = 6

FLAG_NEAR_TIE = 1
FLAG_SUBPIX_TIE = 2
FLAG_SECONDARY_TIE = 4

FIX_CORREL_MIN = 1
FIX_DISPLACEMENT = 2
FIX_NEIGHBOUR = 4
FIX_REPLACED = 8
FIX_STATIC_MAX_VECTORS = 262144

SUBPIX_METHODS = {"2d_gaussian2": 0, "2d_gaussian": 1, "centroid": 2, "no_subpix": 3}
#: precision forms of the tensor-core pass (FI_TC_*)
TC_FORMS = {"bf16x1": 0, "bf16x3": 1, "fp16x3": 2}
#: window size of the tensor-core pass
TC_WINDOW = 32
#: windows per work item of the batch kernel, per window size (autotuner choices)
BATCH_WPB = {8: (16, 8), 12: (16, 8), 16: (16, 8), 24: (8, 4), 32: (8, 4), 48: (2, 1),
             64: (2, 1)}
MAX_NSUBPIX = 4
MAX_PEAKS = 4
PEAK_FIELDS = 5

PRE_U8, PRE_U16, PRE_F32, PRE_F64 = 0, 1, 2, 3
MODES = {"reflect": 0, "constant": 1, "nearest": 2, "mirror": 3, "wrap": 4}

GRID_COCIRCULAR = 1
GRID_NEAREST_TIE = 2

P = C.c_void_p


class PivPassArgs(C.Structure):
    _fields_ = [
        ("im0", P), ("im1", P), ("dtype", C.c_int), ("height", C.c_int), ("width", C.c_int),
        ("im_min", P), ("n", C.c_int), ("ixvecs", P), ("nx", C.c_int), ("iyvecs", P),
        ("ny", C.c_int), ("dxin", P), ("dyin", P), ("mask", P),
        ("box_i0_start", C.c_int), ("box_i0_stop", C.c_int), ("box_i1_start", C.c_int),
        ("box_i1_stop", C.c_int), ("particle_radius", C.c_int), ("apply_subpix", C.c_int),
        ("deltaxs", P), ("deltays", P), ("correls_max", P), ("errors", P), ("xs", P),
        ("ys", P), ("norms", P), ("planes", P), ("flags", P),
        ("subpix_method", C.c_int), ("nsubpix", C.c_int), ("subpix_minv", P),
        ("nb_peaks", C.c_int), ("peaks_count", P), ("peaks", P), ("peaks_err", P),
    ]


class FixArgs(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("deltaxs", P), ("deltays", P), ("correls_max", P),
        ("errors", P), ("correl_min", C.c_float), ("use_displacement_max", C.c_int),
        ("displacement_max", C.c_float), ("use_threshold", C.c_int), ("threshold", C.c_float),
        ("deltaxs_out", P), ("deltays_out", P), ("fix_flags", P), ("diff2", P), ("work", P),
        ("nb_peaks", C.c_int), ("peaks_count", P), ("peaks", P), ("peaks_err", P),
        ("dxin", P), ("dyin", P),
        ("threshold64", C.c_double), ("displacement_max64", C.c_double),
        ("correls_max_out", P), ("replaced", P),
    ]


#: bytes of a TPS plan buffer (header + compaction scratch), FI_TPS_PLAN_BYTES
TPS_PLAN_BYTES = 256 + 24 * 1024


class TpsPlan(C.Structure):
    _fields_ = [
        ("num_centers", C.c_int), ("nb_subdomx", C.c_int), ("nb_subdomy", C.c_int),
        ("status", C.c_int), ("smoothing", C.c_double), ("x_min", C.c_double),
        ("x_max", C.c_double), ("y_min", C.c_double), ("y_max", C.c_double),
        ("buffer_x", C.c_double), ("buffer_y", C.c_double),
    ]


_SIGNATURES = {
    "fi_last_error": (C.c_char_p, []),
    "fi_version": (C.c_char_p, []),
    "fi_abi_sizes": (C.c_int, [P]),
    "fi_memcpy_d2h": (C.c_int, [P, P, C.c_int64, P]),
    "fi_launch_count": (C.c_longlong, []),
    "fi_images_min": (C.c_int, [P, P, C.c_int, C.c_int64, P, P]),
    "fi_piv_pass": (C.c_int, [P, P]),
    "fi_piv_pass_tc": (C.c_int, [P, C.c_int, P, P]),
    "fi_piv_pass_batch": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P]),
    "fi_piv_batch_items": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "fi_piv_batch_max_blocks": (C.c_int, [C.c_int, C.c_int]),
    "fi_images_min_batch": (C.c_int, [P, C.c_int, P, P]),
    "fi_fix_batch": (C.c_int, [P, P, C.c_int, C.c_int, P]),
    "fi_dc_warp": (C.c_int, [P, P, C.c_int, P, C.c_int, C.c_float, P, C.c_int, C.c_int,
                             C.c_int, C.c_int, P, P]),
    "fi_dc_windows": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_float, P, P, P, P]),
    "fi_dc_windows_backward": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_float, P, P, P,
                                         P]),
    "fi_dc_warp_backward": (C.c_int, [P, P, C.c_int, P, C.c_int, C.c_float, P, C.c_int, C.c_int,
                                      C.c_int, C.c_int, P, P, P, P]),
    "fi_correl_windows": (C.c_int, [P, P, C.c_int, C.c_int, P, P, P]),
    "fi_peaks_from_planes": (
        C.c_int,
        [P, P, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
         C.c_int, C.c_int, P, C.c_int, P, P, P, P, P, P, P, P, P, P],
    ),
    "fi_subpix_at": (C.c_int, [P, C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P, P]),
    "fi_fix": (C.c_int, [P, P]),
    "fi_fix_static": (C.c_int, [P, P]),
    "fi_tps_plan_make": (
        C.c_int,
        [P, P, P, P, C.c_int, C.c_int, C.c_double, C.c_double, P, P, P, P, P, P, P],
    ),
    "fi_tps_lattice": (C.c_int, [P, P, C.c_int, P, P, P]),
    "fi_tps_y_bounds": (C.c_int, [P, C.c_int, P, P, P]),
    "fi_tps_offsets": (C.c_int, [P, P, C.c_int, P, P, P, P, P, P, P]),
    "fi_tps_members": (C.c_int, [P, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P]),
    "fi_tps_layout": (
        C.c_int,
        [P, C.c_int, P, P, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "fi_tps_members_fill": (
        C.c_int,
        [P, C.c_int, P, P, C.c_int, P, P, C.c_int, P, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "fi_tps_solve": (
        C.c_int,
        [P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, C.c_double, C.c_int, P, P, P, P,
         P, P, P, P, P, P],
    ),
    "fi_tps_phi_table": (C.c_int, [P, C.c_int64, P]),
    "fi_tps_phi_table2": (C.c_int, [P, C.c_int64, P]),
    "fi_tps_solve_mp": (
        C.c_int,
        [P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, P, P, C.c_int64, P, P,
         C.c_double, C.c_int, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "fi_rank_filter": (
        C.c_int,
        [P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
         C.c_double, P, P],
    ),
    "fi_subtract_weighted": (
        C.c_int, [P, P, C.c_int, C.c_int64, C.c_double, C.c_int, C.c_int, P, P]),
    "fi_clamp": (C.c_int, [P, C.c_int, C.c_int64, C.c_double, C.c_double, P, P]),
    "fi_sq_sum_max": (C.c_int, [P, C.c_int, C.c_int64, P, P, C.c_int, P]),
    "fi_tanh_rescale": (C.c_int, [P, C.c_int, C.c_int64, C.c_double, C.c_double, P, P]),
    "fi_min_max": (C.c_int, [P, C.c_int, C.c_int64, P, C.c_int, P]),
    "fi_rescale_intensity": (C.c_int, [P, C.c_int, C.c_int64, P, C.c_int, C.c_double, C.c_double,
                                       P, P]),
    "fi_gamma": (C.c_int, [P, C.c_int, C.c_int64, C.c_double, C.c_double, P, P, P]),
    "fi_equalize_hist_int": (C.c_int, [P, C.c_int, C.c_int64, P, P, P, P]),
    "fi_equalize_hist_float": (C.c_int, [P, C.c_int, C.c_int64, P, C.c_int, C.c_double,
                                         C.c_double, P, P, P, P, P]),
    "fi_clahe": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                           P, P, P]),
    "fi_to_ubyte": (C.c_int, [P, C.c_int, C.c_int64, P, P]),
    "fi_rank_equalize": (C.c_int, [P, C.c_int, C.c_int, C.c_int, P, P]),
    "fi_gaussian_filter": (C.c_int, [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int, P]),
    "fi_sharpen_combine": (C.c_int, [P, P, C.c_int, C.c_int64, C.c_double, P, P]),
    "fi_image_unpack": (C.c_int, [P, C.c_int64, P, C.c_int, C.c_int, C.c_int, C.c_int, P,
                                  C.c_int, P, P, P]),
    "fi_png_unfilter": (C.c_int, [P, C.c_int, C.c_int, C.c_int, P]),
    "fi_tps_blend_centers": (C.c_int, [P, C.c_int, P, P, P, P, P, P, P, P, P, P, P]),
    "fi_tps_smooth_fields": (C.c_int, [P, P, C.c_int, P, P, C.c_int, C.c_double, C.c_double, P,
                                       C.c_int, P, P, P, P, P, P, P, P, P]),
    "fi_griddata": (
        C.c_int,
        [P, P, P, P, P, C.c_int, P, C.c_int, P, C.c_int, P, P, C.c_int, P, P, P, P, P, P, P,
         P],
    ),
    "fi_griddata_scratch_ints": (C.c_int64, [C.c_int, C.c_int]),
    "fi_tps_interpolate": (
        C.c_int,
        [P, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, C.c_int, P, P, P, P, P, P,
         P, P, P, P, P, P, C.c_int64, P, P, C.c_int, P],
    ),
}

_lib = None


def library_path() -> Path:
    return _build.library_path()


def load() -> C.CDLL:
    """Load the CUDA library (build it first with ``fluidimage_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"{path} is missing: build it with `python -m fluidimage_gb300.build` "
            "(the GB300 path has no CPU fallback)"
        )
    lib = C.CDLL(str(path))
    for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _lib = lib
    return lib


class CudaLibError(RuntimeError):
    pass


def check(rc: int, what: str = ""):
    if rc != FI_OK:
        msg = load().fi_last_error().decode(errors="replace")
        raise CudaLibError(f"{what or 'fluidimage_gb300'} failed ({rc}): {msg}")


def ptr(t) -> int | None:
    """Device pointer of a torch tensor (None for None)."""
    return None if t is None else t.data_ptr()


def stream_handle(stream=None) -> int:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
