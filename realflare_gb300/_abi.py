"""ctypes mirror of include/realflare_gb300.h and the loader of the CUDA library.

The library is ``realflare_gb300/librealflare_gb300.so``, built in-tree by
``realflare_gb300/build.py`` for sm_103a. Loading fails loudly when it is missing: there is
no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

from .data import RealflareError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'librealflare_gb300.so')

RF_OK = 0
RF_ERR_INVALID_ARG = 1
RF_ERR_OUT_OF_MEMORY = 2
RF_ERR_CUDA = 4
RF_ERR_WORKSPACE = 5
RF_ERR_NOT_SUPPORTED = 6
STATUS_NAMES = {
    0: 'ok', 1: 'invalid argument', 2: 'out of memory', 3: 'device timeout', 4: 'CUDA error',
    5: 'workspace too small', 6: 'not supported',
}

RAY_PLANES = 6
VERTEX_FLOATS = 8
SPECTRUM_WIDTH = 340


class TraceArgs(ctypes.Structure):
    _fields_ = [
        ('element_count', ctypes.c_int32),
        ('aperture_index', ctypes.c_int32),
        ('path_count', ctypes.c_int32),
        ('wavelength_count', ctypes.c_int32),
        ('grid_count', ctypes.c_int32),
        ('grid_length', ctypes.c_float),
        ('coating_min_ior', ctypes.c_float),
        ('coating_layer_ior', ctypes.c_float * 2),
        ('direction', ctypes.c_float * 4),
    ]


class RasterArgs(ctypes.Structure):
    _fields_ = [
        ('width', ctypes.c_int32),
        ('height', ctypes.c_int32),
        ('bin_size', ctypes.c_int32),
        ('tile_size', ctypes.c_int32),
        ('path_count', ctypes.c_int32),
        ('wavelength_count', ctypes.c_int32),
        ('wavelength_sub_count', ctypes.c_int32),
        ('grid_count', ctypes.c_int32),
        ('sub_steps', ctypes.c_int32),
        ('screen_transform', ctypes.c_float),
        ('intensity', ctypes.c_float),
        ('ghost_scale', ctypes.c_float),
        ('ghost_width', ctypes.c_int32),
        ('ghost_height', ctypes.c_int32),
    ]


class StarburstArgs(ctypes.Structure):
    _fields_ = [
        ('width', ctypes.c_int32),
        ('height', ctypes.c_int32),
        ('spectrum_width', ctypes.c_int32),
        ('spectrum_height', ctypes.c_int32),
        ('spectrum_count', ctypes.c_int32),
        ('samples', ctypes.c_int32),
        ('blur', ctypes.c_float),
        ('rotation', ctypes.c_float),
        ('rotation_weight', ctypes.c_float),
        ('vignetting', ctypes.c_float * 2),
        ('intensity', ctypes.c_float),
        ('offset', ctypes.c_float * 2),
        ('scale', ctypes.c_float * 2),
        ('lambda_first', ctypes.c_float),
        ('lambda_step', ctypes.c_float),
    ]


class Frame(ctypes.Structure):
    """rf_frame: one frame of a batched render."""
    _fields_ = [
        ('trace', TraceArgs),
        ('raster', RasterArgs),
        ('area_orig', ctypes.c_float),
        ('min_area', ctypes.c_float),
        ('element_offset', ctypes.c_int32),
        ('path_offset', ctypes.c_int32),
        ('wavelength_offset', ctypes.c_int32),
        ('ghost_offset', ctypes.c_int64),
        ('image_offset', ctypes.c_int64),
        ('ray_offset', ctypes.c_int64),
        ('prim_offset', ctypes.c_int64),
        ('inten_offset', ctypes.c_int64),
        ('vertex_offset', ctypes.c_int64),
        ('pair_offset', ctypes.c_int64),
        ('trace_block', ctypes.c_int64),
        ('quad_block', ctypes.c_int64),
        ('vertex_block', ctypes.c_int64),
        ('pair_block', ctypes.c_int64),
        ('tile_offset', ctypes.c_int32),
        ('tile_count', ctypes.c_int32),
        ('direction_n', ctypes.c_float * 3),
        ('pad1', ctypes.c_int32),
        ('ghost_texture', ctypes.c_uint64),
    ]


class BatchSizes(ctypes.Structure):
    """rf_batch_sizes."""
    _fields_ = [
        ('frame_count', ctypes.c_int32),
        ('tile_size', ctypes.c_int32),
        ('rays_per_thread', ctypes.c_int32),
        ('tiles', ctypes.c_int32),
        ('rays', ctypes.c_int64),
        ('prims', ctypes.c_int64),
        ('intensities', ctypes.c_int64),
        ('vertices', ctypes.c_int64),
        ('pairs', ctypes.c_int64),
        ('trace_blocks', ctypes.c_int64),
        ('quad_blocks', ctypes.c_int64),
        ('vertex_blocks', ctypes.c_int64),
        ('pair_blocks', ctypes.c_int64),
        ('image_pixels', ctypes.c_int64),
        ('ghost_floats', ctypes.c_int64),
        ('max_colors', ctypes.c_int32),
        ('max_sub', ctypes.c_int32),
        ('max_sub_steps', ctypes.c_int32),
        ('ghost_textures', ctypes.c_int32),
    ]


P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
F32 = ctypes.c_float

# name -> argtypes (every entry point returns int status)
SIGNATURES = {
    'rf_trace': [P, P, P, ctypes.POINTER(TraceArgs), P, P],
    'rf_trace_accurate': [P, P, P, ctypes.POINTER(TraceArgs), P, P],
    'rf_trace_intersections': [P, P, P, ctypes.POINTER(TraceArgs), P, P, I32, P],
    'rf_diagram': [P, I32, I32, F32, P, I32, I32, I32, I32, P, P],
    'rf_quad_setup': [P, I32, I32, I32, F32, F32, P, P, P],
    'rf_vertex': [P, P, I32, I32, I32, F32, I32, I32, P, P],
    'rf_bin_masks': [P, I32, F32, I32, I32, I32, P, P],
    'rf_bin_workspace_size': [ctypes.POINTER(RasterArgs), I64, ctypes.POINTER(ctypes.c_size_t)],
    'rf_bin_tiles': [P, P, ctypes.POINTER(RasterArgs), P, ctypes.c_size_t, P, P, I64,
                     ctypes.POINTER(ctypes.c_int64), P],
    'rf_raster_tiles': [ctypes.POINTER(RasterArgs), ctypes.POINTER(I32), ctypes.POINTER(I32)],
    'rf_raster': [P, P, P, P, P, ctypes.POINTER(RasterArgs), P, P],
    'rf_tile_order_workspace_size': [I32, ctypes.POINTER(ctypes.c_size_t)],
    'rf_tile_order': [P, I32, P, ctypes.c_size_t, P, P],
    'rf_raster_ordered': [P, P, P, P, P, P, ctypes.POINTER(RasterArgs), P, P],
    'rf_raster_masks': [P, P, I32, P, P, ctypes.POINTER(RasterArgs), P, P],
    'rf_fft2': [P, P, I32, I32, I32, I32, F32, P],
    'rf_starburst_spectrum': [P, I32, I32, ctypes.POINTER(F32), I32, F32, P, P, P],
    'rf_starburst': [P, P, ctypes.POINTER(StarburstArgs), P, P],
    'rf_ghost_frft': [P, I32, I32, F32, P, P, P],
    'rf_ghost_frft_static': [P, I32, I32, F32, P, P],
    'rf_aperture_shape': [P, I32, I32, F32, F32, I32, F32, F32, F32, P],
    'rf_aperture_dust': [P, I32, I32, F32, F32, F32, F32, F32, F32, F32, F32, P],
    'rf_aperture_noise_dust': [P, P, P, I32, I32, F32, F32, P],
    'rf_axpby': [P, F32, P, F32, P, I64, P],
    'rf_accumulate_mirrored': [P, P, I32, I32, I32, F32, P, P],
    'rf_trace_adjoint': [P, P, P, ctypes.POINTER(TraceArgs), P, P, P, P],
    'rf_raster_backward': [P, P, P, P, P, ctypes.POINTER(RasterArgs), P, P, P, P],
    'rf_vertex_backward': [P, P, I32, I32, I32, P, P, P, P],
    'rf_quad_setup_backward': [P, I32, I32, I32, F32, F32, P, P, P],
    'rf_batch_plan': [ctypes.POINTER(Frame), I32, I32, I32, ctypes.POINTER(BatchSizes)],
    'rf_trace_batch': [P, ctypes.POINTER(BatchSizes), P, P, P, P, P],
    'rf_quad_setup_batch': [P, ctypes.POINTER(BatchSizes), P, P, P, P],
    'rf_vertex_batch': [P, ctypes.POINTER(BatchSizes), P, P, P, P],
    'rf_batch_workspace_size': [ctypes.POINTER(BatchSizes), I64, ctypes.POINTER(ctypes.c_size_t)],
    'rf_bin_tiles_batch': [P, ctypes.POINTER(BatchSizes), P, P, P, ctypes.c_size_t, P, P, I64, P, P],
    'rf_ghost_texture_object': [P, I32, I32, ctypes.POINTER(ctypes.c_uint64)],
    'rf_ghost_textures_forget': [],
    'rf_raster_batch': [P, ctypes.POINTER(BatchSizes), P, P, P, P, P, P, ctypes.c_size_t, I64, P, P, P],
}

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded CUDA library; raises RealflareError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RealflareError(
                f'CUDA library not built: {LIB_PATH} (run realflare_gb300.build.build())'
            )
        handle = ctypes.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int
        handle.rf_version.restype = ctypes.c_char_p
        handle.rf_last_cuda_error.restype = ctypes.c_char_p
        handle.rf_launch_count.restype = ctypes.c_longlong
        _lib = handle
    return _lib


def check(status: int, what: str) -> None:
    if status != RF_OK:
        detail = ''
        if status == RF_ERR_CUDA and _lib is not None:
            detail = ': ' + _lib.rf_last_cuda_error().decode(errors='replace')
        raise RealflareError(f'{what} failed: {STATUS_NAMES.get(status, status)}{detail}')
