"""ctypes declarations of include/itkg.h and loading of libitkg.so.

The library is built in-tree (itk-rs_gb300/lib/libitkg.so) by
itk-rs_gb300/build.py; importing this module never falls back to anything
else: if the library is missing, `lib()` raises.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_PKG), "lib", "libitkg.so")

SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_UNSUPPORTED = 2
ERROR_CUDA = 3
ERROR_OUT_OF_MEMORY = 4
ERROR_NO_DEVICE = 5
ERROR_TIMEOUT = 6

F32, I16, U8, BF16, F16 = 0, 1, 2, 3, 4
DEVICE, HOST = 0, 1
ARITH_F32, ARITH_PIXEL_U8 = 0, 1
ROUND_REFERENCE, ROUND_FMA = 0, 1
ALGO_AUTO, ALGO_FUSED, ALGO_PER_AXIS, ALGO_TWO_PASS, ALGO_ONE_TRIP = 0, 1, 2, 3, 4

c_i64_3 = ctypes.c_int64 * 3
c_u64_3 = ctypes.c_uint64 * 3
c_f64_3 = ctypes.c_double * 3


class itkg_region(ctypes.Structure):
    _fields_ = [("index", c_i64_3), ("size", c_u64_3)]


class itkg_image(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("components", ctypes.c_int32),
        ("location", ctypes.c_int32),
        ("region", itkg_region),
        ("pitch", c_i64_3),
        ("spacing", c_f64_3),
        ("origin", c_f64_3),
        ("data", ctypes.c_void_p),
    ]


class itkg_gaussian_params(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_double),
        ("arithmetic", ctypes.c_int32),
        ("rounding", ctypes.c_int32),
        ("algorithm", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class itkg_separable_params(ctypes.Structure):
    _fields_ = [
        ("radius", ctypes.c_uint64 * 3),
        ("weights", ctypes.c_void_p * 3),
        ("repetitions", ctypes.c_uint64),
        ("arithmetic", ctypes.c_int32),
        ("rounding", ctypes.c_int32),
        ("algorithm", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class itkg_recursive_params(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_double),
        ("axis", ctypes.c_int32),
        ("rounding", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
    ]


class itkg_unsharp_params(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_double),
        ("amount", ctypes.c_double),
        ("threshold", ctypes.c_double),
        ("rounding", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class itkg_recursive_derivative_params(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_double),
        ("sigma2", ctypes.c_double),
        ("kind", ctypes.c_int32),
        ("axis", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("rounding", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 2),
    ]


# name -> (restype, argtypes); every symbol include/itkg.h declares.
P = ctypes.c_void_p
R = ctypes.POINTER(itkg_region)
I = ctypes.POINTER(itkg_image)
G = ctypes.POINTER(itkg_gaussian_params)
st = ctypes.c_int
SIGNATURES = {
    "itkg_abi_version": (ctypes.c_int32, []),
    "itkg_last_error": (ctypes.c_char_p, []),
    "itkg_last_kernel": (ctypes.c_char_p, []),
    "itkg_launch_counter": (ctypes.c_uint64, []),
    "itkg_scratch_alloc_counter": (ctypes.c_uint64, []),
    "itkg_debug_fail_scratch_alloc": (None, [ctypes.c_int64]),
    "itkg_debug_set_wait_limit": (None, [ctypes.c_int64]),
    "itkg_debug_set_2d_kernel": (None, [ctypes.c_int32]),
    "itkg_kernel_radius": (ctypes.c_uint64, [ctypes.c_double, ctypes.c_double]),
    "itkg_build_kernel": (st, [ctypes.c_double, ctypes.c_uint64, P]),
    "itkg_region_padded_per_axis": (st, [R, ctypes.c_int32, P, R]),
    "itkg_region_clipped_to": (st, [R, ctypes.c_int32, R, R]),
    "itkg_gaussian_input_region_for_output": (st, [R, R, ctypes.c_int32, P, ctypes.c_double, R]),
    "itkg_split_region": (st, [R, ctypes.c_int32, ctypes.c_uint64, R, ctypes.c_uint64,
                               ctypes.POINTER(ctypes.c_uint64)]),
    "itkg_device_count": (st, [ctypes.POINTER(ctypes.c_int32)]),
    "itkg_set_device": (st, [ctypes.c_int32]),
    "itkg_device_alloc": (st, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "itkg_device_free": (st, [P]),
    "itkg_host_alloc_pinned": (st, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "itkg_host_free_pinned": (st, [P]),
    "itkg_memcpy": (st, [P, P, ctypes.c_size_t, ctypes.c_int32, P]),
    "itkg_memset_device": (st, [P, ctypes.c_int32, ctypes.c_size_t, P]),
    "itkg_stream_synchronize": (st, [P]),
    "itkg_demons_registration": (st, [I, I, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_double, I, P]),
    "itkg_n4_bias_field_correction": (st, [I, R, ctypes.c_int32, ctypes.c_double, ctypes.c_double, I,
                                           ctypes.POINTER(ctypes.c_int32), P]),
    "itkg_stream_create": (st, [ctypes.POINTER(ctypes.c_void_p)]),
    "itkg_stream_destroy": (st, [P]),
    "itkg_device_fault": (st, [ctypes.c_int32, ctypes.POINTER(ctypes.c_uint32)]),
    "itkg_image_alloc_device": (st, [I, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, R, P, P]),
    "itkg_image_free": (st, [I]),
    "itkg_image_copy_from": (st, [I, I, P]),
    "itkg_gaussian_generate_region": (st, [I, R, R, G, I, P]),
    "itkg_stream_full": (st, [I, R, G, ctypes.c_uint64, I, P]),
    "itkg_gaussian_generate_region_noalloc": (st, [I, R, R, G, I, P]),
    "itkg_box_kernel": (st, [ctypes.c_uint64, P]),
    "itkg_yvv_coeffs": (st, [ctypes.c_double, P]),
    "itkg_recursive_gaussian_generate_region": (st, [I, R, R, ctypes.POINTER(itkg_recursive_params), I, P]),
    "itkg_recursive_gaussian_derivative_generate_region": (st, [I, R, R,
                                                                ctypes.POINTER(itkg_recursive_derivative_params),
                                                                I, P]),
    "itkg_unsharp_kernel": (st, [ctypes.c_double, ctypes.POINTER(ctypes.c_uint64), P, ctypes.c_uint64]),
    "itkg_unsharp_mask_generate_region": (st, [I, R, R, ctypes.POINTER(itkg_unsharp_params), I, P]),
    "itkg_slice_by_slice_generate_region": (st, [I, R, G, I, P]),
    "itkg_bspline_downsample_generate_region": (st, [I, R, G, I, P]),
    "itkg_separable_input_region_for_output": (st, [R, R, ctypes.c_int32, P, ctypes.c_uint64, R]),
    "itkg_separable_generate_region": (st, [I, R, R, ctypes.POINTER(itkg_separable_params), I, P]),
    "itkg_gaussian_vjp": (st, [I, I, G, I, ctypes.POINTER(ctypes.c_double), ctypes.c_int32, P]),
    "itkg_gaussian_scale_stack_loss_vjp": (st, [I, I, ctypes.POINTER(ctypes.c_double), ctypes.c_int32,
                                                I, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double), ctypes.c_int32, P]),
    "itkg_batch_create": (st, [ctypes.POINTER(ctypes.c_void_p)]),
    "itkg_batch_destroy": (st, [P]),
    "itkg_batch_add": (st, [P, I, R, R, G, I]),
    "itkg_batch_add_vjp": (st, [P, I, I, G, I, P, ctypes.c_int32]),
    "itkg_batch_plan": (st, [P, ctypes.c_int32, P]),
    "itkg_batch_run": (st, [P, P]),
    "itkg_batch_describe": (ctypes.c_char_p, [P]),
}

_lib = None


class ItkgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"itkg status {status}: {message}")
        self.status = status


def lib():
    """Load libitkg.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libitkg.so not built: run python itk-rs_gb300/build.py ({LIB_PATH})")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != SUCCESS:
        raise ItkgError(status, lib().itkg_last_error().decode())
    return status
