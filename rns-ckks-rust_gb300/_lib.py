"""ctypes binding of the C ABI in include/rnsckks_gpu.h (librnsckks_gpu.so).

This is the Python counterpart of the FFI stub a Rust caller would write: every
entry point keeps its C signature, and a non-zero status raises with the
library's message.  There is no fallback: if the shared library is missing or
fails to load, importing the package's GPU API raises.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "librnsckks_gpu.so"

RC_OK = 0
RC_ERR_INVALID_ARGUMENT = 1
RC_ERR_CUDA = 2
RC_ERR_OUT_OF_MEMORY = 3
RC_ERR_UNSUPPORTED = 4


class RcError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class RcPrime(ctypes.Structure):
    _fields_ = [("modulus", ctypes.c_uint64), ("primitive_root", ctypes.c_uint64)]


class RcParams(ctypes.Structure):
    _fields_ = [
        ("poly_degree", ctypes.c_uint64),
        ("primes", ctypes.POINTER(RcPrime)),
        ("prime_count", ctypes.c_uint32),
        ("aux_primes", ctypes.POINTER(RcPrime)),
        ("aux_count", ctypes.c_uint32),
        ("scale_bits", ctypes.c_uint32),
    ]


class RcCiphertext(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("level", ctypes.c_int32), ("scale_bits", ctypes.c_int32)]


# (name, restype, argtypes) for every exported entry point of include/rnsckks_gpu.h
_vp, _u32, _i32, _u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64
_CT = ctypes.POINTER(RcCiphertext)
SIGNATURES = [
    ("rc_context_create", ctypes.c_int, [ctypes.POINTER(RcParams), ctypes.POINTER(_vp)]),
    ("rc_context_destroy", None, [_vp]),
    ("rc_last_error", ctypes.c_char_p, [_vp]),
    ("rc_context_info", ctypes.c_int, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u32), ctypes.POINTER(_u32),
                                       ctypes.POINTER(_u32)]),
    ("rc_decomp_digits", ctypes.c_int, [_vp, _i32, ctypes.POINTER(_u32)]),
    ("rc_reserve", ctypes.c_int, [_vp, _i32, _u32, _vp]),
    ("rc_tune_set", ctypes.c_int, [_vp, ctypes.c_char_p, _i32]),
    ("rc_tune_get", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_i32)]),
    ("rc_ksk_upload", ctypes.c_int, [_vp, _vp, _u32, _i32, _u32, _u64, ctypes.POINTER(_vp)]),
    ("rc_ksk_upload_device", ctypes.c_int, [_vp, _vp, _u32, _i32, _u32, _u64, ctypes.POINTER(_vp)]),
    ("rc_ksk_upload_dnum", ctypes.c_int, [_vp, _vp, _i32, _u32, _i32, ctypes.POINTER(_vp)]),
    ("rc_ksk_truncate", ctypes.c_int, [_vp, _vp, _i32, ctypes.POINTER(_vp)]),
    ("rc_ksk_info", ctypes.c_int, [_vp, ctypes.POINTER(_u32), ctypes.POINTER(_i32), ctypes.POINTER(_u32),
                                   ctypes.POINTER(_u64)]),
    ("rc_ksk_destroy", None, [_vp]),
    ("rc_ksk_serialized_size", ctypes.c_int, [_vp, ctypes.POINTER(_u64)]),
    ("rc_ksk_serialize", ctypes.c_int, [_vp, _vp, _vp, _u64, _vp]),
    ("rc_ksk_deserialize", ctypes.c_int, [_vp, _vp, _u64, ctypes.POINTER(_vp)]),
    ("rc_ct_serialized_size", ctypes.c_int, [_vp, _i32, _u32, ctypes.POINTER(_u64)]),
    ("rc_ct_serialize", ctypes.c_int, [_vp, _CT, _u32, _vp, _u64, _vp]),
    ("rc_ct_header", ctypes.c_int, [_vp, _u64, ctypes.POINTER(_u64), ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                    ctypes.POINTER(_u32)]),
    ("rc_ct_deserialize", ctypes.c_int, [_vp, _vp, _u64, _CT, _u64, _vp]),
    ("rc_ntt_forward", ctypes.c_int, [_vp, _vp, _u32, _u32, _i32, _vp]),
    ("rc_ntt_inverse", ctypes.c_int, [_vp, _vp, _u32, _u32, _i32, _vp]),
    ("rc_poly_multiply", ctypes.c_int, [_vp, _vp, _vp, _vp, _u32, _i32, _vp]),
    ("rc_poly_add", ctypes.c_int, [_vp, _vp, _vp, _vp, _u32, _i32, _vp]),
    ("rc_poly_sub", ctypes.c_int, [_vp, _vp, _vp, _vp, _u32, _i32, _vp]),
    ("rc_poly_mul_scalar", ctypes.c_int, [_vp, _vp, _vp, _vp, _u32, _i32, _vp]),
    ("rc_poly_multiply_noalloc", ctypes.c_int, [_vp, _vp, _vp, _vp, _u32, _i32, _vp]),
    ("rc_poly_automorphism", ctypes.c_int, [_vp, _vp, _vp, _u32, _u64, _vp]),
    ("rc_sample_uniform", ctypes.c_int, [_vp, _u64, _u64, _vp, _u32, _i32, _vp]),
    ("rc_sample_error", ctypes.c_int, [_vp, _u64, _u64, _vp, _u32, _i32, _vp]),
    ("rc_sample_ternary", ctypes.c_int, [_vp, _u64, _u64, _vp, _u32, _i32, _vp]),
    ("rc_add", ctypes.c_int, [_vp, _CT, _CT, _CT, _vp]),
    ("rc_mult_plain", ctypes.c_int, [_vp, _CT, _vp, _CT, _vp]),
    ("rc_multiply_plain_rns", ctypes.c_int, [_vp, _CT, _vp, _CT, _vp]),
    ("rc_mult_plain_accumulate", ctypes.c_int, [_vp, _u32, _CT, _i32, _vp, _i32, _CT, _vp]),
    ("rc_add_batch", ctypes.c_int, [_vp, _u32, _CT, _CT, _CT, _vp]),
    ("rc_multiply_plain_rns_batch", ctypes.c_int, [_vp, _u32, _CT, _vp, _CT, _vp]),
    ("rc_rescale_batch", ctypes.c_int, [_vp, _u32, _CT, _CT, _vp]),
    ("rc_lift_to_aux", ctypes.c_int, [_vp, _vp, _vp, _u32, _u32, _vp]),
    ("rc_mod_raise", ctypes.c_int, [_vp, _CT, _CT, _vp]),
    ("rc_mult", ctypes.c_int, [_vp, _CT, _CT, _CT, _vp]),
    ("rc_rescale", ctypes.c_int, [_vp, _CT, _CT, _vp]),
    ("rc_rescale_quadratic", ctypes.c_int, [_vp, _CT, _CT, _vp]),
    ("rc_keyswitch", ctypes.c_int, [_vp, _vp, _i32, _vp, _CT, _vp]),
    ("rc_relinearize", ctypes.c_int, [_vp, _CT, _vp, _CT, _vp]),
    ("rc_mult_relinearized", ctypes.c_int, [_vp, _CT, _CT, _vp, _CT, _vp]),
    ("rc_rotate", ctypes.c_int, [_vp, _CT, _vp, _CT, _vp]),
    ("rc_automorphism", ctypes.c_int, [_vp, _CT, _u64, _CT, _vp]),
    ("rc_mult_relinearized_batch", ctypes.c_int, [_vp, _u32, _CT, _CT, ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_relinearize_batch", ctypes.c_int, [_vp, _u32, _CT, ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_rotate_batch", ctypes.c_int, [_vp, _u32, _CT, ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_rotate_hoisted", ctypes.c_int, [_vp, _u32, _CT, _u32, ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_kernel_errors", ctypes.c_int, [ctypes.POINTER(_i32), _i32]),
    ("rc_relinearize_rescale_batch", ctypes.c_int, [_vp, _u32, _CT, ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_total_sum_batch", ctypes.c_int, [_vp, _u32, _CT, _u32, ctypes.POINTER(_vp), _u32, _CT, _vp]),
    ("rc_halevi_shoup_batch", ctypes.c_int, [_vp, _u32, _CT, _vp, _u32, ctypes.POINTER(_vp), _u32, _CT, _vp]),
    ("rc_paterson_stockmeyer_batch", ctypes.c_int, [_vp, _u32, _CT, _vp, _u32, ctypes.POINTER(_vp), _u32, _CT,
                                                    _vp]),
    ("rc_bsgs_apply_batch", ctypes.c_int, [_vp, _u32, _CT, _u32, _u32, ctypes.POINTER(_vp), _u32, _i32, _i32,
                                           ctypes.POINTER(_vp), ctypes.POINTER(_vp), _CT, _vp]),
    ("rc_graph_begin", ctypes.c_int, [_vp, _vp]),
    ("rc_graph_end", ctypes.c_int, [_vp, _vp, ctypes.POINTER(_vp)]),
    ("rc_graph_launch", ctypes.c_int, [_vp, _vp]),
    ("rc_graph_destroy", None, [_vp]),
    ("rc_mult_relinearized_host", ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp, _vp, ctypes.POINTER(_i32), _vp]),
    ("rc_mult_relinearized_batch_host", ctypes.c_int, [_vp, _u32, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                                       ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                                       ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                                       ctypes.POINTER(_i32), _vp]),
    ("rc_mult_relinearized_batch_host_async", ctypes.c_int, [_vp, _u32, ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                                             ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                                             ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                                             ctypes.POINTER(_i32), _vp]),
    ("rc_host_join", ctypes.c_int, [_vp, _vp]),
    ("rc_encode", ctypes.c_int, [_vp, _vp, _i32, _u32, _vp]),
    ("rc_decode", ctypes.c_int, [_vp, _vp, _i32, _u32, _vp]),
    ("rc_encode_device", ctypes.c_int, [_vp, _vp, _u32, _i32, _u32, _vp, _vp]),
    ("rc_decode_device", ctypes.c_int, [_vp, _vp, _u32, _i32, _u32, _vp, _vp]),
    ("rc_slots_to_real_coeffs", ctypes.c_int, [_u64, _vp, _vp]),
    ("rc_complex_coeffs_to_slots", ctypes.c_int, [_u64, _vp, _vp]),
    ("rc_profile_enable", ctypes.c_int, [ctypes.c_int]),
    ("rc_profile_report", ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
]


def build(jobs: int = 8) -> Path:
    """Compile the CUDA library for sm_103a with the package Makefile."""
    subprocess.run(["make", "-s", f"-j{jobs}", "-C", str(PKG_DIR)], check=True)
    return BUILD_DIR / LIB_NAME


_lib = None


def lib():
    """Load librnsckks_gpu.so (raises when it is missing: there is no CPU fallback)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("RNSCKKS_GPU_LIB", BUILD_DIR / LIB_NAME))
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build the CUDA library first (make -C {PKG_DIR})")
        L = ctypes.CDLL(str(path))
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


_probe = None


def probe_lib():
    """Load librnsckks_probe.so, the measurement probes of the benchmark (not part of the library's ABI)."""
    global _probe
    if _probe is None:
        path = BUILD_DIR / "librnsckks_probe.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it first (make -C {PKG_DIR})")
        P = ctypes.CDLL(str(path))
        P.rc_measure_multiply_rates.restype = ctypes.c_int
        P.rc_measure_multiply_rates.argtypes = [_vp, _vp]
        _probe = P
    return _probe


def check(status: int) -> None:
    if status != RC_OK:
        msg = lib().rc_last_error(None)
        raise RcError(status, msg.decode() if msg else f"status {status}")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
