"""ctypes binding of libqrochet_gpu.so (the C ABI declared in include/qrochet_gpu.h).

The library is required: importing a GPU entry point without it raises, there is no CPU
fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libqrochet_gpu.so")

QR_OK, QR_EINVAL, QR_EASSERT, QR_ENO_SCHMIDT, QR_EDIM, QR_ENOMEM, QR_ECUDA, QR_ENODEV, QR_ENOCONV, QR_EHOST = range(10)
QR_FP64, QR_MIXED = 0, 1
QR_DIR_LEFT, QR_DIR_RIGHT = 0, 1
QR_METHOD_QR, QR_METHOD_SVD = 0, 1


class ArgumentError(ValueError):
    """Julia ``ArgumentError``."""


class DimensionMismatch(ValueError):
    """Julia ``DimensionMismatch``."""


class MissingSchmidtCoefficientsException(RuntimeError):
    """``MissingSchmidtCoefficientsException`` (src/Ansatz.jl:91-99)."""

    def __init__(self, bond, msg=None):
        super().__init__(msg or f"Can't access the spectrum on bond {bond}")
        self.bond = bond


class GPUError(RuntimeError):
    """CUDA failure, missing device, allocation failure or non-convergence."""


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_PI = C.POINTER(C.c_int)
_PD = C.POINTER(C.c_double)
_S = C.c_char_p

# name -> argtypes (all return int status)
SIGNATURES = {
    "qr_version": [_PI, _PI],
    "qr_device_count": [_PI],
    "qr_set_device": [_I],
    "qr_launch_count": [C.POINTER(C.c_uint64)],
    "qr_prof_enable": [_I],
    "qr_prof_read": [_I, _PD, C.POINTER(C.c_uint64), _PD, _PD],
    "qr_probe_peak": [_I, _PD],
    "qr_host_alloc": [C.c_uint64, C.POINTER(_P)],
    "qr_host_free": [_P],
    "qr_chain_create": [_I, _I, _PI, C.POINTER(_P)],
    "qr_chain_free": [_P],
    "qr_chain_create_periodic": [_I, _I, _PI, C.POINTER(_P)],
    "qr_chain_boundary": [_P, _PI],
    "qr_chain_copy": [_P, C.POINTER(_P)],
    "qr_chain_upload_site": [_P, _I, _PD, _S],
    "qr_chain_download_site": [_P, _I, _PD, _S],
    "qr_chain_site_dims": [_P, _I, _PI, _PI, _PI],
    "qr_chain_bond_dims": [_P, _PI],
    "qr_chain_has_lambda": [_P, _I, _PI],
    "qr_chain_get_lambda": [_P, _I, _PD, _PI],
    "qr_chain_set_lambda": [_P, _I, _PD, _I],
    "qr_chain_ntensors": [_P, _PI],
    "qr_chain_nsites": [_P, _PI],
    "qr_chain_set_precision": [_P, _I],
    "qr_chain_save": [_P, _S],
    "qr_chain_random": [_I, _I, _I, C.c_uint64, _I, C.POINTER(_P)],
    "qr_mpo_random": [_I, _I, _I, C.c_uint64, _I, C.POINTER(_P)],
    "qr_mpo_download_site": [_P, _I, _PD, _S],
    "qr_chain_load": [_S, C.POINTER(_P)],
    "qr_chain_get_precision": [_P, _PI],
    "qr_chain_stream": [_P, C.POINTER(_P)],
    "qr_chain_sync": [_P],
    "qr_canonize_site": [_P, _I, _I, _I],
    "qr_canonize": [_P],
    "qr_mixed_canonize": [_P, _I],
    "qr_normalize": [_P, _I],
    "qr_contract_between": [_P, _I, _I, _I, _I],
    "qr_canonicality_error": [_P, _I, _I, _PD],
    "qr_truncate": [_P, _I, _I, _D, _I],
    "qr_evolve_1site": [_P, _I, _PD],
    "qr_evolve_2site": [_P, _I, _PD, _D, _I, _I, _I],
    "qr_evolve_layer": [_P, _I, _PI, _PD, _D, _I, _I, _I, _I],
    "qr_overlap": [_P, _P, _PD],
    "qr_norm": [_P, _PD],
    "qr_expect": [_P, _I, _PI, _PI, _PD, _PD],
    "qr_mpo_create": [_I, _I, _PI, C.POINTER(_P)],
    "qr_mpo_free": [_P],
    "qr_mpo_upload_site": [_P, _I, _PD, _S],
    "qr_mpo_expect": [_P, _P, _PD],
    "qr_server_create": [_I, _I, C.c_uint64, _I, C.POINTER(_P)],
    "qr_server_free": [_P],
    "qr_server_footprint": [_I, _I, C.POINTER(C.c_uint64)],
    "qr_server_submit": [_P, _I, _I, _D, _I, _PI, _PD, _I, _PI, _PI, _PI, C.POINTER(C.c_uint64)],
    "qr_server_wait": [_P, C.c_uint64, _D, _PI, _PI, _PD, _PD, _PD],
    "qr_server_stats": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), _PI, C.POINTER(C.c_uint64), _PI],
    "qr_batch_create": [_I, C.POINTER(_P)],
    "qr_batch_free": [_P],
    "qr_batch_set_precision": [_P, _I],
    "qr_batch_add": [_P, _I, _I, _D, _I, _PI, _PD, _I, _PI, _PI, _PI, _PI],
    "qr_batch_plan": [_P, _I, _PI, _PI],
    "qr_batch_run": [_P, _PD],
    "qr_batch_result": [_P, _I, _PI, _PD],
    "qr_batch_bond_dims": [_P, _I, _PI],
    "qr_batch_lambda": [_P, _I, _I, _PD, _PI],
    "qr_batch_info": [_P, _PI, _PI, _PI, _PI, _PI, _PD, _PD],
    "qr_svd_noalloc": [_I, _I, _P, C.c_long, _P, C.c_long, _P, _P, C.c_long, _P],
    "qr_test_zgemm": [_I, _I, _I, _I, _I, _PD, _PD, C.c_long, _PD, C.c_long, _PD, _PD, C.c_long, _PD, _I, _PD],
    "qr_test_zgemm_tc": [_I, _I, _I, _I, _I, _I, _PD, C.c_long, C.c_long, _PD, C.c_long, C.c_long, _PD, C.c_long,
                         _I, _PD],
    "qr_test_zgemm_df": [_I, _I, _I, _I, _I, _PD, C.c_long, _PD, C.c_long, _PD, _PD, C.c_long, _I, _PD],
    "qr_test_svd": [_I, _I, _I, _PD, _PD, _PD, _PD, _PD],
    "qr_test_svd_paths": [C.POINTER(C.c_uint64), _I, C.POINTER(C.c_int)],
    "qr_test_schedule_pairs": [C.c_void_p, C.c_void_p, _I, _I, C.c_void_p, C.c_void_p, C.POINTER(C.c_long),
                               C.POINTER(C.c_int)],
    "qr_test_qr": [_I, _I, _PD, _PD, _PD, _PD],
    "qr_test_host_exception": [_I],
}

_lib = None
_lock = threading.Lock()


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libqrochet_gpu.so not found at {LIB_PATH}; build it first "
                "(python qrochet.jl_gb300/build.py or __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.qr_last_error_string.argtypes = []
        L.qr_last_error_string.restype = C.c_char_p
        _lib = L
        return L


def last_error():
    return lib().qr_last_error_string().decode(errors="replace")


def check(rc, bond=None):
    if rc == QR_OK:
        return
    msg = last_error()
    if rc == QR_EINVAL:
        raise ArgumentError(msg)
    if rc == QR_EASSERT:
        raise AssertionError(msg)
    if rc == QR_ENO_SCHMIDT:
        raise MissingSchmidtCoefficientsException(bond, msg)
    if rc == QR_EDIM:
        raise DimensionMismatch(msg)
    raise GPUError(f"status {rc}: {msg}")


def launch_count():
    c = C.c_uint64(0)
    check(lib().qr_launch_count(C.byref(c)))
    return int(c.value)


def dptr(a):
    """Pointer to a contiguous complex128/float64 NumPy buffer as double*."""
    return a.ctypes.data_as(_PD)
