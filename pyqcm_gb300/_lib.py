"""ctypes binding of the qcmg C ABI (include/qcmg.h).

The library is built in-tree (pyqcm_gb300/_build/libqcmg.so).  There is no
CPU fallback: if the library is missing or cannot be loaded, every call
raises QcmgError.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqcmg.so")

QCMG_DEVICE_PTRS = 1
QCMG_ACCUMULATE = 2
QCMG_ASYNC = 4

ERRORS = {-1: "invalid argument", -2: "CUDA failure", -3: "out of device memory",
          -4: "no convergence", -5: "no usable GPU", -6: "numerical breakdown"}


class QcmgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"qcmg error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None

c_int, c_uint, c_double, c_size_t = ctypes.c_int, ctypes.c_uint, ctypes.c_double, ctypes.c_size_t
vp = ctypes.c_void_p
size_p = ctypes.POINTER(ctypes.c_size_t)
int_p = ctypes.POINTER(ctypes.c_int)
dbl_p = ctypes.POINTER(ctypes.c_double)

SIGNATURES = {
    "qcmg_version": (ctypes.c_char_p, []),
    "qcmg_last_error": (c_size_t, [ctypes.c_char_p, c_size_t]),
    "qcmg_set_device": (c_int, [c_int]),
    "qcmg_halfbasis": (c_int, [c_int, c_int, vp, c_size_t, size_p]),
    "qcmg_halfbasis_rank": (c_int, [c_int, c_int, vp, c_size_t, vp]),
    "qcmg_hamiltonian_create": (c_int, [c_int, c_int, c_int, c_int, vp, vp, vp, c_int, vp, vp, vp,
                                        c_int, vp, vp, vp, ctypes.POINTER(vp)]),
    "qcmg_hamiltonian_destroy": (c_int, [vp]),
    "qcmg_hamiltonian_set_stream": (c_int, [vp, vp]),
    "qcmg_hamiltonian_dims": (c_int, [vp, size_p, size_p, size_p]),
    "qcmg_hamiltonian_halfop": (c_int, [vp, c_int, size_p, vp, vp, vp, vp]),
    "qcmg_matvec": (c_int, [vp, vp, vp, c_uint]),
    "qcmg_hamiltonian_set_path": (c_int, [vp, c_int]),
    "qcmg_hamiltonian_fx_available": (c_int, [vp, int_p]),
    "qcmg_fx_from_f64": (c_int, [c_size_t, vp, vp, int_p, int_p, vp]),
    "qcmg_fx_to_f64": (c_int, [c_size_t, vp, c_int, vp, vp]),
    "qcmg_matvec_fx": (c_int, [vp, vp, c_int, c_int, vp, int_p, c_uint]),
    "qcmg_multidot": (c_int, [c_int, vp, vp, c_size_t, vp, vp]),
    "qcmg_multidot_noalloc": (c_int, [c_int, vp, vp, c_size_t, vp, vp]),
    "qcmg_seeded_vector": (c_int, [c_size_t, c_uint, vp]),
    "qcmg_lanczos_ground_state": (c_int, [vp, vp, c_uint, c_double, c_int, c_int, dbl_p, vp,
                                          int_p, vp, vp, c_int]),
    "qcmg_lanczos_batch": (c_int, [c_int, vp, c_uint, c_double, c_int, c_int, vp, vp, vp, vp]),
    "qcmg_lanczos_last_stats": (c_int, [vp, dbl_p, dbl_p, dbl_p, int_p, int_p, int_p]),
    "qcmg_fp64_fma_rate": (c_int, [dbl_p]),
    "qcmg_band_lanczos": (c_int, [vp, c_int, vp, c_int, c_int, c_double, c_double, int_p, vp,
                                  vp, c_int]),
    "qcmg_band_lanczos_ptrs": (c_int, [vp, c_int, vp, c_int, c_int, c_double, c_double, int_p,
                                       vp, vp, c_int]),
    "qcmg_band_lanczos_device": (c_int, [vp, c_int, vp, c_int, c_int, c_double, c_double, int_p,
                                         vp, vp, c_int]),
    "qcmg_lanczos_green": (c_int, [vp, vp, c_uint, c_double, c_int, int_p, vp, vp, c_int]),
    "qcmg_block_lanczos": (c_int, [vp, c_int, vp, c_uint, c_int, c_int, c_double, c_double, int_p,
                                   int_p, vp, vp, vp, c_int]),
    "qcmg_apply_c": (c_int, [c_int, c_int, c_int, c_int, c_int, vp, vp, c_double, c_uint]),
    "qcmg_green_function": (c_int, [c_int, c_int, vp, vp, c_int, vp, vp]),
    "qcmg_self_energy": (c_int, [c_int, c_int, vp, vp, c_int, vp, vp, vp, c_int, vp, vp, vp]),
    "qcmg_lattice_create": (c_int, [c_int, c_int, vp, c_int, vp, vp, vp, vp, vp, vp,
                                    ctypes.POINTER(vp)]),
    "qcmg_lattice_destroy": (c_int, [vp]),
    "qcmg_lattice_set_green": (c_int, [vp, c_int, vp, vp, c_int, vp, vp]),
    "qcmg_sef_grid": (c_int, [vp, c_int, vp, vp, c_int, c_int, c_int, dbl_p]),
    "qcmg_cpt_periodized": (c_int, [vp, c_int, vp, c_int, vp, vp]),
    "qcmg_cdmft_projected": (c_int, [vp, c_int, vp, c_int, c_int, vp]),
    "qcmg_lattice_kmean": (c_int, [vp, c_int, vp, c_int, c_int, c_int, c_double, vp]),
    "qcmg_lattice_kmoments": (c_int, [vp, c_int, vp, c_int, c_int, c_int, c_double, c_int, vp, vp]),
    "qcmg_bath_fit": (c_int, [c_int, c_int, c_int, c_int, vp, vp, vp, c_int, c_int, vp, vp, vp, vp,
                              vp, vp, vp, vp, c_int, c_double, c_double, c_double, vp, vp, vp]),
    "qcmg_mlp_create": (c_int, [c_int, vp, ctypes.POINTER(vp)]),
    "qcmg_mlp_destroy": (c_int, [vp]),
    "qcmg_mlp_num_params": (c_int, [vp, size_p]),
    "qcmg_mlp_set_params": (c_int, [vp, vp]),
    "qcmg_mlp_get_params": (c_int, [vp, vp]),
    "qcmg_mlp_forward": (c_int, [vp, c_int, vp, vp]),
    "qcmg_mlp_loss_grad": (c_int, [vp, c_int, vp, vp, vp, vp]),
    "qcmg_mlp_train": (c_int, [vp, c_int, vp, vp, c_int, c_int, ctypes.c_float, ctypes.c_uint,
                               vp]),
}


def exported_symbols():
    return sorted(SIGNATURES)


def lib():
    """Loads libqcmg.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise QcmgError(-5, f"native library missing: {LIB_PATH}")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().qcmg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code):
    if code != 0:
        raise QcmgError(code, last_error())


def ptr(a):
    """Data pointer of a C-contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags.c_contiguous, "array must be C-contiguous"
    return a.ctypes.data


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)
