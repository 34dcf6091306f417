"""ctypes binding of libkitgpu.so (include/kitgpu.h).

The shared library is the only compute path of this package.  Loading fails
loudly when it is missing or when no CUDA device is present; there is no CPU
fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkitgpu.so")

KB_OK = 0
KB_ERR_ARG, KB_ERR_CONFIG, KB_ERR_CUDA, KB_ERR_NUMERIC = -1, -2, -3, -4
KB_ERR_TIMEOUT, KB_ERR_NOMEM, KB_ERR_STATE = -5, -6, -7
ERRORS = {
    -1: "KB_ERR_ARG", -2: "KB_ERR_CONFIG", -3: "KB_ERR_CUDA", -4: "KB_ERR_NUMERIC",
    -5: "KB_ERR_TIMEOUT", -6: "KB_ERR_NOMEM", -7: "KB_ERR_STATE",
}
FLUX = {"kfvs": 0, "kcu": 1, "ugks": 2}
COLLISION = {"bgk": 0, "shakhov": 1}
BOUNDARY = {"fix": 0, "extra": 1, "period": 2, "maxwell": 3}
PRECISION = {"fp64": 0, "fp32": 1}


class KitGPUError(RuntimeError):
    """A libkitgpu call returned a negative status."""

    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "KB_ERR"), code, message))
        self.code = code


class KbConfig(ctypes.Structure):
    """kb_config_t of include/kitgpu.h."""

    _fields_ = [
        ("dim", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("ngx", ctypes.c_int32), ("ngy", ctypes.c_int32),
        ("nu", ctypes.c_int32), ("nv", ctypes.c_int32),
        ("flux", ctypes.c_int32), ("collision", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 4), ("interp_order", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("x0", ctypes.c_double), ("x1", ctypes.c_double),
        ("y0", ctypes.c_double), ("y1", ctypes.c_double),
        ("umax", ctypes.c_double), ("vmax", ctypes.c_double),
        ("K", ctypes.c_double), ("gamma", ctypes.c_double), ("mu_ref", ctypes.c_double),
        ("omega", ctypes.c_double), ("Pr", ctypes.c_double),
        ("nf", ctypes.c_int32),
    ]


_D = ctypes.POINTER(ctypes.c_double)
_H = ctypes.c_void_p
_lib = None

# name -> argtypes (every function returns int)
SIGNATURES = {
    "kb_create": [ctypes.POINTER(KbConfig), _D, _D, _D, ctypes.POINTER(_H)],
    "kb_destroy": [_H],
    "kb_set_wall": [_H, ctypes.c_int, _D],
    "kb_upload_state": [_H, _D, _D, _D, _D],
    "kb_init_equilibrium": [_H, _D, _D],
    "kb_download_state": [_H, _D, _D, _D, _D],
    "kb_timestep": [_H, ctypes.c_double, ctypes.c_double, ctypes.c_double, _D],
    "kb_reconstruct": [_H],
    "kb_evolve": [_H, ctypes.c_double],
    "kb_update": [_H, ctypes.c_double, _D],
    "kb_step": [_H, ctypes.c_double, ctypes.c_int32, _D],
    "kb_step_cfl": [_H, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int32, _D, _D],
    "kb_download_faces": [_H, ctypes.c_double, _D, _D, _D],
    "kb_download_slopes": [_H, _D, _D, _D],
    "kb_upload_slopes": [_H, _D],
    "kb_status": [_H],
    "kb_device_bytes": [_H, ctypes.POINTER(ctypes.c_int64)],
    "kb_launch_count": [_H, ctypes.POINTER(ctypes.c_int64)],
    "kb_set_timing": [_H, ctypes.c_int],
    "kb_get_timing": [_H, _D, ctypes.POINTER(ctypes.c_int64)],
    "kb_get_stream": [_H, ctypes.POINTER(ctypes.c_void_p)],
    "kb_set_tuning": [_H, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32],
    "kb_step_async": [_H, ctypes.c_double, ctypes.c_int32],
    "kb_timestep_noalloc": [ctypes.POINTER(KbConfig), ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p],
    "kb_query": [_H, _D, ctypes.POINTER(ctypes.c_int32)],
    "kb_get_tuning": [_H, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32],
    "kb_wait_probe": [ctypes.c_double, ctypes.POINTER(ctypes.c_int32), _D],
    "kb_group_create": [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)],
    "kb_group_destroy": [ctypes.c_void_p],
    "kb_group_add": [ctypes.c_void_p, _H, ctypes.c_double],
    "kb_group_remove": [ctypes.c_void_p, _H],
    "kb_group_step_async": [ctypes.c_void_p, ctypes.c_int32],
    "kb_group_query": [ctypes.c_void_p, _D, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)],
    "kb_group_info": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)],
}
STAGES = ("reconstruct", "face_param", "moments", "wall", "cell_param", "update", "finish")


def load(path=None):
    """Load libkitgpu.so and declare its signatures (no CUDA call is made)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            "libkitgpu.so not found at %s: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % p)
    lib = ctypes.CDLL(p)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.kb_version.restype = ctypes.c_char_p
    lib.kb_version.argtypes = []
    lib.kb_last_error.restype = ctypes.c_char_p
    lib.kb_last_error.argtypes = []
    if path is None:
        _lib = lib
    return lib


def check(rc):
    if rc != KB_OK:
        raise KitGPUError(rc, load().kb_last_error().decode())
    return rc


def ptr(a):
    """Pointer to a C-contiguous float64 array (or None)."""
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_D)


def cuda_device_count():
    """Number of CUDA devices visible to the runtime (0 without a GPU)."""
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        import glob
        cands = sorted(glob.glob("/usr/local/cuda*/lib64/libcudart.so*"))
        if not cands:
            return 0
        rt = ctypes.CDLL(cands[-1])
    n = ctypes.c_int(0)
    if rt.cudaGetDeviceCount(ctypes.byref(n)) != 0:
        return 0
    return n.value
