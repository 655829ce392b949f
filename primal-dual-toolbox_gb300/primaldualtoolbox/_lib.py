"""ctypes binding of libpdt.so (include/pdt.h) and the array plumbing shared by ``mri`` and ``denoising``.

The engine is native (CUDA for sm_103a); this module only marshals arrays. There is no CPU fallback:
if libpdt.so has not been built, importing ``primaldualtoolbox`` raises ImportError.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_PKG), "_build", "libpdt.so")

# pdt_status
OK = 0
STATUS_NAMES = {0: "PDT_OK", 1: "PDT_ERR_INVALID_ARGUMENT", 2: "PDT_ERR_SIZE", 3: "PDT_ERR_CONSTANTS",
                4: "PDT_ERR_CONFIG", 5: "PDT_ERR_STATE", 6: "PDT_ERR_CUDA", 7: "PDT_ERR_UNSUPPORTED",
                8: "PDT_ERR_NUMERIC", 9: "PDT_ERR_TIMEOUT", 10: "PDT_ERR_ALLOC"}
# pdt_dtype
F32, C64 = 0, 1
# pdt_op_kind
OP_CARTESIAN, OP_CARTESIAN_ROOS, OP_SAMPLING, OP_RADIAL, OP_RADIAL_SINGLECOIL = range(5)
# pdt_opt_kind
OPT_TV, OPT_TGV, OPT_TV_OP, OPT_TGV_OP, OPT_TGV_MRI = range(5)

EXPORTED = ["pdt_last_error", "pdt_version", "pdt_launch_count", "pdt_host_alloc", "pdt_host_free",
            "pdt_stream_synchronize", "pdt_op_create", "pdt_op_destroy", "pdt_op_add_constant", "pdt_op_input_size",
            "pdt_op_output_size", "pdt_op_forward", "pdt_op_adjoint", "pdt_op_describe", "pdt_op_adjointness",
            "pdt_op_tuning", "pdt_op_replace_constant",
            "pdt_opt_create", "pdt_opt_destroy", "pdt_opt_get_params", "pdt_opt_set_params", "pdt_opt_set_operator",
            "pdt_opt_set_noisy_data", "pdt_opt_set_input0", "pdt_opt_solve", "pdt_opt_result_size",
            "pdt_opt_get_result", "pdt_opt_profile", "pdt_opt_set_input0_uv", "pdt_opt_get_field", "pdt_opt_energy",
            "pdt_opt_gap", "pdt_opt_set_field", "pdt_opt_status", "pdt_debug_drop_arrival", "pdt_opt_set_steps",
            "pdt_op_norm", "pdt_dist2", "pdt_batch_create", "pdt_batch_destroy", "pdt_batch_add",
            "pdt_batch_solve", "pdt_cnn_create", "pdt_cnn_destroy", "pdt_cnn_num_params", "pdt_cnn_get_params",
            "pdt_cnn_set_params", "pdt_cnn_get_grads", "pdt_cnn_train_step", "pdt_cnn_predict",
            "pdt_cartesian_forward_noalloc"]


class PdtError(RuntimeError):
    """An error reported by the engine (the reference raises IuException at the same places)."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.status_name = STATUS_NAMES.get(status, str(status))


class pdt_kv(ctypes.Structure):
    _fields_ = [("key", ctypes.c_char_p), ("value", ctypes.c_char_p)]


class pdt_params(ctypes.Structure):
    _fields_ = [("alpha0", ctypes.c_double), ("alpha1", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("reduction", ctypes.c_double), ("max_iter", ctypes.c_uint32), ("check", ctypes.c_uint32)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libpdt.so is not built ({LIB_PATH}); run `python -c 'import __graft_entry__ as g; "
                          f"g.build()'` or `python primal-dual-toolbox_gb300/build_native.py`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, i64p, st = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.c_int
    L.pdt_last_error.restype = ctypes.c_char_p
    L.pdt_launch_count.restype = ctypes.c_uint64
    L.pdt_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    L.pdt_host_free.argtypes = [vp]
    L.pdt_stream_synchronize.argtypes = [vp]
    L.pdt_op_create.argtypes = [i, ctypes.POINTER(pdt_kv), i, ctypes.POINTER(vp)]
    L.pdt_op_destroy.argtypes = [vp]
    L.pdt_op_add_constant.argtypes = [vp, i, i, i64p, vp, i]
    L.pdt_op_input_size.argtypes = [vp, i, i64p, ctypes.POINTER(i), i64p]
    L.pdt_op_output_size.argtypes = [vp, i, i64p, ctypes.POINTER(i), i64p]
    L.pdt_op_forward.argtypes = [vp, vp, i, i64p, vp, i, i64p, i, vp]
    L.pdt_op_adjoint.argtypes = [vp, vp, i, i64p, vp, i, i64p, i, vp]
    L.pdt_op_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.pdt_op_tuning.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.pdt_op_adjointness.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]
    L.pdt_opt_create.argtypes = [i, i, ctypes.POINTER(vp)]
    L.pdt_opt_destroy.argtypes = [vp]
    L.pdt_opt_get_params.argtypes = [vp, ctypes.POINTER(pdt_params)]
    L.pdt_opt_set_params.argtypes = [vp, ctypes.POINTER(pdt_params)]
    L.pdt_opt_set_operator.argtypes = [vp, vp]
    L.pdt_opt_set_noisy_data.argtypes = [vp, vp, i, i64p, i, vp]
    L.pdt_opt_set_input0.argtypes = [vp, vp, i, i64p, i, vp]
    L.pdt_opt_solve.argtypes = [vp, i, vp]
    L.pdt_opt_result_size.argtypes = [vp, ctypes.POINTER(i), i64p]
    L.pdt_opt_get_result.argtypes = [vp, vp, i, vp]
    L.pdt_opt_profile.argtypes = [vp, i, vp, i, ctypes.POINTER(i), ctypes.c_char_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_double)]
    L.pdt_opt_set_input0_uv.argtypes = [vp, vp, vp, i, i64p, i, vp]
    L.pdt_opt_get_field.argtypes = [vp, i, vp, i, vp]
    L.pdt_opt_set_field.argtypes = [vp, i, vp, i, vp]
    L.pdt_opt_status.argtypes = [vp, vp]
    L.pdt_opt_set_steps.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.pdt_debug_drop_arrival.argtypes = [i]
    L.pdt_opt_energy.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_double)]
    L.pdt_opt_gap.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_double)]
    L.pdt_op_replace_constant.argtypes = [vp, i, i, i, ctypes.POINTER(ctypes.c_int64), vp, i, vp]
    L.pdt_op_norm.argtypes = [vp, i, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]
    L.pdt_dist2.argtypes = [i, vp, vp, ctypes.c_size_t, vp, ctypes.POINTER(ctypes.c_double)]
    L.pdt_batch_create.argtypes = [ctypes.POINTER(vp)]
    L.pdt_batch_destroy.argtypes = [vp]
    L.pdt_batch_add.argtypes = [vp, vp]
    L.pdt_batch_solve.argtypes = [vp, i, vp]
    L.pdt_cartesian_forward_noalloc.argtypes = [i, vp, vp, i, i, i, vp, vp, vp]
    for name in EXPORTED:
        if name not in ("pdt_last_error", "pdt_version", "pdt_launch_count"):
            getattr(L, name).restype = st
    return L


lib = _load()


def check(status: int) -> None:
    if status != OK:
        raise PdtError(status, lib.pdt_last_error().decode(errors="replace"))


def launch_count() -> int:
    """Kernels launched by libpdt.so since it was loaded (graph replays count each kernel node)."""
    return int(lib.pdt_launch_count())


def iu_size(shape) -> ctypes.Array:
    """numpy shape (slowest first) -> ImageUtilities size array (fastest first)."""
    dims = list(shape)[::-1]
    return (ctypes.c_int64 * max(1, len(dims)))(*dims)


def np_shape(n: int, size) -> tuple:
    return tuple(int(size[k]) for k in range(n))[::-1]


class Buffer:
    """An argument array: a host numpy array or a device array exposing __cuda_array_interface__."""

    def __init__(self, arr, dtype):
        self.keep = arr
        cai = getattr(arr, "__cuda_array_interface__", None)
        if cai is not None:
            want = np.dtype(dtype)
            if np.dtype(cai["typestr"]) != want:
                raise TypeError(f"device array dtype {cai['typestr']} != {want}")
            if cai.get("strides") not in (None, _c_strides(cai["shape"], want.itemsize)):
                raise ValueError("device arrays must be C-contiguous")
            self.ptr = ctypes.c_void_p(int(cai["data"][0]))
            self.shape = tuple(cai["shape"])
            self.is_device = 1
        else:
            a = np.ascontiguousarray(arr, dtype=dtype)
            self.keep = a
            self.ptr = a.ctypes.data_as(ctypes.c_void_p)
            self.shape = a.shape
            self.is_device = 0


def _c_strides(shape, itemsize):
    strides, acc = [], itemsize
    for d in reversed(shape):
        strides.append(acc)
        acc *= d
    return tuple(reversed(strides))


def stream_handle(stream) -> ctypes.c_void_p:
    """None / int handle / object with .cuda_stream (torch.cuda.Stream) -> cudaStream_t."""
    if stream is None:
        return ctypes.c_void_p(None)
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(int(stream.cuda_stream))
    return ctypes.c_void_p(int(stream))


class PinnedArray(np.ndarray):
    """numpy array in page-locked host memory (pdt_host_alloc); freed with the array."""

    def __array_finalize__(self, obj):
        pass


class _PinnedOwner:
    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        check(lib.pdt_host_alloc(nbytes, ctypes.byref(p)))
        self.ptr = p

    def __del__(self):
        try:
            lib.pdt_host_free(self.ptr)
        except Exception:
            pass


def pinned_empty(shape, dtype) -> np.ndarray:
    """An uninitialised numpy array in pinned host memory, for fast host<->device copies."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    owner = _PinnedOwner(max(n, 1))
    buf = (ctypes.c_char * max(n, 1)).from_address(owner.ptr.value)
    arr = np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)
    arr = arr.view(PinnedArray)
    arr._owner = owner
    return arr
