"""Operator, parameter and optimizer classes shared by ``primaldualtoolbox.mri`` and ``.denoising``.

They mirror the reference's boost.python classes (python/pyMriReconstruction.cpp:112-268,
python/pyDenoising.cpp:39-94): the same class and method names, numpy arrays in C order (ImageUtilities
order reversed), float32 / complex64 data, and exceptions where the reference throws.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import Buffer, check, lib


# ---------------------------------------------------------------------------------------------------
# Parameters (TvParameters, TgvParameters, TgvMriParameters). getParameters() returns a live view:
# assignments write through to the optimizer as the reference's return_internal_reference does.
# ---------------------------------------------------------------------------------------------------
class _Params:
    _fields: tuple = ()
    _title = ""
    _order: tuple = ()

    def __init__(self, owner=None):
        # `owner` is the optimizer object itself, kept alive by this view (return_internal_reference)
        object.__setattr__(self, "_owner", owner)
        if owner is None:
            p = _lib.pdt_params(1.0, 1.0, 1.0, 1.0, 1, 100)
            object.__setattr__(self, "_local", p)

    def _get(self):
        if self._owner is None:
            return self._local
        p = _lib.pdt_params()
        check(lib.pdt_opt_get_params(self._owner._h, ctypes.byref(p)))
        return p

    def _set(self, p):
        if self._owner is None:
            object.__setattr__(self, "_local", p)
        else:
            check(lib.pdt_opt_set_params(self._owner._h, ctypes.byref(p)))

    def __getattr__(self, name):
        fields = type(self)._fields
        if name in fields:
            v = getattr(self._get(), fields[name])
            return int(v) if name in ("max_iter", "check") else float(v)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        fields = type(self)._fields
        if name not in fields:
            raise AttributeError(f"{type(self).__name__} has no attribute {name!r}")
        p = self._get()
        if name in ("max_iter", "check"):
            value = int(value)
            if value < 0:
                raise OverflowError("can't convert negative value to unsigned int")
            setattr(p, fields[name], value)
        else:
            setattr(p, fields[name], float(np.float32(value)))  # the reference stores floatX = float
        self._set(p)

    def __str__(self):
        lines = [f"{self._title}:"]
        for name in self._order:
            v = getattr(self, name)
            lines.append(f" {name if name != 'Lambda' else 'lambda'}={v:g}" if isinstance(v, float)
                         else f" {name}={v}")
        return "\n".join(lines) + "\n"


class TvParameters(_Params):
    """TvParameters (tvoptimizer.h:31-45): Lambda, max_iter, check."""
    _fields = {"Lambda": "lambda_", "max_iter": "max_iter", "check": "check"}
    _title = "TvParameters"
    _order = ("check", "Lambda", "max_iter")


class TgvParameters(_Params):
    """TgvParameters (tgvoptimizer.h:34-66): Lambda, max_iter, check, alpha0, alpha1."""
    _fields = {"Lambda": "lambda_", "max_iter": "max_iter", "check": "check", "alpha0": "alpha0",
               "alpha1": "alpha1"}
    _title = "TgvParameters"
    _order = ("check", "Lambda", "alpha0", "alpha1", "max_iter")


class TgvMriParameters(_Params):
    """TgvMriParameters (tgvmrioptimizer.h:32-66): reduction, max_iter, check, alpha0, alpha1."""
    _fields = {"reduction": "reduction", "max_iter": "max_iter", "check": "check", "alpha0": "alpha0",
               "alpha1": "alpha1"}
    _title = "TgvMriParameters"
    _order = ("alpha0", "alpha1", "check", "reduction", "max_iter")


# ---------------------------------------------------------------------------------------------------
# Operators
# ---------------------------------------------------------------------------------------------------
class _Operator:
    _kind = -1
    _input_dtype = np.complex64
    _output_dtype = np.complex64

    def __init__(self, config=None):
        h = ctypes.c_void_p()
        kvs, keep = None, []
        n = 0
        if config is not None:
            if not isinstance(config, dict):
                raise TypeError("config must be a dict")
            n = len(config)
            kvs = (_lib.pdt_kv * max(1, n))()
            for k, (key, val) in enumerate(config.items()):
                kb, vb = str(key).encode(), str(val).encode()  # values go through str() like the reference
                keep += [kb, vb]
                kvs[k].key, kvs[k].value = kb, vb
        check(lib.pdt_op_create(self._kind, kvs, n, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pdt_op_destroy(h)
            self._h = None

    def _add_constant(self, arr, dtype, pdt_dtype):
        b = Buffer(arr, dtype)
        size = _lib.iu_size(b.shape)
        check(lib.pdt_op_add_constant(self._h, pdt_dtype, len(b.shape), size, b.ptr, b.is_device))

    def replaceConstant(self, idx, arr, stream=None):
        """Replaces constant `idx` (same type and rank) in place, ordered on `stream` -- e.g. the coil
        sensitivities of the next slice. No counterpart in the reference (pdt_op_replace_constant)."""
        types = self._constant_types
        c = types[idx] if 0 <= idx < len(types) else (np.asarray(arr).dtype, _lib.C64)  # the engine reports it
        b = Buffer(arr, c[0])
        size = _lib.iu_size(b.shape)
        check(lib.pdt_op_replace_constant(self._h, int(idx), c[1], len(b.shape), size, b.ptr, b.is_device,
                                          _lib.stream_handle(stream)))

    def _apply(self, adjoint, arr, out=None, stream=None):
        src = Buffer(arr, np.complex64)
        ssize = _lib.iu_size(src.shape)
        nd = ctypes.c_int()
        dsize = (ctypes.c_int64 * 4)()
        fn = lib.pdt_op_input_size if adjoint else lib.pdt_op_output_size
        check(fn(self._h, len(src.shape), ssize, ctypes.byref(nd), dsize))
        dshape = _lib.np_shape(nd.value, dsize)
        if src.is_device:
            if out is None:
                raise ValueError("device inputs need a device `out` array")
            dst = Buffer(out, np.complex64)
            if dst.shape != dshape:
                raise ValueError(f"out has shape {dst.shape}, expected {dshape}")
            res = out
        else:
            res = np.empty(dshape, dtype=np.complex64)
            dst = Buffer(res, np.complex64)
        call = lib.pdt_op_adjoint if adjoint else lib.pdt_op_forward
        check(call(self._h, src.ptr, len(src.shape), ssize, dst.ptr, len(dshape), _lib.iu_size(dshape),
                   src.is_device, _lib.stream_handle(stream)))
        return res

    def forward(self, x, out=None, stream=None):
        """Apply the forward operator (image -> k-space)."""
        return self._apply(False, x, out, stream)

    def adjoint(self, y, out=None, stream=None):
        """Apply the adjoint operator (k-space -> image)."""
        return self._apply(True, y, out, stream)

    def norm(self, iters=30, seed=0):
        """Operator norm ||K|| by power iteration on K^H K with FP64 norms (the TGV step sizes assume <= 1)."""
        out = ctypes.c_double()
        check(lib.pdt_op_norm(self._h, int(iters), int(seed), ctypes.byref(out)))
        return out.value

    def adjointnessCheck(self, seed=42):
        """Random u, p: returns (<Au, p>, <u, A^H p>) as complex numbers (adjointnessCheck of the reference)."""
        out = (ctypes.c_double * 4)()
        check(lib.pdt_op_adjointness(self._h, int(seed), out))
        return complex(out[0], out[1]), complex(out[2], out[3])

    def tuning(self):
        """The kernel configuration the autotuner picked for this operator (text)."""
        buf = ctypes.create_string_buffer(1024)
        check(lib.pdt_op_tuning(self._h, buf, 1024))
        return buf.value.decode()

    def __str__(self):
        buf = ctypes.create_string_buffer(512)
        check(lib.pdt_op_describe(self._h, buf, 512))
        return buf.value.decode()


# ---------------------------------------------------------------------------------------------------
# Optimizers
# ---------------------------------------------------------------------------------------------------
class _Optimizer:
    _kind = -1
    _dtype = np.complex64
    _params_cls = TvParameters
    _operators: tuple = ()

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib.pdt_opt_create(self._kind, _lib.C64 if self._dtype == np.complex64 else _lib.F32, ctypes.byref(h)))
        self._h = h
        self._op = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pdt_opt_destroy(h)
            self._h = None

    def getParameters(self):
        return self._params_cls(self)

    _noisy_shape = None
    _tgv = True
    _with_op = True

    def setNoisyData(self, f, stream=None):
        b = Buffer(f, self._dtype)
        self._noisy_shape = b.shape
        check(lib.pdt_opt_set_noisy_data(self._h, b.ptr, len(b.shape), _lib.iu_size(b.shape), b.is_device,
                                         _lib.stream_handle(stream)))

    def _set_input0(self, u0, stream=None):
        b = Buffer(u0, self._dtype)
        check(lib.pdt_opt_set_input0(self._h, b.ptr, len(b.shape), _lib.iu_size(b.shape), b.is_device,
                                     _lib.stream_handle(stream)))

    def _set_operator(self, op):
        if self._operators and not isinstance(op, self._operators):
            names = ", ".join(c.__name__ for c in self._operators)
            raise TypeError(f"setOperator expects one of: {names}")
        check(lib.pdt_opt_set_operator(self._h, op._h))
        self._op = op

    FIELDS = {"u": 0, "ubar": 1, "vx": 2, "vy": 3, "vbarx": 4, "vbary": 5, "px": 6, "py": 7, "qxx": 8, "qyy": 9,
              "qxy": 10, "r": 11}
    _TV_FIELDS = ("u", "ubar", "px", "py")

    def setInput0UV(self, u0, v0=None, stream=None):
        """Warm start of both TGV primals: u = u0, v = v0 (shape (2, H, W): vx, vy); duals reset to 0."""
        b = Buffer(u0, self._dtype)
        vb = None if v0 is None else Buffer(v0, self._dtype)
        if vb is not None and vb.is_device != b.is_device:
            raise ValueError("u0 and v0 must both be host or both be device arrays")
        check(lib.pdt_opt_set_input0_uv(self._h, b.ptr, vb.ptr if vb else None, len(b.shape), _lib.iu_size(b.shape),
                                        b.is_device, _lib.stream_handle(stream)))

    def _field_shape(self, name):
        if name == "r":
            if self._noisy_shape is None:
                raise _lib.PdtError(5, "No noisy data is set!")
            return self._noisy_shape
        nd = ctypes.c_int()
        size = (ctypes.c_int64 * 4)()
        check(lib.pdt_opt_result_size(self._h, ctypes.byref(nd), size))
        return _lib.np_shape(nd.value, size)

    def getField(self, name, out=None, stream=None):
        """One plane of the solver state ('u', 'ubar', 'vx', 'vy', 'vbarx', 'vbary', 'px', 'py', 'qxx', 'qyy',
        'qxy'), or 'r', the k-space dual of the with-operator optimizers, shaped like the noisy data."""
        shape = self._field_shape(name)
        if out is None:
            out = np.empty(shape, dtype=self._dtype)
        b = Buffer(out, self._dtype)
        if b.shape != shape:
            raise ValueError(f"out has shape {b.shape}, expected {shape}")
        check(lib.pdt_opt_get_field(self._h, self.FIELDS[name], b.ptr, b.is_device, _lib.stream_handle(stream)))
        return out

    def setField(self, name, arr, stream=None):
        """Replace one plane of the solver state (names as getField); the next solve() continues from it."""
        shape = self._field_shape(name)
        b = Buffer(arr, self._dtype)
        if b.shape != shape:
            raise ValueError(f"{name} has shape {b.shape}, expected {shape}")
        check(lib.pdt_opt_set_field(self._h, self.FIELDS[name], b.ptr, b.is_device, _lib.stream_handle(stream)))

    def _state_names(self):
        names = list(self.FIELDS) if self._tgv else list(self._TV_FIELDS) + ["r"]
        return names if self._with_op else [n for n in names if n != "r"]

    def getState(self, stream=None):
        """Every primal and dual variable as a dict of numpy arrays (u, ubar, v, vbar, p, q and, with an
        operator, r): with setState it resumes a solve exactly in another optimizer or process."""
        return {n: self.getField(n, stream=stream) for n in self._state_names()}

    def setState(self, state, stream=None):
        """Import a state exported by getState (setNoisyData and setInput0 first: they size the state)."""
        for n in self._state_names():
            self.setField(n, state[n], stream=stream)

    def energy(self, stream=None):
        """FP64 energy of the current state: {'total', 'data', 'first_order', 'second_order'}."""
        out = (ctypes.c_double * 4)()
        check(lib.pdt_opt_energy(self._h, _lib.stream_handle(stream), out))
        return {"total": out[0], "data": out[1], "first_order": out[2], "second_order": out[3]}

    def gap(self, stream=None):
        """FP64 primal-dual gap of a with-operator optimizer: {'gap', 'primal', 'dual', 'residual_u'
        (|div p - K^H r|), 'residual_v' (|p + div_h q|), 'norm_khr' (|K^H r|)}; gap and residuals vanish
        at the saddle point."""
        out = (ctypes.c_double * 6)()
        check(lib.pdt_opt_gap(self._h, _lib.stream_handle(stream), out))
        keys = ("gap", "primal", "dual", "residual_u", "residual_v", "norm_khr")
        return {k: out[i] for i, k in enumerate(keys)}

    def solve(self, verbose=False, stream=None):
        """Run max_iter + 1 primal-dual iterations (asynchronous when a stream is given). Without a stream,
        raises PdtError (PDT_ERR_NUMERIC) when a NaN or Inf appeared in u or v (with-operator solvers)."""
        check(lib.pdt_opt_solve(self._h, int(bool(verbose)), _lib.stream_handle(stream)))

    def setSteps(self, tau=0.0, sigma=0.0):
        """Primal / dual step sizes of the following solves (with-operator optimizers); 0 restores the
        reference's (tau = 1/16 for TGV-MRI, else 1/8; sigma = 1/8)."""
        check(lib.pdt_opt_set_steps(self._h, float(tau), float(sigma)))

    def checkFinite(self, stream=None):
        """The non-finite check of solves enqueued on a stream: waits for it and raises PdtError
        (PDT_ERR_NUMERIC) if a NaN or Inf appeared in u or v since the last check."""
        check(lib.pdt_opt_status(self._h, _lib.stream_handle(stream)))

    def profile(self, iters=10, stream=None):
        """Run `iters` further iterations launch by launch and return {kernel phase: mean ms per iteration}
        measured with CUDA events on the launching stream (advances the state like solve())."""
        n = ctypes.c_int()
        ms = (ctypes.c_double * 16)()
        names = ctypes.create_string_buffer(1024)
        check(lib.pdt_opt_profile(self._h, int(iters), _lib.stream_handle(stream), 16, ctypes.byref(n), names, 1024,
                                  ms))
        keys = names.value.decode().split(",") if n.value else []
        return {k: ms[i] for i, k in enumerate(keys)}

    def getResult(self, out=None, stream=None):
        """The primal variable u as a numpy array (or copied into the device array `out`)."""
        nd = ctypes.c_int()
        size = (ctypes.c_int64 * 4)()
        check(lib.pdt_opt_result_size(self._h, ctypes.byref(nd), size))
        shape = _lib.np_shape(nd.value, size)
        if out is not None:
            b = Buffer(out, self._dtype)
            if b.shape != shape:
                raise ValueError(f"out has shape {b.shape}, expected {shape}")
            check(lib.pdt_opt_get_result(self._h, b.ptr, b.is_device, _lib.stream_handle(stream)))
            return out
        res = np.empty(shape, dtype=self._dtype)
        check(lib.pdt_opt_get_result(self._h, res.ctypes.data_as(ctypes.c_void_p), 0, _lib.stream_handle(stream)))
        return res
