"""primaldualtoolbox.batch -- many independent reconstructions advanced together.

    batch = BatchSolver([opt_a, opt_b, ...])   # optimizers with their operators and data set
    batch.solve()                               # same results as opt.solve() on each, in one graph

Problems may differ in size, coil count, sampling mask, optimizer kind and max_iter; each optimizer needs
its own operator object. There is no counterpart in the reference, which solves one reconstruction per
call.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check, lib


class BatchSolver:
    def __init__(self, optimizers=()):
        h = ctypes.c_void_p()
        check(lib.pdt_batch_create(ctypes.byref(h)))
        self._h = h
        self._opts = []
        for o in optimizers:
            self.add(o)

    def add(self, optimizer):
        check(lib.pdt_batch_add(self._h, optimizer._h))
        self._opts.append(optimizer)  # keeps the optimizers (and their operators) alive

    def __len__(self):
        return len(self._opts)

    def solve(self, verbose=False, stream=None):
        """Run every optimizer's max_iter + 1 iterations (asynchronously when a stream is given)."""
        check(lib.pdt_batch_solve(self._h, int(bool(verbose)), _lib.stream_handle(stream)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.pdt_batch_destroy(h)
            self._h = None
