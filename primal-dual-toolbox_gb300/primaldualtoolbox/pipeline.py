"""primaldualtoolbox.pipeline -- the reference scripts' data layouts, and a streaming multi-slice loop.

Layouts (the reference's bin/ scripts):
  Cartesian, Python (bin/mri_cartesian_test.py:28-37): rawdata and coil sensitivities ``(C, FE, PE)``
      complex, mask ``(FE, PE)``; the ROOS reference image is rows [FE/4 + 1, 3 FE/4 + 1).
  Cartesian, MATLAB (bin/mri_cartesian_test.m:24-33): rawdata and sensitivities ``(FE, PE, C)``.
  Radial, Python (bin/mri_radial_test.py:28-40): trajectory k ``(FE, spokes)`` complex; rawdata
      ``(C, FE, spokes)`` reshaped to ``(C, FE*spokes)`` in C order; trajectory rows ``[imag k, real k]``;
      density weights ``sqrt|k|`` as ``(1, Ns)``.
  Radial, MATLAB (bin/mri_radial_test.m:25-46): rawdata ``(FE, spokes, C)`` reshaped to
      ``(FE*spokes, C)`` in column order; trajectory columns ``[real k, imag k]`` of ``col(k)``.
The converters below return the Python layouts the operators take.

``SliceStream`` reconstructs a sequence of same-sized Cartesian slices, overlapping each slice's
host-to-device upload and the previous slice's device-to-host download with the solve on the GPU.
"""
from __future__ import annotations

import os

import numpy as np

from . import mri


def cartesian_from_matlab(rawdata, sensitivities=None, mask=None):
    """MATLAB-layout Cartesian arrays (FE, PE, C) -> the Python layout (C, FE, PE) complex64; the mask
    (FE, PE) is returned as float32."""
    out = {"rawdata": np.ascontiguousarray(np.transpose(rawdata, (2, 0, 1)), dtype=np.complex64)}
    if sensitivities is not None:
        out["sens"] = np.ascontiguousarray(np.transpose(sensitivities, (2, 0, 1)), dtype=np.complex64)
    if mask is not None:
        out["mask"] = np.ascontiguousarray(mask, dtype=np.float32)
    return out


def roos_crop(image):
    """The readout-oversampling-removed part of a full-FOV image, rows [FE/4 + 1, 3 FE/4 + 1)
    (bin/mri_cartesian_test.py:45-47)."""
    n = image.shape[0]
    return image[int(n * 0.25 + 1):int(n * 0.75 + 1)]


def radial_inputs(k, rawdata, layout="python", trajectory_order="python"):
    """Radial trajectory k (FE, spokes) complex and multi-coil rawdata -> {'trajectory' (2, Ns) float32,
    'dcf' (1, Ns) float32 = sqrt|k|, 'rawdata' (C, Ns) complex64}. layout: 'python' for rawdata
    (C, FE, spokes), 'matlab' for (FE, spokes, C). trajectory_order 'python' gives rows [imag k, real k]
    (the Python sample), 'matlab' rows [real k, imag k] (the MATLAB sample) -- the two samples differ."""
    k = np.asarray(k)
    if layout == "python":
        kc = k.flatten()  # sample index fe * spokes + spoke
        C = rawdata.shape[0]
        raw = np.reshape(rawdata, (C, -1))
    elif layout == "matlab":
        kc = k.flatten(order="F")  # sample index fe + FE * spoke
        nfe, nsp, C = rawdata.shape
        raw = np.reshape(rawdata, (nfe * nsp, C), order="F").T
    else:
        raise ValueError("layout must be 'python' or 'matlab'")
    if trajectory_order == "python":
        traj = np.array([np.imag(kc), np.real(kc)])
    elif trajectory_order == "matlab":
        traj = np.array([np.real(kc), np.imag(kc)])
    else:
        raise ValueError("trajectory_order must be 'python' or 'matlab'")
    return {"trajectory": np.ascontiguousarray(traj, dtype=np.float32),
            "dcf": np.ascontiguousarray(np.sqrt(np.abs(kc))[np.newaxis, :], dtype=np.float32),
            "rawdata": np.ascontiguousarray(raw, dtype=np.complex64)}


def load_array(path, name=None):
    """A .npy array, or a variable of a MATLAB v5 .mat file (the only non-metadata one when `name` is
    None; MATLAB v7.3 / HDF5 files need h5py, which this package does not use)."""
    if path.endswith(".npy"):
        return np.load(path)
    if path.endswith(".mat"):
        from scipy.io import loadmat

        d = {k: v for k, v in loadmat(path).items() if not k.startswith("__")}
        if name is None:
            if len(d) != 1:
                raise ValueError(f"{os.path.basename(path)} holds {sorted(d)}; pass name=")
            return next(iter(d.values()))
        return d[name]
    raise ValueError("expected a .npy or .mat file")


def load_cartesian(rawdata_path, sensitivities_path, mask_path):
    """The Cartesian sample's three files (.npy in the Python layout, or .mat in the MATLAB layout)."""
    raw, sens, mask = (load_array(p) for p in (rawdata_path, sensitivities_path, mask_path))
    if rawdata_path.endswith(".mat"):
        return cartesian_from_matlab(raw, sens, mask)
    return {"rawdata": np.ascontiguousarray(raw, dtype=np.complex64),
            "sens": np.ascontiguousarray(sens, dtype=np.complex64),
            "mask": np.ascontiguousarray(mask, dtype=np.float32)}


class SliceStream:
    """TGV^2 reconstruction (TgvMriOptimizer_2c3c) of a sequence of same-sized Cartesian slices.

    Two slots alternate. Each owns pinned host staging, device buffers, an operator and an optimizer
    that are reused from slice to slice (constants replaced in place), so nothing is allocated or freed
    per slice. Uploads run on one stream, solves on another and downloads on a third, ordered by events:
    the upload of slice i+1 and the download of slice i-1 overlap the solve of slice i.

        stream = SliceStream(C=15, H=640, W=368, roos=True, alpha1=0.05, max_iter=1000)
        for index, image in stream.run(slices):   # slices: dicts of host rawdata, sens, mask
            ...
    """

    def __init__(self, C, H, W, roos=True, alpha1=0.05, alpha0=None, reduction=2e-8, max_iter=1000, torch=None):
        if torch is None:
            import torch
        self.torch = torch
        self.C, self.H, self.W, self.roos = C, H, W, roos
        self.Hi = H // 2 if roos else H
        self.params = dict(alpha1=alpha1, alpha0=2 * alpha1 if alpha0 is None else alpha0, reduction=reduction,
                           max_iter=max_iter)
        self.up, self.compute, self.down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        self.slots = [self._slot() for _ in range(2)]

    def _slot(self):
        t = self.torch
        C, H, W, Hi = self.C, self.H, self.W, self.Hi
        return {"raw_h": t.empty((C, H, W), dtype=t.complex64, pin_memory=True),
                "sens_h": t.empty((C, H, W), dtype=t.complex64, pin_memory=True),
                "out_h": t.empty((Hi, W), dtype=t.complex64, pin_memory=True),
                "raw_d": t.empty((C, H, W), dtype=t.complex64, device="cuda"),
                "sens_d": t.empty((C, H, W), dtype=t.complex64, device="cuda"),
                "u0_d": t.empty((Hi, W), dtype=t.complex64, device="cuda"),
                "u_d": t.empty((Hi, W), dtype=t.complex64, device="cuda"),
                "uploaded": t.cuda.Event(), "solved": t.cuda.Event(), "downloaded": t.cuda.Event(),
                "op": None, "opt": None, "index": None}

    def _issue(self, slot, sl):
        t = self.torch
        slot["raw_h"].numpy()[...] = sl["rawdata"]
        slot["sens_h"].numpy()[...] = sl["sens"]
        with t.cuda.stream(self.up):
            slot["raw_d"].copy_(slot["raw_h"], non_blocking=True)
            slot["sens_d"].copy_(slot["sens_h"], non_blocking=True)
            slot["uploaded"].record(self.up)
        cs = self.compute
        cs.wait_event(slot["uploaded"])
        mask = np.ascontiguousarray(sl["mask"], dtype=np.float32)
        if slot["op"] is None:
            slot["uploaded"].synchronize()  # adding constants copies on the legacy default stream
            op = (mri.MriCartesianRemoveROOSOperator if self.roos else mri.MriCartesianOperator)()
            op.setCoilSens(slot["sens_d"])
            op.setMask(mask)
            opt = mri.TgvMriOptimizer_2c3c()
            prm = opt.getParameters()
            for k, v in self.params.items():
                setattr(prm, k, v)
            opt.setOperator(op)
            slot["op"], slot["opt"] = op, opt
        else:
            slot["op"].replaceCoilSens(slot["sens_d"], stream=cs)
            slot["op"].replaceMask(mask, stream=cs)  # a no-op when the mask is unchanged
        op, opt = slot["op"], slot["opt"]
        opt.setNoisyData(slot["raw_d"], stream=cs)  # r = 0
        op.adjoint(slot["raw_d"], out=slot["u0_d"], stream=cs)
        opt.setInput0(slot["u0_d"], stream=cs)  # u = u-bar = A^H f, v = p = q = 0
        opt.solve(stream=cs)
        opt.getResult(out=slot["u_d"], stream=cs)
        slot["solved"].record(cs)
        self.down.wait_event(slot["solved"])
        with t.cuda.stream(self.down):
            slot["out_h"].copy_(slot["u_d"], non_blocking=True)
            slot["downloaded"].record(self.down)

    def _collect(self, slot):
        slot["downloaded"].synchronize()
        out = (slot["index"], slot["out_h"].numpy().copy())
        slot["index"] = None
        return out

    def run(self, slices):
        """Yields (index, image) for every slice, in order; images are host complex64 (Hi, W) arrays."""
        n = 0
        for i, sl in enumerate(slices):
            slot = self.slots[i % 2]
            if slot["index"] is not None:
                yield self._collect(slot)
            self._issue(slot, sl)
            slot["index"] = i
            n = i + 1
        for i in range(max(0, n - 2), n):
            slot = self.slots[i % 2]
            if slot["index"] is not None:
                yield self._collect(slot)
