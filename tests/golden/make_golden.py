"""Regenerates the fixtures in tests/golden/ from the reference project's data/ directory.

Run in a checkout that has the reference next to it:  python tests/golden/make_golden.py /path/to/reference
Fixtures (all derived from the reference's own sample data, data/*.npy):
  mask_random4_lines.npy, mask_regular4_lines.npy  sampled phase-encode columns of the 768 x 384 masks
  knee_roos_crop.npy   data/knee_cartesian_reference.npy rows [int(768*0.25+1), int(768*0.75+1)), normalised
                       to max |.| = 1: the input of bin/denoising_complex_test.py
  brain_trajectory.npy data/brain_trajectory.npy (512 samples x 64 spokes, complex k-space positions)
"""
import os
import sys

import numpy as np

here = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
ref = sys.argv[1]
data = os.path.join(ref, "data")

for name in ("random4", "regular4"):
    m = np.load(os.path.join(data, f"mask_cartesian_{name}.npy"))
    assert m.shape == (768, 384)
    cols = np.nonzero(m.any(axis=0))[0].astype(np.int32)
    assert np.array_equal(m, np.repeat((m.any(axis=0))[None].astype(m.dtype), 768, axis=0))  # full lines
    np.save(os.path.join(here, f"mask_{name}_lines.npy"), cols)

knee = np.load(os.path.join(data, "knee_cartesian_reference.npy"))
nFE = knee.shape[0]
crop = knee[int(nFE * 0.25 + 1):int(nFE * 0.75 + 1), :]
crop = (crop / np.max(np.abs(crop))).astype(np.complex64)
np.save(os.path.join(here, "knee_roos_crop.npy"), crop)

traj = np.load(os.path.join(data, "brain_trajectory.npy")).astype(np.complex64)
np.save(os.path.join(here, "brain_trajectory.npy"), traj)
print("written to", here)
