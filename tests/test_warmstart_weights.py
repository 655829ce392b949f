"""The committed warm-start weights: parameter count of the 8-layer network and the training record."""
import json
import os

import numpy as np

from conftest import PKG_DIR


def test_committed_weights_have_the_network_layout():
    path = os.path.join(PKG_DIR, "primaldualtoolbox", "data", "warmstart_15c_640x368.npz")
    with np.load(path) as z:
        params, meta = z["params"], json.loads(str(z["meta"]))
    # conv_in 2->32, six 32->32, conv_out 32->8: weights 9*Cout*Cin + bias Cout per layer
    n = (9 * 32 * 2 + 32) + 6 * (9 * 32 * 32 + 32) + (9 * 8 * 32 + 8)
    assert params.shape == (n,) and np.all(np.isfinite(params))
    assert meta["shape"] == [15, 640, 368] and meta["target_iters"] > 0
    assert meta["held_out"]["rel_l2_network"] < meta["held_out"]["rel_l2_plain"]
