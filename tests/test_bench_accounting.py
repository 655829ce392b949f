"""bench.py's roofline bookkeeping on the CPU: per-launch algorithmic bytes of the TGV-MRI iteration (with
the dual update in its own kernel or in the adjoint-rows launch) and the committed per-launch DRAM traffic,
which must not exceed the algorithmic bytes (no wasted re-reads) plus the constant tables a launch reads."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NS = 92  # sampled phase-encode columns of the 15-coil 640 x 368 workload's 4x mask


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, ROOT)
    import bench as b

    return b


def test_fused_dual_moves_its_bytes_into_the_adjoint_launch(bench):
    apart = bench._phase_bytes(NS, 1)
    fused = bench._phase_bytes(NS, 1, fused_dual=True)
    assert "mri_dual_tgv" not in fused and "mri_dual_tgv" in apart
    assert fused["cart_rows_adj"] == apart["cart_rows_adj"] + apart["mri_dual_tgv"]
    assert sum(fused.values()) == sum(apart.values())
    # dual: u-bar, v-bar (2), p (2), q (3) read and p (2), q (3) written, 8-byte complex values
    assert apart["mri_dual_tgv"] == 8 * (bench.H // 2) * bench.W * 13


def test_committed_traffic_within_algorithmic_bytes(bench):
    traffic = bench._ncu_traffic()
    apart = bench._phase_bytes(NS, 1)
    fused = bench._phase_bytes(NS, 1, fused_dual=True)
    # the tensor-core adjoint also reads its DFT-factor operand tiles (constant operator data, not in the
    # algorithmic bytes): 3 output-column ranges x 6 K chunks x hi/lo x 256 columns x 128 bytes
    tiles = 3 * ((2 * NS + 31) // 32) * 2 * 256 * 128
    assert traffic["cart_rows_adj+dual"] <= fused["cart_rows_adj"] + tiles
    assert traffic["cart_rows_adj"] <= apart["cart_rows_adj"] + tiles
    for k in ("cart_rows_fwd", "cart_cols_prox", "mri_dual_tgv", "mri_primal_tgv"):
        assert 0 < traffic[k] <= apart[k], k


def test_khr_planes_from_the_tuning_report(bench):
    solo_tc = ("W=368 H=640 C=15 sampled_columns=92 rows_fwd=lane_fft(46x8,warps=8) "
               "rows_adj=tensor_dft(tf32x3,n_ranges=3,row_tiles=40x8rows,stages=2,coil_sum_on_chip) "
               "cols=lane_fft(10x64,warps=2) in_batch=lane_fft_rows(batch_adj_groups=2,partials)")
    solo_fft = ("W=256 H=256 C=12 sampled_columns=60 rows_fwd=lane_fft(16x16,warps=4) "
                "rows_adj=lane_fft(warps=2,coil_groups=6,partials,staged) cols=lane_fft(16x16,warps=4) "
                "in_batch=lane_fft_rows(batch_adj_groups=2,partials)")
    cluster = ("rows_adj=lane_fft(warps=2,coil_groups=4,cluster) "
               "in_batch=lane_fft_rows(batch_adj_groups=2,cluster)")
    # alone: one plane from the tensor-core rows (coil sum on chip), one per coil group from the FFT rows
    assert bench._khr_planes(solo_tc) == 1
    assert bench._khr_planes(solo_fft) == 6
    assert bench._khr_planes(cluster) == 1
    # in a batch: the lane-FFT rows with at most two coil groups
    assert bench._batch_khr_planes(solo_tc) == (2, True)
    assert bench._batch_khr_planes(solo_fft) == (2, True)
    assert bench._batch_khr_planes(cluster) == (1, True)
    # an operator without lane-FFT rows (no in_batch report) keeps its solo figure
    assert bench._batch_khr_planes("rows_adj=stockham(coil_groups=3)") == (3, False)
