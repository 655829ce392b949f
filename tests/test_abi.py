"""The C ABI library: it loads, exports every entry point include/pdt.h declares, and the host-side
checks behave like the reference's throw sites. No GPU compute is issued here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "pdt.h")).read()
    return sorted(set(re.findall(r"PDT_API\s+[\w\s\*]*?\b(pdt_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    assert "pdt_opt_solve" in names and "pdt_op_forward" in names and len(names) >= 25


def test_library_exports_every_declared_symbol(pdt):
    lib = ctypes.CDLL(pdt.LIB_PATH)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    from primaldualtoolbox import _lib

    assert set(_lib.EXPORTED) == set(_declared())


def test_cartesian_rejects_config(pdt):
    with pytest.raises(pdt.PdtError) as e:
        pdt.mri.MriCartesianOperator.__mro__[1].__init__(pdt.mri.MriCartesianOperator.__new__(
            pdt.mri.MriCartesianOperator), {"osf": 2})
    assert e.value.status_name == "PDT_ERR_CONFIG"
    assert "Invalid amount of configuration parameters (min: 0 max: 0)" in str(e.value)


def test_operator_print(pdt):
    assert str(pdt.mri.MriCartesianOperator()) == "MriCartesianOperator: Added constants: (0/2)"
    assert str(pdt.mri.MriCartesianRemoveROOSOperator()) == "MriCartesianRemoveROOSOperator: Added constants: (0/2)"
    assert str(pdt.mri.MriSamplingOperator()) == "MriSamplingOperator: Added constants: (0/1)"


def test_optimizer_state_errors(pdt):
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    with pytest.raises(pdt.PdtError, match="No operator is set!"):
        opt.solve()
    op = pdt.mri.MriCartesianOperator()
    opt.setOperator(op)
    with pytest.raises(pdt.PdtError, match="No noisy data is set!"):
        opt.solve()
    with pytest.raises(pdt.PdtError, match="There is no result yet!"):
        opt.getResult()
    den = pdt.denoising.TvOptimizer_2f()
    with pytest.raises(pdt.PdtError, match="No noisy data is set!"):
        den.solve()


def test_set_operator_type_check(pdt):
    with pytest.raises(TypeError):
        pdt.mri.TgvMriOptimizer_2c3c().setOperator(pdt.mri.MriSamplingOperator())
    with pytest.raises(TypeError):
        pdt.mri.TgvMriOptimizer_2c2c().setOperator(pdt.mri.MriCartesianOperator())


def test_parameters_defaults_and_write_through(pdt):
    p = pdt.mri.TgvMriParameters()
    assert (p.alpha0, p.alpha1, p.reduction, p.max_iter, p.check) == (1.0, 1.0, 1.0, 1, 100)
    opt = pdt.mri.TgvMriOptimizer_2c3c()
    prm = opt.getParameters()
    prm.max_iter = 1000
    prm.alpha1 = 0.05
    prm.alpha0 = 2 * prm.alpha1
    prm.reduction = 2e-8
    again = opt.getParameters()
    assert again.max_iter == 1000
    assert again.alpha0 == pytest.approx(0.1, rel=1e-6)
    assert again.reduction == float(np.float32(2e-8))
    t = pdt.denoising.TvOptimizer_2f().getParameters()
    t.Lambda = 10
    assert t.Lambda == 10.0
    assert "TvParameters:" in str(t) and "lambda=10" in str(t)
    with pytest.raises(AttributeError):
        t.alpha0 = 1
    with pytest.raises(OverflowError):
        t.max_iter = -1


def test_radial_config_errors(pdt):
    """OperatorBase(..., config, 4, 4) and getConfigDouble/Int (mriradialoperator.cu:28-35)."""
    with pytest.raises(pdt.PdtError, match=r"\(min: 4 max: 4\) required, got \(3\)"):
        pdt.mri.MriRadialOperator({"osf": 2, "sector_width": 8, "kernel_width": 3})
    with pytest.raises(pdt.PdtError, match="could not parse configuration parameter 'osf'"):
        pdt.mri.MriRadialOperator({"osf": "two", "sector_width": 8, "kernel_width": 3, "img_dim": 64})
    # img_dim given as a float, as bin/mri_radial_test.py does (nFE/2), parses like the reference's stringstream
    op = pdt.mri.MriRadialOperator({"osf": 2, "sector_width": 8, "kernel_width": 3, "img_dim": 64 / 2})
    assert str(op) == "MriRadialOperator: Added constants: (0/3)"
    assert str(pdt.mri.MriRadialSinglecoilOperator(
        {"osf": 2, "sector_width": 8, "kernel_width": 3, "img_dim": 32})) == "MriRadialOperator: Added constants: (0/2)"


def test_launch_count_starts_at_zero_without_gpu(pdt):
    assert pdt.launch_count() >= 0
