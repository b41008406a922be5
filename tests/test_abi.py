"""CPU-side checks of the C ABI: the engine library builds for sm_103a, loads,
and exports every entry point include/lfdem_gb300.h declares (no device
calls); the header declares nothing the library lacks."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from lf_dem_gb300 import build as B
    path = B.build()
    return ctypes.CDLL(path)


def declared():
    txt = open(os.path.join(ROOT, "include", "lfdem_gb300.h")).read()
    return sorted(set(re.findall(r"\b(lfg_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_library_agree(lib):
    import lf_dem_gb300 as E
    names = declared()
    assert names, "no declarations found"
    for nm in names:
        assert hasattr(lib, nm), f"{nm} declared but not exported"
    assert sorted(E.EXPORTS) == names


def test_default_options(lib):
    import lf_dem_gb300 as E
    E._lib = None
    o = E.default_options()
    assert o.precision == E.PREC_FP64 and o.use_graphs == 1 and o.refine_tol == 2e-10


def test_no_device_reports_cleanly(lib):
    """Without a GB300 every constructor returns LFG_ERR_NO_DEVICE (no fallback)."""
    import lf_dem_gb300 as E
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(E.LFGError) as ei:
        E.Solver(10)
    assert ei.value.code == E.LFG_ERR_NO_DEVICE
