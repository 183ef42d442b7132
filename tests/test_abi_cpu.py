"""Host-only checks of the C ABI library: it loads, exports every entry point
include/pargo_gpu.h declares, and its host-side parts (neighbourhood parsing,
argument checks before any device work) behave like the reference."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pargo_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:pargo_status|const char\*|int64_t|int)\s+(pargo_\w+)\s*\(", text, re.M)))


def test_header_declares_the_operator_entry_points():
    syms = declared_symbols()
    for s in ("pargo_create", "pargo_destroy", "pargo_slope", "pargo_d8", "pargo_slope_d8", "pargo_fill",
              "pargo_sca", "pargo_batch_slope_d8", "pargo_slope_fwd", "pargo_slope_bwd", "pargo_slope_loss_grad",
              "pargo_nbr_parse", "pargo_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from pargo_gb300 import abi
    L = abi.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert L.pargo_abi_version() == 1


def test_nbr_parse_moore():
    from pargo_gb300 import abi
    n = abi.nbr_parse(abi.MOORE)
    assert (n.count, n.min_row, n.min_col, n.max_row, n.max_col) == (9, -1, -1, 1, 1)


def test_nbr_parse_like_reference_files():
    """neighbor/local.nbr (1 cell), neighbor/moore20.nbr ("1681": automatic 41x41)."""
    from pargo_gb300 import abi
    n = abi.nbr_parse("1\n0 0 1.0\n")
    assert (n.count, n.min_row, n.max_row) == (1, 0, 0)
    n = abi.nbr_parse("1681\n")
    assert (n.count, n.min_row, n.min_col, n.max_row, n.max_col) == (1681, -20, -20, 20, 20)


@pytest.mark.parametrize("text", ["", "0\n", "2\n1 0 1\n0 1 1\n", "2\n0 0 1\n0 0 1\n", "3\n0 0 1\n1 1\n"])
def test_nbr_parse_rejects_what_the_reference_rejects(text):
    """Empty set, no (0,0), duplicates (neighborhood.h:113-137), truncated text."""
    from pargo_gb300 import abi
    with pytest.raises(abi.PargoError) as e:
        abi.nbr_parse(text)
    assert e.value.status == 1


def test_create_without_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pargo_gb300 import abi
    with pytest.raises(abi.PargoError) as e:
        abi.Context(0)
    assert e.value.status_name == "PARGO_ERR_NO_DEVICE"


def test_null_context_is_rejected():
    from pargo_gb300 import abi
    L = abi.lib()
    r = abi.Raster()
    assert L.pargo_slope(None, ctypes.byref(r), ctypes.byref(r), None, 0, 0, None) == 1
    assert L.pargo_fill(None, ctypes.byref(r), ctypes.byref(r), None, None, None, None) == 1
    assert L.pargo_sca(None, ctypes.byref(r), ctypes.byref(r), None, 0, None) == 1
