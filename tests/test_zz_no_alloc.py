"""pargo_sca_noalloc -- SCA for callers that cannot allocate device memory.

Such callers (a plugin that is handed device buffers and a stream only, a host
runtime that owns the device-memory budget) get the SCA through an entry point
whose scratch is a fixed array inside the library, not a context.  This file
runs last.  Through the C ABI it checks that calls in a row -- smaller then
larger, larger then smaller, a padded pitch with float32 output -- give
exactly what the context-based pargo_sca and the oracle give (SCA is
bit-exact, so the tolerance is zero), that a warm call leaves the device's
free memory unchanged, and that rasters beyond the fixed scratch or with a
misaligned pointer or pitch are refused before anything is launched.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import bits_equal

pytestmark = pytest.mark.gpu

ND = -9999.0


def _codes(seed, shape):
    import oracle
    from pargo_gb300 import synth
    O = oracle.Oracle()
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed)
    d8 = O.d8(O.fill(dem, ND), ND)
    return d8, np.where(d8 == ND, -128, d8).astype(np.int8)


def _noalloc(codes_t, out_t, contract, out_nodata=ND):
    from pargo_gb300 import abi
    return abi.lib().pargo_sca_noalloc(ctypes.byref(abi.raster(codes_t, -128)),
                                       ctypes.byref(abi.raster(out_t, out_nodata)), None, contract, None)


@pytest.mark.parametrize("contract", [0, 1])
def test_sca_noalloc_matches_pargo_sca_and_oracle_on_calls_in_a_row(contract, oracle_lib):
    from pargo_gb300 import abi
    ctx = abi.Context(0)
    # smaller -> larger -> smaller: a call after a larger one finds stale scratch
    # beyond its own cells and must not read it
    for seed, shape in ((61, (513, 700)), (62, (1024, 1024)), (63, (300, 400))):
        d8, codes = _codes(seed, shape)
        ct = torch.from_numpy(codes).cuda()
        ref = torch.full(shape, 7.0, dtype=torch.float64, device="cuda")
        ctx.sca(abi.raster(ct, -128), abi.raster(ref, ND), contract=contract)
        out = torch.full(shape, 5.0, dtype=torch.float64, device="cuda")
        assert _noalloc(ct, out, contract) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert bits_equal(got, ref.cpu().numpy()), shape
        assert bits_equal(got, oracle_lib.sca(d8, ND, shipped=bool(contract))), shape
    ctx.close()


def test_sca_noalloc_padded_pitch_float32_output(oracle_lib):
    from pargo_gb300 import abi
    d8, codes = _codes(64, (257, 301))
    cbuf = torch.full((257, 320), -128, dtype=torch.int8, device="cuda")     # 320-byte rows
    cbuf[:, :301] = torch.from_numpy(codes).cuda()
    obuf = torch.full((257, 304), 3.0, dtype=torch.float32, device="cuda")   # 1216-byte rows
    assert _noalloc(cbuf[:, :301], obuf[:, :301], 0) == 0
    torch.cuda.synchronize()
    want = oracle_lib.sca(d8, ND).astype(np.float32)
    assert np.array_equal(obuf[:, :301].cpu().numpy(), want)
    assert (obuf[:, 301:].cpu().numpy() == 3.0).all()        # nothing written past the row


def test_sca_noalloc_warm_call_allocates_nothing():
    _, codes = _codes(65, (640, 512))
    ct = torch.from_numpy(codes).cuda()
    out = torch.empty((640, 512), dtype=torch.float64, device="cuda")
    assert _noalloc(ct, out, 0) == 0                           # warm: the array's address is known
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for contract in (0, 1, 0):
        assert _noalloc(ct, out, contract) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_sca_noalloc_refuses_rasters_beyond_its_scratch():
    codes = torch.full((1025, 1024), -1, dtype=torch.int8, device="cuda")
    out = torch.empty((1025, 1024), dtype=torch.float64, device="cuda")
    assert _noalloc(codes, out, 0) == 1  # PARGO_ERR_INVALID_ARG


def test_sca_noalloc_refuses_misaligned_pointer_and_pitch():
    """Refused on the host before any launch: a float64 output one byte off
    its alignment, and a pitch that is not a whole number of elements."""
    from pargo_gb300 import abi
    L = abi.lib()
    codes = torch.full((64, 64), -1, dtype=torch.int8, device="cuda")
    raw = torch.empty(64 * 64 * 8 + 64, dtype=torch.uint8, device="cuda")
    rc_codes = abi.raster(codes, -128)
    bad_ptr = abi.Raster(raw.data_ptr() + 1, abi.F64, abi.DEVICE, 64, 64, 0, ND, 1.0)
    assert L.pargo_sca_noalloc(ctypes.byref(rc_codes), ctypes.byref(bad_ptr), None, 0, None) == 1
    bad_pitch = abi.Raster(raw.data_ptr(), abi.F64, abi.DEVICE, 64, 64, 64 * 8 + 4, ND, 1.0)
    assert L.pargo_sca_noalloc(ctypes.byref(rc_codes), ctypes.byref(bad_pitch), None, 0, None) == 1
    short_pitch = abi.Raster(raw.data_ptr(), abi.F64, abi.DEVICE, 64, 64, 64 * 8 - 8, ND, 1.0)
    assert L.pargo_sca_noalloc(ctypes.byref(rc_codes), ctypes.byref(short_pitch), None, 0, None) == 1
    # dimensions whose product overflows 64 bits must not slip under the cell limit
    huge_in = abi.Raster(codes.data_ptr(), abi.I8, abi.DEVICE, 1 << 40, 1 << 40, 0, -128.0, 1.0)
    huge_out = abi.Raster(raw.data_ptr(), abi.F64, abi.DEVICE, 1 << 40, 1 << 40, 0, ND, 1.0)
    assert L.pargo_sca_noalloc(ctypes.byref(huge_in), ctypes.byref(huge_out), None, 0, None) == 1
