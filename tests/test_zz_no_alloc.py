"""pargo_sca_noalloc -- SCA for callers that cannot allocate device memory.

Such callers (a plugin that is handed device buffers and a stream only, a host
runtime that owns the device-memory budget) get the SCA through an entry point
whose scratch is a fixed array inside the library, not a context.  This file
runs last: it checks, through the C ABI, that two calls in a row give exactly
what the context-based pargo_sca gives (SCA is bit-exact, so the tolerance is
zero), and that rasters beyond the fixed scratch are refused.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _codes(seed, shape):
    import oracle
    from pargo_gb300 import synth
    O = oracle.Oracle()
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed)
    d8 = O.d8(O.fill(dem, -9999.0), -9999.0)
    return np.where(d8 == -9999.0, -128, d8).astype(np.int8)


@pytest.mark.parametrize("contract", [0, 1])
def test_sca_noalloc_matches_pargo_sca_on_two_calls(contract):
    from pargo_gb300 import abi
    L = abi.lib()
    ctx = abi.Context(0)
    for seed, shape in ((61, (513, 700)), (62, (1024, 1024))):
        codes = torch.from_numpy(_codes(seed, shape)).cuda()
        ref = torch.full(shape, 7.0, dtype=torch.float64, device="cuda")
        ctx.sca(abi.raster(codes, -128), abi.raster(ref, -9999.0), contract=contract)
        out = torch.full(shape, 5.0, dtype=torch.float64, device="cuda")
        rc = L.pargo_sca_noalloc(ctypes.byref(abi.raster(codes, -128)), ctypes.byref(abi.raster(out, -9999.0)),
                                 None, contract, None)
        assert rc == 0
        torch.cuda.synchronize()
        assert bits_equal(out.cpu().numpy(), ref.cpu().numpy())
    ctx.close()


def test_sca_noalloc_refuses_rasters_beyond_its_scratch():
    from pargo_gb300 import abi
    L = abi.lib()
    codes = torch.full((1025, 1024), -1, dtype=torch.int8, device="cuda")
    out = torch.empty((1025, 1024), dtype=torch.float64, device="cuda")
    rc = L.pargo_sca_noalloc(ctypes.byref(abi.raster(codes, -128)), ctypes.byref(abi.raster(out, -9999.0)), None, 0,
                             None)
    assert rc == 1  # PARGO_ERR_INVALID_ARG
