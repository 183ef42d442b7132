"""The FP64 CPU adjoint of the Horn slope loss (tests/grad_ref.py), the
reference the GPU gradient is checked against, pinned on the CPU: within
1e-6 relative of FP64 central differences on 10^4 seeded cells, nodata
windows included."""
import numpy as np

from grad_ref import ND, adjoint64, fd_errors
from pargo_gb300 import synth


def test_fp64_adjoint_matches_central_differences():
    R, C, cs = 384, 320, 30.0
    z = synth.slope_dem(R, C, seed=3, hurst=0.75, relief=3000.0)
    z[100:110, 50:60] = ND
    zr = synth.perturbed(z, seed=3, sigma=0.5)
    g64 = adjoint64(z, zr, cs)
    assert (g64[101:109, 51:59] == 0).all()           # no window through nodata contributes
    cells = np.random.default_rng(3).integers(0, R * C, size=10000)
    errs, _, _ = fd_errors(z, zr, cs, g64, cells, h=1e-4)
    assert len(errs) > 9000
    assert errs.max() <= 1e-6, errs.max()
