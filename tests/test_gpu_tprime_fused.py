"""The one-pass restriction + T' (gm_tprime_inject) against the two-pass
gm_restrict + gm_interp of getNewTprime (computeFunctions.py:2060-2099) on
the single-track and part-scale windows, Level 3 -> Level 2 and Level 2 ->
Level 1: the same restricted coarse field and the same T'.  On these aligned
hierarchies every restriction weight is 0 or 1 to the rounding of the
coordinates (about 1e-12 at the part-scale window's 10 mm), so the two agree
to that rounding."""

import copy

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _engine(name, dtype):
    import workloads
    from engine import Engine
    from levels import setup_properties

    cfg = workloads.single_track() if name == "single_track" else workloads.part_scale_raster()
    P = setup_properties(cfg["properties"])
    eng = Engine(copy.deepcopy(cfg), P, 10, 10, dtype=dtype)
    vstart = np.asarray(cfg["properties"]["laser_center"], dtype=float)
    row = np.array([vstart[0] + 0.013, vstart[1] - 0.021, 0.0, 1, 1, 1.5e-6, 200.0])
    eng.set_layer(row)
    eng.move(row, vstart)
    torch.cuda.synchronize()
    return eng


@pytest.mark.parametrize("name", ["single_track", "part_scale"])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 1e-6)])
@pytest.mark.parametrize("fine_lev", [3, 2])
def test_tprime_inject_equals_two_pass(name, dtype, tol, fine_lev):
    eng = _engine(name, dtype)
    key = "inj32" if fine_lev == 3 else "inj21"
    assert eng.tables[key] is not None  # aligned hierarchy: the restriction is an injection
    g = eng.geo
    rng = np.random.default_rng(11)
    nf, nc = g.L[fine_lev].nn, g.L[fine_lev - 1].nn
    fine = torch.as_tensor(300 + 1500 * rng.random(nf), dtype=dtype, device="cuda")
    coarse0 = torch.as_tensor(300 + 1500 * rng.random(nc), dtype=dtype, device="cuda")
    ca, cb = coarse0.clone(), coarse0.clone()
    ta, tb = torch.full_like(fine, np.nan), torch.full_like(fine, np.nan)
    eng._new_tprime(fine_lev, fine, ca, ta, fused=False)
    eng._new_tprime(fine_lev, fine, cb, tb, fused=True)
    torch.cuda.synchronize()
    scale = float(fine.abs().max())
    # the restricted coarse field: the injected fine values (the two-pass weights are 0 / 1 to rounding),
    # the rest untouched
    assert float((ca - cb).abs().max()) <= tol * scale
    assert torch.equal(ca == coarse0, cb == coarse0) and int((cb != coarse0).sum()) > 0
    assert float((ta - tb).abs().max()) <= tol * scale
    assert bool(torch.isfinite(tb).all())
