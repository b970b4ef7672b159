"""GPU parity of the bulk-flux column kernel against the oracle, through the
C ABI (host and device entry points).  Tolerance: relative L2 <= 1e-13 per
output array (FP64; the GPU's exp/log/pow differ from glibc's by an ulp and
multiply-adds may be fused), elementwise rtol 1e-11."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

OUTS = ["WindStressX", "WindStressY", "SenHFlx", "QVapMFlx", "LatHFlx", "SfcVelTransCoef",
        "SfcTempTransCoef", "SfcQVapTransCoef", "DelVarImplCPL", "SUwRFlx", "LUwRFlx",
        "SfcHFlx_ns", "SfcHFlx_sr", "DSfcHFlxDTs", "SfcTemp", "SfcAlbedo"]


def _case(synth, nx, ny, seed, ice_frac=0.0):
    lat = np.linspace(-1.5, 1.5, ny)
    rng = np.random.default_rng(seed)
    ice = None
    if ice_frac > 0:
        ice = np.where(rng.uniform(size=(nx, ny)) < ice_frac, rng.uniform(0, 1, (nx, ny)), 0.0)
    d, grid = synth.surface_state(lat, nx, seed=seed, sea_ice=ice, halo_fill=-5.0)
    d["SfcAirTemp"][1:-1, 1:-1] += rng.normal(0, 3.0, (nx, ny))  # both stability branches
    d["ImplCplCoef2"][1:-1, 1:-1, :] = rng.normal(0, 0.01, (nx, ny, 4))
    d.update(synth.flux_outputs(grid[0], grid[1], fill=-999.0))
    return d, grid


def _copy(d):
    return {k: (v.copy(order="F") if v.ndim > 1 else v.copy()) for k, v in d.items()}


def _compare(got, ref, grid):
    IA, JA, IS, IE, JS, JE = grid
    for n in OUTS:
        a, b = got[n], ref[n]
        assert rel_l2(a[IS - 1:IE, JS - 1:JE], b[IS - 1:IE, JS - 1:JE]) <= 1e-13, n
        # elementwise: relative to the array's scale (sensible heat flux and
        # the Richardson number cancel near neutral stability)
        scale = np.nanmax(np.abs(b[IS - 1:IE, JS - 1:JE]))
        assert np.allclose(a, b, rtol=1e-11, atol=1e-12 * scale, equal_nan=True), n
        # halo and untouched slots keep the caller's values
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[:, -1], b[:, -1]), n


@pytest.mark.parametrize("nx,ny,ice", [(12, 8, 0.5), (128, 64, 0.0), (360, 180, 0.2), (1, 1, 0.0)])
def test_flux_host_entry_matches_oracle(dccm, oracle, synth, nx, ny, ice):
    d, grid = _case(synth, nx, ny, seed=nx + ny, ice_frac=ice)
    ref, got = _copy(d), _copy(d)
    oracle.sfc_bulk_flux(ref, *grid)
    dccm.DSFCM_Util_SfcBulkFlux_Get(got, *grid)
    _compare(got, ref, grid)
    # slot 3 of the net-heat-flux outputs is never written
    for n in ("SfcHFlx_ns", "SfcHFlx_sr", "DSfcHFlxDTs"):
        assert np.all(got[n][..., 2] == -999.0)


def test_flux_device_entry_matches_oracle(dccm, oracle, synth, cuda):
    torch = cuda
    d, grid = _case(synth, 256, 128, seed=3, ice_frac=0.3)
    ref = _copy(d)
    oracle.sfc_bulk_flux(ref, *grid)
    dev = {}
    for k, v in d.items():
        if k == "a_Sig1Info":
            dev[k] = v
        else:  # Fortran order == transpose of a C-contiguous tensor
            dev[k] = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
    dccm.DSFCM_Util_SfcBulkFlux_Get(dev, *grid, device=True)
    torch.cuda.synchronize()
    got = {k: (np.asfortranarray(dev[k].cpu().numpy().T) if k != "a_Sig1Info" else v)
           for k, v in d.items()}
    _compare(got, ref, grid)


def test_flux_golden_fixture(dccm, synth):
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "flux_small.npz"))
    IA, JA, IS, IE, JS, JE = (int(z[k]) for k in ("IA", "JA", "IS", "IE", "JS", "JE"))
    d = {k[3:]: np.asfortranarray(z[k]).copy(order="F") for k in z.files if k.startswith("in_")}
    d.update(synth.flux_outputs(IA, JA, fill=0.0))
    dccm.DSFCM_Util_SfcBulkFlux_Get(d, IA, JA, IS, IE, JS, JE)
    it = (slice(IS - 1, IE), slice(JS - 1, JE))
    for n in ("WindStressX", "SenHFlx", "LatHFlx", "DelVarImplCPL", "SfcQVapTransCoef"):
        assert rel_l2(d[n][it], z["out_" + n]) <= 1e-13, n
    assert rel_l2(d["SfcHFlx_ns"][it][..., :2], z["out_SfcHFlx_ns"]) <= 1e-13


def test_flux_empty_interior_is_noop(dccm, synth):
    d, grid = _case(synth, 4, 4, seed=1)
    before = _copy(d)
    IA, JA = grid[0], grid[1]
    dccm.DSFCM_Util_SfcBulkFlux_Get(d, IA, JA, 3, 2, 2, JA - 1)  # IS > IE
    for n in OUTS:
        assert np.array_equal(d[n], before[n], equal_nan=True)
    with pytest.raises(dccm.DccmError):
        dccm.DSFCM_Util_SfcBulkFlux_Get(d, IA, JA, 0, IA, 1, JA)  # IS < 1
