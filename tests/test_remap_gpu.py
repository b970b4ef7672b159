"""GPU parity of the Jones-99 table generator and the CSR remap apply
against the oracle, through the C ABI.  Integer/index work and the REF
weights are compared bit-exact; the apply is bit-exact too (products and
sums rounded separately in table order, as the reference loop)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def grids(synth):
    g = {
        "T21": synth.gaussian_axes(64, 32),
        "T42": synth.gaussian_axes(128, 64),
        "T85": synth.gaussian_axes(256, 128),
        "1deg": synth.regular_axes(360, 180),
        "zonal": (np.zeros(1), synth.gaussian_axes(1, 64)[1], np.full(1, 2 * np.pi), synth.gaussian_axes(1, 64)[3]),
    }
    return g


CASES = [("T21", "T42", 1, 0), ("T42", "T42", 1, 0), ("T42", "T21", 1, 0), ("T85", "1deg", 1, 0),
         ("T42", "zonal", 1, 0), ("zonal", "T42", 1, 0), ("T21", "T42", 2, 0), ("T42", "T21", 2, 0),
         ("T21", "T42", 1, 1), ("T42", "T21", 1, 1), ("T85", "1deg", 1, 1), ("1deg", "T85", 1, 1)]


def _gen(dccm, S, D, order, mode, mask=None):
    t = dccm.gen_gridmapfile_lonlat2lonlat(S[0], S[1], D[0], D[1], S[2], S[3], D[2], D[3],
                                           accuracy_order=order, weight_mode=mode, dst_mask=mask)
    return t


@pytest.mark.parametrize("src,dst,order,mode", CASES)
def test_j99_table_bit_exact(dccm, oracle, synth, src, dst, order, mode):
    G = grids(synth)
    S, D = G[src], G[dst]
    rows = _gen(dccm, S, D, order, mode).rows()
    ref = oracle.j99_gen(S[0], S[1], D[0], D[1], S[3], D[3], order, mode)
    assert len(rows[0]) == len(ref[0])
    for a, b in zip(rows, ref):
        assert np.array_equal(a, b)


def test_j99_mask_drops_land_rows(dccm, oracle, synth):
    G = grids(synth)
    S, D = G["T85"], G["1deg"]
    mask = synth.land_mask(360, 180, 0.3, seed=0)
    iD, jD, iS, jS, w = _gen(dccm, S, D, 1, 1, mask).rows()
    full = oracle.j99_gen(S[0], S[1], D[0], D[1], S[3], D[3], 1, 1)
    keep = mask[(full[0] - 1) + 360 * (full[1] - 1)] == 1
    assert np.array_equal(iD, full[0][keep]) and np.array_equal(w, full[4][keep])
    assert np.all(mask[(iD - 1) + 360 * (jD - 1)] == 1)


@pytest.mark.parametrize("src,dst,mode", [("T21", "T42", 0), ("T42", "T42", 0), ("T85", "1deg", 1),
                                          ("1deg", "T85", 1), ("T42", "T21", 1)])
def test_interpolate_data_bit_exact(dccm, oracle, synth, src, dst, mode):
    G = grids(synth)
    S, D = G[src], G[dst]
    iD, jD, iS, jS, w = oracle.j99_gen(S[0], S[1], D[0], D[1], S[3], D[3], 1, mode)
    nS, nD = len(S[0]) * len(S[1]), len(D[0]) * len(D[1])
    send, recv = oracle.table_to_index(iD, jD, iS, jS, len(S[0]), len(D[0]))
    plan = dccm.RemapPlan(nS, nD, send, recv, w)
    assert plan.info() == (len(w), nS, nD)
    rng = np.random.default_rng(1)
    fields = np.asfortranarray(rng.standard_normal((nS, 6)) * 300.0)
    ref = oracle.remap_apply(send, recv, w, fields, nD)
    out = np.full((nD, 6), np.nan, order="F")
    plan.interpolate_data(fields, out, 6)
    assert np.array_equal(out, ref)


def test_exchange_pattern_identity_bit_exact(dccm, synth):
    """field_def.f90:586 pattern i + 100 j + 1e4 code through the identity map."""
    lon, lat, lw, w = synth.gaussian_axes(128, 64)
    t = dccm.gen_gridmapfile_lonlat2lonlat(lon, lat, lon, lat, lw, w, lw, w)
    send, recv, coef = t.index(128, 128)
    assert np.all(coef == 1.0) and np.array_equal(send, recv)
    plan = dccm.RemapPlan(8192, 8192, send, recv, coef)
    ii, jj = np.meshgrid(np.arange(1, 129), np.arange(1, 65), indexing="ij")
    f = np.asfortranarray(np.stack([(ii + 100 * jj + 1e4 * c).ravel(order="F") for c in range(1, 7)], 1))
    out = np.zeros((8192, 6), order="F")
    plan.interpolate_data(f, out, 6)
    assert np.array_equal(out, f)


def test_remap_device_entry_and_conservation(dccm, oracle, synth, cuda):
    torch = cuda
    G = grids(synth)
    S, D = G["T85"], G["1deg"]
    t = _gen(dccm, S, D, 1, 1)
    send, recv, coef = t.index(256, 360)
    nS, nD = 256 * 128, 360 * 180
    plan = dccm.RemapPlan(nS, nD, send, recv, coef)
    rng = np.random.default_rng(2)
    f = rng.standard_normal((6, nS)) + 5.0
    src = torch.from_numpy(f).cuda()
    dst = torch.zeros((6, nD), dtype=torch.float64, device="cuda")
    plan.apply_dev(src, nS, dst, nD, 6)
    torch.cuda.synchronize()
    ref = oracle.remap_apply(send, recv, coef, np.asfortranarray(f.T), nD)
    assert np.array_equal(dst.cpu().numpy().T, ref)
    # global area-weighted integrals conserved (true-overlap weights)
    areaS = np.outer(S[3], S[2]).ravel()  # (lat, lon) -> lon fastest
    areaD = np.outer(D[3], D[2]).ravel()
    aS = torch.from_numpy(areaS).cuda()
    aD = torch.from_numpy(areaD).cuda()
    for k in range(6):
        IS_ = dccm.area_integral_dev(src[k].contiguous(), aS)
        ID_ = dccm.area_integral_dev(dst[k].contiguous(), aD)
        assert abs(ID_ - IS_) / abs(IS_) <= 1e-12
        assert abs(IS_ - oracle.area_integral(f[k], areaS)) <= 1e-14 * abs(IS_)


def test_plan_rejects_out_of_range_indices(dccm, oracle, synth):
    """Coarsening in REF mode writes source indices <= 0 for the wrap cell
    (a reference defect); with jS = 1 the linear index leaves the grid and
    the plan refuses it instead of reading out of bounds."""
    G = grids(synth)
    S, D = G["T42"], G["T21"]
    iD, jD, iS, jS, w = _gen(dccm, S, D, 1, 0).rows()
    assert (iS <= 0).any()
    send, recv = oracle.table_to_index(iD, jD, iS, jS, 128, 64)
    with pytest.raises(dccm.DccmError) as e:
        dccm.RemapPlan(128 * 64, 64 * 32, send, recv, w)
    assert e.value.status == -4


def test_empty_table_zeroes_recv(dccm):
    plan = dccm.RemapPlan(10, 7, np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0))
    out = np.full((7, 3), 4.0, order="F")
    plan.interpolate_data(np.ones((10, 3), order="F"), out, 3)
    assert np.all(out == 0.0)


@pytest.mark.parametrize("fc,threads", [(0, 0), (1, 32), (2, 64), (3, 128), (4, 256), (6, 96)])
def test_sliced_apply_ragged_rows_bit_exact(dccm, oracle, cuda, fc, threads):
    """Rows of 0 to 40 entries (empty rows and long rows in one 32-row
    slice), 7 fields (not a multiple of the fields a thread takes), every
    launch shape: bit-exact against the oracle's COO loop, including the
    sign of zero (0 + -0 = +0 for a row whose products are all -0)."""
    torch = cuda
    rng = np.random.default_rng(11)
    nS, nD = 5000, 3001
    counts = rng.integers(0, 6, nD)
    counts[rng.choice(nD, 40, replace=False)] = rng.integers(20, 41, 40)
    counts[:64] = 0  # two whole slices of empty rows
    recv = np.repeat(np.arange(1, nD + 1), counts).astype(np.int32)
    send = rng.integers(1, nS + 1, recv.size).astype(np.int32)
    coef = rng.uniform(-1, 1, recv.size)
    perm = rng.permutation(recv.size)  # table order is not row order
    recv, send, coef = recv[perm], send[perm], coef[perm]
    f = rng.standard_normal((nS, 7)) * 10.0
    f[rng.choice(nS, 500, replace=False), :] = -0.0
    coef[rng.choice(coef.size, 50, replace=False)] = 0.0
    plan = dccm.RemapPlan(nS, nD, send, recv, coef)
    ref = oracle.remap_apply(send, recv, coef, np.asfortranarray(f), nD)
    saved = {k: dccm.tune_get(k) for k in ("remap_fc", "remap_threads")}
    try:
        dccm.tune_set("remap_fc", fc)
        dccm.tune_set("remap_threads", threads)
        src = torch.from_numpy(np.ascontiguousarray(f.T)).cuda()
        dst = torch.full((7, nD), np.nan, dtype=torch.float64, device="cuda")
        plan.apply_dev(src, nS, dst, nD, 7)
        torch.cuda.synchronize()
        got = dst.cpu().numpy().T
        assert np.array_equal(got.view(np.int64), np.ascontiguousarray(ref).view(np.int64))
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)
