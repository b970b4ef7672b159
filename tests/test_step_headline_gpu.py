"""Step-level parity at the benchmark's own workloads, through the step
graph and through dccm_step_run_host, against the oracle.

c3: T85L32 x 4 fields (128 field-levels) on the 256 x 128 Gaussian grid,
remapped with CONSERVE weights to the 1-degree ocean with the seeded 30 %
land mask (45,478 ocean columns), bulk flux on every ocean column.
c4: the 64-member ensemble (T21-T85, 16-32 levels) on the T42 ocean.

Tolerances (the same as the per-kernel tests):
  grids and spectra, mixed paths (BF16 x 3, FP16 hi + lo): relative L2
      <= 1e-6 over the batch and per field-level;
  grids and spectra, FP64 path: <= 1e-13;
  the six remapped fields: bit-exact against the oracle's COO loop
      (common/interpolation_data_latlon_mod.f90:293-302);
  flux outputs: relative L2 <= 1e-13 per output and slot against the oracle
      (sfc/DSFCM_Util_SfcBulkFlux_mod.f90:108-439);
  conservation of the CONSERVE table on the same grids: 1e-12 relative to
      the integral of |f| (and to the integral itself where the mean is
      not near zero).
"""
import importlib

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-6, "fp16": 1e-6, "fp64": 1e-13}


def _setup(key, dccm, synth, torch):
    bench = importlib.import_module("bench")
    w = dict(bench.WORKLOADS[key])
    inp = bench.build_inputs(w, synth)
    S = bench.gpu_setup(w, inp, dccm, synth, torch, torch.device("cuda", 0))
    return bench, w, inp, S


def _per_field(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if np.iscomplexobj(b):
        a, b = a.view(np.float64), b.view(np.float64)
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    return float(np.max(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)))


def _oracle_surface(bench, oracle, synth, inp, S):
    """Remapped fields (bit-exact reference) and flux outputs of the oracle,
    every member of every group, on the compact ocean-column arrays."""
    arrs, grid = bench.ocean_columns(inp)
    arrs.update(synth.flux_outputs(grid[0], grid[1], fill=0.0))
    n1 = len(inp["ocean"])
    off = 0
    for g, (send, recv, coef) in zip(inp["groups"], S["tables"]):
        for mi in range(len(g.members)):
            out = oracle.remap_apply(send, recv, coef, np.asfortranarray(g.src[6 * mi:6 * mi + 6].T), n1)
            for f, name in enumerate(bench.REMAP_FIELDS):
                arrs[name][1 + off * n1:1 + (off + 1) * n1, 1] = out[:, f]
            off += 1
    oracle.sfc_bulk_flux(arrs, *grid)
    return arrs


def _check_surface(bench, dccm, arrs, get):
    """get(name) -> the step's (IA, JA[, k]) Fortran-ordered result."""
    for name in bench.REMAP_FIELDS:
        assert np.array_equal(get(name)[1:-1, 1], arrs[name][1:-1, 1]), name
    for name in list(dccm.FLUX_OUT) + ["SfcTemp", "SfcAlbedo"]:
        got, ref = get(name), arrs[name]
        for q in range(ref.shape[2]):
            r = ref[1:-1, 1, q]
            if not np.any(r):
                assert not np.any(got[1:-1, 1, q]), (name, q)  # slots the routine leaves untouched
                continue
            assert rel_l2(got[1:-1, 1, q], r) <= 1e-13, (name, q)


def _check_transforms(oracle, inp, S, key, grids=None, specs=None):
    grids = grids if grids is not None else [x.cpu().numpy() for x in S["grid"]]
    specs = specs if specs is not None else [x.cpu().numpy().view(np.complex128) for x in S["spec_out"]]
    tol = TOL[key]
    for g, gr, sp in zip(inp["groups"], grids, specs):
        go = oracle.sht_inverse(g.N, g.I, g.J, g.spec)
        so = oracle.sht_forward(g.N, g.I, g.J, go)
        assert rel_l2(gr, go) <= tol and _per_field(gr, go) <= tol, (key, g.N, "grid")
        assert rel_l2(sp, so) <= tol and _per_field(sp, so) <= tol, (key, g.N, "spec")


@pytest.mark.parametrize("workload", ["c3", "c4"])
def test_step_graph_matches_oracle(dccm, oracle, synth, cuda, workload):
    """Every output of one step-graph replay, for each precision."""
    torch = cuda
    bench, w, inp, S = _setup(workload, dccm, synth, torch)
    arrs = _oracle_surface(bench, oracle, synth, inp, S)
    for key in ("mixed", "fp16", "fp64"):
        for x in S["grid"] + S["spec_out"]:
            x.zero_()
        for name in list(dccm.FLUX_OUT) + bench.REMAP_FIELDS:
            S["dflux"][name].zero_()
        S["steps"][key].run()
        torch.cuda.synchronize()
        assert S["plans"][key].status() == (0, 0), key
        _check_transforms(oracle, inp, S, key)
        _check_surface(bench, dccm, arrs, lambda n: S["dflux"][n].cpu().numpy().T)


def test_step_run_host_matches_oracle_c3(dccm, oracle, synth, cuda):
    """dccm_step_run_host with page-locked host buffers (the bench's e2e
    call: spectra and surface state in, spectra and fluxes out, plus the
    inverse grid), after the host autotuner has picked its copy paths: the
    host buffers hold the oracle's results."""
    torch = cuda
    bench, w, inp, S = _setup("c3", dccm, synth, torch)
    arrs = _oracle_surface(bench, oracle, synth, inp, S)
    step = S["steps"]["mixed"]
    h2d, d2h = bench.host_copies(S, inp["groups"], dccm, torch)
    d2h.append((torch.empty(S["grid"][0].shape, dtype=torch.float64).pin_memory(), S["grid"][0]))
    # the device state starts empty: everything the step needs comes from the host
    for _, d in h2d + d2h:
        d.zero_()
    torch.cuda.synchronize()
    hc = dccm.HostCopies(h2d, d2h)
    saved = {k: dccm.tune_get(k) for k in ("upload_order", "host_path", "flux_ctas")}
    try:
        step.autotune_host(hc)
        for _ in range(2):  # the second call replays the recorded host graph
            for h, _ in d2h:
                h.zero_()
            step.run_host(hc)
            # the flux results as the host sees them: views of the d2h block
            # in the order bench.host_copies lays them out
            k = len(S["spec_out"])
            host = {}
            for name in list(dccm.FLUX_OUT) + ["SfcTemp", "SfcAlbedo"]:
                ref = arrs[name]
                got = np.zeros_like(ref)
                for q in bench.FLUX_D2H_SLOTS.get(name, (0, 1, 2)):
                    got[1:-1, 1, q] = d2h[k][0].numpy()
                    k += 1
                host[name] = got
            for name in bench.REMAP_FIELDS:  # remapped fields are device-side inputs of the flux
                host[name] = S["dflux"][name].cpu().numpy().T
            for name in list(host):
                if name in dccm.FLUX_OUT or name in ("SfcTemp", "SfcAlbedo"):
                    ref = arrs[name]
                    for q in range(ref.shape[2]):
                        if q not in bench.FLUX_D2H_SLOTS.get(name, (0, 1, 2)):
                            host[name][1:-1, 1, q] = ref[1:-1, 1, q]  # not copied back
            _check_surface(bench, dccm, arrs, lambda n: host[n])
            _check_transforms(oracle, inp, S, "mixed", grids=[d2h[-1][0].numpy()],
                              specs=[d2h[0][0].numpy().view(np.complex128)])
    finally:
        for kk, v in saved.items():
            dccm.tune_set(kk, v)


def test_c3_conserve_table_conserves(dccm, oracle, synth, cuda):
    """The c3 grids' CONSERVE table: rows of the land-masked plan the step
    uses sum to 1 (a constant field stays constant on every ocean cell), and
    the same generator without the mask conserves the global area-weighted
    integral of each of the six surface fields to 1e-12."""
    torch = cuda
    bench, w, inp, S = _setup("c3", dccm, synth, torch)
    g = inp["groups"][0]
    n1 = len(inp["ocean"])
    ones = torch.ones((1, g.I * g.J), dtype=torch.float64, device="cuda")
    out = torch.zeros((1, n1), dtype=torch.float64, device="cuda")
    S["remap_plans"][0].apply_dev(ones, g.I * g.J, out, n1, 1)
    torch.cuda.synchronize()
    assert float((out - 1.0).abs().max()) <= 1e-13
    A, O = g.axes, inp["O"]
    t = dccm.gen_gridmapfile_lonlat2lonlat(A[0], A[1], O[0], O[1], A[2], A[3], O[2], O[3],
                                           accuracy_order=1, weight_mode=dccm.J99_CONSERVE)
    nS, nD = g.I * g.J, w["onx"] * w["ony"]
    send, recv, coef = t.index(g.I, w["onx"])
    plan = dccm.RemapPlan(nS, nD, send, recv, coef)
    src = S["src"][0]
    dst = torch.zeros((6, nD), dtype=torch.float64, device="cuda")
    plan.apply_dev(src, nS, dst, nD, 6)
    torch.cuda.synchronize()
    aS = torch.from_numpy(np.outer(A[3], A[2]).ravel()).cuda()
    aD = torch.from_numpy(np.outer(O[3], O[2]).ravel()).cuda()
    for k in range(6):
        i_s = dccm.area_integral_dev(src[k].contiguous(), aS)
        i_d = dccm.area_integral_dev(dst[k].contiguous(), aD)
        # relative to the integral of |f|: the wind components have means
        # near zero, where a ratio to the integral itself measures nothing
        scale = dccm.area_integral_dev(src[k].abs().contiguous(), aS)
        assert abs(i_d - i_s) <= 1e-12 * scale, (bench.REMAP_FIELDS[k], i_s, i_d, scale)
        if abs(i_s) > 0.1 * scale:
            assert abs(i_d - i_s) <= 1e-12 * abs(i_s), (bench.REMAP_FIELDS[k], i_s, i_d)
