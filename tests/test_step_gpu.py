"""GPU tests of the ensemble transforms and the coupling-step graph, against
the oracle, through the C ABI.  Tolerances as in test_sht_gpu.py (mixed
1e-6, FP64 1e-13 relative L2); remap bit-exact; flux 1e-13."""
import importlib

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GROUPS = [(21, 64, 32, 20), (42, 128, 64, 10), (63, 192, 96, 7), (85, 256, 128, 5)]


@pytest.mark.parametrize("prec,tol", [(1, 1e-6), (2, 1e-6), (0, 1e-13)])
def test_ensemble_matches_oracle(dccm, oracle, synth, cuda, prec, tol):
    torch = cuda
    ens = dccm.Ensemble([g for g in GROUPS], prec)
    specs = [synth.spectra(N, B, seed=N + B) for N, I, J, B in GROUPS]
    ds = [torch.from_numpy(s.view(np.float64).copy()).cuda() for s in specs]
    dg = [torch.empty((B, J, I), dtype=torch.float64, device="cuda") for N, I, J, B in GROUPS]
    ds2 = [torch.empty_like(x) for x in ds]
    batch = [B for *_, B in GROUPS]
    ens.inverse_dev(ds, dg, batch)
    ens.forward_dev(dg, ds2, batch)
    torch.cuda.synchronize()
    assert ens.status() == (0, 0)
    for (N, I, J, B), s, g, s2 in zip(GROUPS, specs, dg, ds2):
        go = oracle.sht_inverse(N, I, J, s)
        assert rel_l2(g.cpu().numpy(), go) <= tol, N
        assert rel_l2(s2.cpu().numpy().view(np.complex128), s) <= tol, N
    # a group with no field-levels this call is skipped
    ens.inverse_dev(ds, dg, [0, 10, 0, 5])
    torch.cuda.synchronize()
    assert rel_l2(dg[1].cpu().numpy(), oracle.sht_inverse(42, 128, 64, specs[1])) <= tol


def _small_step(dccm, synth, oracle, torch, prec):
    """T21L16 x 3 -> T42 ocean (conservative weights), 8192 flux columns."""
    bench = importlib.import_module("bench")
    w = dict(bench.WORKLOADS["c1"])
    inp = bench.build_inputs(w, synth)
    S = bench.gpu_setup(w, inp, dccm, synth, torch, torch.device("cuda", 0))
    return bench, w, inp, S


def test_step_outputs_match_oracle(dccm, oracle, synth, cuda):
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    g = inp["groups"][0]
    for key, tol in (("mixed", 1e-6), ("fp16", 1e-6), ("fp64", 1e-13)):
        S["steps"][key].run()
        torch.cuda.synchronize()
        go = oracle.sht_inverse(g.N, g.I, g.J, g.spec)
        assert rel_l2(S["grid"][0].cpu().numpy(), go) <= tol, key
        assert rel_l2(S["spec_out"][0].cpu().numpy().view(np.complex128), g.spec) <= tol, key
    # remapped inputs and fluxes on the ocean columns
    send, recv, coef = S["tables"][0]
    n1 = len(inp["ocean"])
    ref = oracle.remap_apply(send, recv, coef, np.asfortranarray(g.src.T), n1)
    arrs, grid = bench.ocean_columns(inp)
    arrs.update(synth.flux_outputs(grid[0], grid[1], fill=0.0))
    for f, name in enumerate(bench.REMAP_FIELDS):
        got = S["dflux"][name].cpu().numpy().T[1:-1, 1]
        assert np.array_equal(got, ref[:, f]), name
        arrs[name][1:-1, 1] = ref[:, f]
    oracle.sfc_bulk_flux(arrs, *grid)
    for name in dccm.FLUX_OUT:
        got = S["dflux"][name].cpu().numpy().T
        assert rel_l2(got[1:-1, 1], arrs[name][1:-1, 1]) <= 1e-13, name


def test_step_timed_and_host_entry(dccm, oracle, synth, cuda):
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    ms = S["steps"]["mixed"].run_timed()
    assert len(ms) == 6 and all(m > 0 for m in ms)
    g = inp["groups"][0]
    h_in = torch.from_numpy(g.spec.view(np.float64).copy()).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    S["spec_out"][0].zero_()
    S["steps"]["mixed"].run_host([(h_in, S["spec_in"][0])], [(h_out, S["spec_out"][0])])
    assert rel_l2(h_out.numpy().view(np.complex128), g.spec) <= 1e-6


@pytest.mark.parametrize("pinned", [True, False])
def test_host_copies_match_device_run(dccm, oracle, synth, cuda, pinned):
    """run_host (copies recorded into the graph beside their stages when the
    host buffers are page-locked; copy-in/graph/copy-out otherwise) returns
    exactly what the device-side run produces, including a read-back of
    uploaded memory (ordered after the whole step) and the inverse grid."""
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    groups = inp["groups"]
    step = S["steps"]["mixed"]
    h2d, d2h = bench.host_copies(S, groups, dccm, torch)
    d2h.append((torch.empty(S["grid"][0].shape, dtype=torch.float64).pin_memory(), S["grid"][0]))
    d2h.append((torch.empty(S["spec_in"][0].shape, dtype=torch.float64).pin_memory(), S["spec_in"][0]))
    if not pinned:
        h2d = [(h.clone(), d) for h, d in h2d]
        d2h = [(torch.empty(h.shape, dtype=h.dtype), d) for h, d in d2h]
        assert not h2d[0][0].is_pinned()
    for h, d in h2d:
        d.copy_(h)
    step.run()
    torch.cuda.synchronize()
    want = [d.cpu().clone() for _, d in d2h]
    for _, d in d2h:
        if d.data_ptr() != S["spec_in"][0].data_ptr():
            d.zero_()
    for h, d in h2d:
        d.zero_()
    torch.cuda.synchronize()
    for _ in range(2):  # the second call replays the cached host graph
        for h, _ in d2h:
            h.zero_()
        step.run_host(h2d, d2h)
        for (h, _), ref in zip(d2h, want):
            assert torch.equal(h, ref)
    # both upload orders and both copy paths, copy lists prepared once,
    # then the per-step choice of the host autotuner
    saved = {k: dccm.tune_get(k) for k in ("upload_order", "host_path")}
    hc = dccm.HostCopies(h2d, d2h)
    assert hc.nbytes()[0] == sum(h.numel() * 8 for h, _ in h2d)

    def check(tag):
        for _ in range(2):
            for h, _ in d2h:
                h.zero_()
            for _, d in h2d + d2h:
                d.zero_()
            torch.cuda.synchronize()
            step.run_host(hc)
            for (h, _), ref in zip(d2h, want):
                assert torch.equal(h, ref), tag
            # the device arrays as the copies leave them (also when the flux
            # kernel reads and writes the host rows itself, path bit 4)
            for (_, d), ref in zip(d2h, want):
                assert torch.equal(d.cpu(), ref), tag
            for h, d in h2d:
                assert torch.equal(d.cpu(), h), tag
    try:
        for order in (1, 2, 0):
            for path in (1, 16, 1 + 2, 1 + 4 + 8, 1 + 16, 32):
                dccm.tune_set("upload_order", order)
                dccm.tune_set("host_path", path)
                step.host_release()
                check((order, path))
        choice = step.autotune_host(hc)
        ms = choice.pop("candidates_ms")
        if pinned:
            assert choice["upload_order"] in (1, 2) and 1 <= choice["host_path"] <= 32 and len(ms) == 32
            base = (choice["host_path"] - 1) % 16 + 1  # without bit 4: the best of the 32
            assert min(ms.values()) in (ms["1,%d" % base], ms["2,%d" % base]) and min(ms.values()) > 0
            if choice["host_path"] <= 16:
                assert min(ms.values()) == ms["%d,%d" % (choice["upload_order"], choice["host_path"])]
            assert choice["flux_ctas"] in (0, dccm.tune_get("flux_ctas"))
        else:
            assert choice == {"upload_order": 0, "host_path": 0, "flux_ctas": 0} and set(ms.values()) == {0.0}
        check(choice)
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)


def test_remap_two_level_destination(dccm, oracle, synth, cuda):
    """nsub/ld_dst2: member m's field f lands at dst + f*ld_dst + m*ld_dst2."""
    torch = cuda
    bench = importlib.import_module("bench")
    w = dict(bench.WORKLOADS["c4"])
    w["members"] = 6
    inp = bench.build_inputs(w, synth)
    S = bench.gpu_setup(w, inp, dccm, synth, torch, torch.device("cuda", 0))
    S["steps"]["mixed"].run()
    torch.cuda.synchronize()
    n1 = len(inp["ocean"])
    off = 0
    for g, (send, recv, coef) in zip(inp["groups"], S["tables"]):
        for mi in range(len(g.members)):
            ref = oracle.remap_apply(send, recv, coef, np.asfortranarray(g.src[6 * mi:6 * mi + 6].T), n1)
            for f, name in enumerate(bench.REMAP_FIELDS):
                got = S["dflux"][name].cpu().numpy().T[1 + off * n1:1 + (off + 1) * n1, 1]
                assert np.array_equal(got, ref[:, f]), (g.N, mi, name)
            off += 1


def test_autotune_keeps_results_and_caches(dccm, oracle, synth, cuda, tmp_path):
    """Every launch shape the autotuner can pick (Legendre CTA count, FFT
    CTA size and row pairs per warp, flux and remap CTA sizes, plain or
    programmatic dependent launches, either branch at the greatest
    priority) computes each output element the same way, so the step's
    outputs are bit-identical before and after tuning; the cache file
    returns the same choice on a second call."""
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    step = S["steps"]["mixed"]
    outs = [S["grid"][0], S["spec_out"][0]] + [S["dflux"][n] for n in dccm.FLUX_OUT]

    def run():
        for o in outs:
            o.zero_()
        step.run()
        torch.cuda.synchronize()
        return [o.cpu().clone() for o in outs]

    extra = ["serial", "flux_ctas", "remap_fc", "tc_shape", "fft_rpw", "prio"]
    saved = {k: dccm.tune_get(k) for k in dccm.Step.KNOBS + extra}
    try:
        want = run()
        cache = str(tmp_path / "tune.jsonl")
        first = step.autotune(cache)
        assert set(first) == set(dccm.Step.KNOBS + extra)
        assert first["serial"] in (0, 1)
        assert all(torch.equal(a, b) for a, b in zip(run(), want))
        line = open(cache).read()
        assert '"serial": ' in line and '"flux_ctas": ' in line and '"step_ms": ' in line
        assert step.autotune(cache) == first
        # a step recorded in either launch mode, or with the flux grid capped
        # at a few CTAs (each walks many columns), gives the same bits
        for knob, v in (("serial", 0), ("serial", 1), ("flux_ctas", 3), ("remap_fc", 1), ("remap_fc", 6),
                        ("remap_fc", 4), ("remap_threads", 32), ("tc_shape", 1), ("tc_shape", 0),
                        ("tc_ctas", 7), ("fft_rpw", 2), ("fft_bb", 4), ("fft_bb", 16), ("fft_rpw", 1),
                        ("prio", 1), ("prio", 2), ("prio", 0)):
            dccm.tune_set(knob, v)
            S = bench.gpu_setup(w, inp, dccm, synth, torch, torch.device("cuda", 0))
            step = S["steps"]["mixed"]
            outs = [S["grid"][0], S["spec_out"][0]] + [S["dflux"][n] for n in dccm.FLUX_OUT]
            assert all(torch.equal(a, b) for a, b in zip(run(), want)), (knob, v)
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)


def test_fp64_peak_probe(dccm, cuda):
    """The measured FP64 FMA rate is that of the CUDA cores: well below the
    FP32 rate, near the nominal 2 DFMA lanes per SM and clock."""
    import bench
    t = dccm.fp64_peak()
    assert 0.25 * bench.FP64_NOMINAL_TFLOPS < t < 1.5 * bench.FP64_NOMINAL_TFLOPS, t


def test_coupled_step_matches_pieces(dccm, oracle, synth, cuda):
    """The step with the implicit coupling around the flux (forward sweep,
    remaps including ImplCplCoef1/2, flux, DelVarImplCPL back onto level 1
    of the tendencies, backward sweep) gives bit for bit what the same
    calls give one by one."""
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    C = bench.coupled_setup(S, w, inp, dccm, synth, torch, torch.device("cuda", 0))
    df, out = S["dflux"], C["out"]
    names = list(dccm.FLUX_OUT) + ["ImplCplCoef1", "ImplCplCoef2"]
    C["step"].run()
    torch.cuda.synchronize()
    want = {k: v.clone() for k, v in out.items()}
    want_f = {n: df[n].clone() for n in names}
    want_s = S["spec_out"][0].clone()
    assert float(df["DelVarImplCPL"].abs().max()) > 0 and bool(torch.isfinite(want["DTempDt"][1:]).all())
    # one by one
    for v in out.values():
        v.zero_()
    for n in names:
        df[n].zero_()
    torch.cuda.synchronize()
    C["plan"].forward_dev(C["prof"], out)
    for plan, nf, src, lds, dst, ldd in C["coef"]:
        plan.apply_dev(src, lds, dst, ldd, nf)
    S["steps"]["mixed"].run()
    for plan, nf, src, lds, dst, ldd in C["post"]:
        plan.apply_dev(src, lds, dst, ldd, nf)
    C["plan"].backward_dev(out)
    torch.cuda.synchronize()
    for k in out:
        assert torch.equal(out[k], want[k]), k
    for n in names:
        assert torch.equal(df[n], want_f[n]), n
    assert torch.equal(S["spec_out"][0], want_s)
    # through run_host: the atmosphere's profiles in and the tendencies and
    # coefficients out go with the surface branch (page-locked buffers)
    step = C["step"]
    h2d = [(v.cpu().pin_memory(), v) for v in C["prof"].values()]
    d2h = [(torch.empty(v.shape, dtype=v.dtype).pin_memory(), v) for v in out.values()]
    for v in out.values():
        v.zero_()
    for _, d in h2d:
        d.zero_()
    torch.cuda.synchronize()
    for order in (1, 2):
        dccm.tune_set("upload_order", order)
        try:
            step.host_release()
            step.run_host(h2d, d2h)
        finally:
            dccm.tune_set("upload_order", 0)
        for (h, _), k in zip(d2h, out):
            assert torch.equal(h, want[k].cpu()), (order, k)


@pytest.mark.parametrize("rpw", [1, 2])
def test_ensemble_mixed_row_lengths_match_oracle(dccm, oracle, synth, cuda, rpw):
    """One FFT launch over groups of one-warp and several-warp rows (T42:
    I = 128, T170: I = 512 over two warps, T255: I = 768 over three, T85:
    I = 256): the launch's CTA size is the largest any group needs, the
    other groups' extra warps idle, each group's exchange buffers are sized
    for the launch's warp groups; with two row pairs a warp (group) or one.
    Mixed path against the oracle at the long-row tolerance."""
    torch = cuda
    groups = [(42, 128, 64, 5), (170, 512, 256, 3), (255, 768, 384, 2), (85, 256, 128, 7)]
    saved = dccm.tune_get("fft_rpw")
    try:
        dccm.tune_set("fft_rpw", rpw)
        ens = dccm.Ensemble(groups, 1)
        specs = [synth.spectra(N, B, seed=N + 7) for N, I, J, B in groups]
        ds = [torch.from_numpy(s.view(np.float64).copy()).cuda() for s in specs]
        dg = [torch.empty((B, J, I), dtype=torch.float64, device="cuda") for N, I, J, B in groups]
        ds2 = [torch.empty_like(x) for x in ds]
        batch = [B for *_, B in groups]
        ens.inverse_dev(ds, dg, batch)
        ens.forward_dev(dg, ds2, batch)
        torch.cuda.synchronize()
        assert ens.status() == (0, 0)
        for (N, I, J, B), s, g, s2 in zip(groups, specs, dg, ds2):
            go = oracle.sht_inverse(N, I, J, s)
            assert rel_l2(g.cpu().numpy(), go) <= 2e-6, N
            assert rel_l2(s2.cpu().numpy().view(np.complex128), s) <= 2e-6, N
    finally:
        dccm.tune_set("fft_rpw", saved)


def test_launch_host_two_instances_in_flight(dccm, oracle, synth, cuda):
    """dccm_step_launch_host: two independent instances of the c1 step (own
    device buffers and transform plans, shared remap plans), their steps
    issued in turn on two streams without synchronising, return exactly
    what dccm_step_run_host returns; pageable buffers are refused."""
    torch = cuda
    bench, w, inp, S = _small_step(dccm, synth, oracle, torch, 1)
    groups = inp["groups"]
    dev = torch.device("cuda", 0)
    S2 = bench.gpu_setup(w, inp, dccm, synth, torch, dev, keys=("mixed",), reuse=S)
    steps = [S["steps"]["mixed"], S2["steps"]["mixed"]]
    hcs = [dccm.HostCopies(*bench.host_copies(X, groups, dccm, torch)) for X in (S, S2)]
    steps[0].run_host(hcs[0])
    want = [h.clone() for h, _ in hcs[0].pairs[1]]
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    # the process-wide choices, the copy engines alone, everything mapped
    for choice in ((0, 0, -1), (1, 1, -1), (2, 16, 0)):
        for st in steps:
            st.host_choice(*choice)
        for hc in hcs:
            for h, _ in hc.pairs[1]:
                h.zero_()
        for k in range(6):
            steps[k % 2].launch_host(hcs[k % 2], stream=streams[k % 2])
        torch.cuda.synchronize()
        for hc in hcs:
            for (h, _), ref in zip(hc.pairs[1], want):
                assert torch.equal(h, ref), choice
    assert S["plans"]["mixed"].status() == (0, 0) and S2["plans"]["mixed"].status() == (0, 0)
    for bad in ((3, 1, -1), (1, 33, -1), (1, 1, -2)):
        with pytest.raises(dccm.DccmError):
            steps[0].host_choice(*bad)
    # pageable host buffers cannot be left in flight
    h_in = torch.from_numpy(groups[0].spec.view(np.float64).copy())
    with pytest.raises(dccm.DccmError):
        steps[1].launch_host([(h_in, S2["spec_in"][0])], [])
