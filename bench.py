"""Coupling-step benchmark: field-levels/s per coupling step on GB300.

Workload (default c3, the headline): T85L32 x 4 fields = 128 field-levels,
256x128 Gaussian grid; inverse + forward spherical-harmonic transforms of all
field-levels, remap of 6 surface fields to a 1-degree 360x180 ocean grid with
a seeded 30 % land mask (conservative Jones-99 weights), bulk flux on the
ocean columns.  One step = one CUDA graph replay.  Inputs are synthetic
(seeded; the reference publishes no data).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1|c2|c3|c5]
                  [--impl ours|reference]

--impl reference times the CPU FP64 implementation of the same step on all
host cores (the oracle restatement: the reference is Fortran and does not
build here), on a bounded sample of field-levels per step.
"""
import argparse
import ctypes
import importlib
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (N, I, J, levels, fields, ocean kind, ocean nx, ocean ny, land fraction, weight mode)
    "c1": dict(N=21, I=64, J=32, lev=16, fld=3, ocean="gauss", onx=128, ony=64, land=0.0, mode=0),
    "c2": dict(N=42, I=128, J=64, lev=26, fld=4, ocean="gauss", onx=128, ony=64, land=0.0, mode=0),
    "c3": dict(N=85, I=256, J=128, lev=32, fld=4, ocean="regular", onx=360, ony=180, land=0.3, mode=1),
    "c5": dict(N=341, I=1024, J=512, lev=48, fld=4, ocean="regular", onx=1440, ony=720, land=0.0, mode=1),
}
NAMES = {"c1": "T21L16 -> T42 ocean", "c2": "T42L26 -> T42 ocean", "c3": "T85L32 -> 1deg, 30% land",
         "c5": "T341L48 -> 0.25deg"}
REMAP_FIELDS = ["WindU", "WindV", "SfcAirTemp", "SfcPress", "QVap1", "LDwRFlx"]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# ----------------------------------------------------------------- inputs
def build_inputs(w, synth, dccm=None):
    """Host-side synthetic inputs and the remap table of a workload."""
    N, I, J = w["N"], w["I"], w["J"]
    nfl = w["lev"] * w["fld"]
    spec = synth.spectra(N, nfl, seed=0)
    lonA, latA, lwA, wA = synth.gaussian_axes(I, J)
    if w["ocean"] == "gauss":
        lonO, latO, lwO, wO = synth.gaussian_axes(w["onx"], w["ony"])
    else:
        lonO, latO, lwO, wO = synth.regular_axes(w["onx"], w["ony"])
    nxo, nyo = w["onx"], w["ony"]
    mask = synth.land_mask(nxo, nyo, w["land"], seed=0) if w["land"] > 0 else np.ones(nxo * nyo, np.uint8)
    ocean = np.flatnonzero(mask)
    # surface fields on the atmosphere grid (lon fastest)
    satm, _ = synth.surface_state(latA, I, seed=1)
    src = np.stack([satm[n][1:-1, 1:-1].ravel(order="F") for n in REMAP_FIELDS])
    # ocean-side flux inputs on the full ocean grid, then the ocean columns
    socn, _ = synth.surface_state(latO, nxo, seed=2)
    return dict(nfl=nfl, spec=spec, A=(lonA, latA, lwA, wA), O=(lonO, latO, lwO, wO), mask=mask,
                ocean=ocean, src=src, socn=socn)


def ocean_columns(inp):
    """Flux arrays on the ocean-column list: Fortran (IA, JA[, k]) with
    IA = n_ocean + 2, JA = 3 (halo 1), interior row j = 2."""
    ocean = inp["ocean"]
    n = len(ocean)
    IA, JA = n + 2, 3
    out = {}
    for name, a in inp["socn"].items():
        if name == "a_Sig1Info":
            out[name] = a.copy()
            continue
        inner = a[1:-1, 1:-1]  # (nx, ny) Fortran
        if inner.ndim == 2:
            v = inner.ravel(order="F")[ocean]
            arr = np.zeros((IA, JA), order="F")
            arr[1:-1, 1] = v
        else:
            k = inner.shape[2]
            arr = np.zeros((IA, JA, k), order="F")
            for q in range(k):
                arr[1:-1, 1, q] = inner[:, :, q].ravel(order="F")[ocean]
        out[name] = arr
    return out, (IA, JA, 2, IA - 1, 2, 2)


def remap_table(w, inp, dccm):
    A, O = inp["A"], inp["O"]
    t = dccm.gen_gridmapfile_lonlat2lonlat(A[0], A[1], O[0], O[1], A[2], A[3], O[2], O[3],
                                           accuracy_order=1, weight_mode=w["mode"],
                                           dst_mask=inp["mask"] if w["land"] > 0 else None)
    send, recv_full, coef = t.index(w["I"], w["onx"])
    rank = np.full(w["onx"] * w["ony"], -1, np.int64)
    rank[inp["ocean"]] = np.arange(len(inp["ocean"]))
    recv = (rank[recv_full - 1] + 1).astype(np.int32)
    assert recv.min() >= 1
    return send, recv, coef


# --------------------------------------------------------------- clocks
class Clocks:
    def __init__(self):
        self.p = None
        self.rows = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self, dev=0):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(dev):
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# -------------------------------------------------------------- CPU step
def cpu_step(oracle, w, inp, plan_cpu, nsample):
    """One step on the host with the oracle: transforms of nsample
    field-levels, the remap of the 6 surface fields, the bulk flux.
    Returns (seconds for transforms of nsample, seconds for remap+flux)."""
    N, I, J = w["N"], w["I"], w["J"]
    t0 = time.perf_counter()
    g = oracle.sht_inverse(N, I, J, inp["spec"][:nsample])
    oracle.sht_forward(N, I, J, g)
    t1 = time.perf_counter()
    send, recv, coef, arrs, grid = plan_cpu
    out = oracle.remap_apply(send, recv, coef, np.asfortranarray(inp["src"].T), len(inp["ocean"]))
    for k, name in enumerate(REMAP_FIELDS):
        arrs[name][1:-1, 1] = out[:, k]
    oracle.sfc_bulk_flux(arrs, *grid)
    t2 = time.perf_counter()
    return t1 - t0, t2 - t1


def cpu_measure(oracle, synth, dccm_like, w, inp, steps, warmup, budget_s=20.0):
    send, recv, coef = dccm_like
    arrs, grid = ocean_columns(inp)
    arrs.update(synth.flux_outputs(grid[0], grid[1], fill=0.0))
    plan_cpu = (send, recv, coef, arrs, grid)
    nfl = inp["nfl"]
    nsample = max(1, min(nfl, 8))
    t_sht, t_rf = cpu_step(oracle, w, inp, plan_cpu, nsample)  # warm and size the sample
    per_fl = t_sht / nsample
    nsample = int(max(1, min(nfl, (budget_s / max(1, steps) - t_rf) / max(per_fl, 1e-9))))
    for _ in range(warmup):
        cpu_step(oracle, w, inp, plan_cpu, nsample)
    ts = []
    for _ in range(steps):
        a, b = cpu_step(oracle, w, inp, plan_cpu, nsample)
        ts.append(a * nfl / nsample + b)
    step_s = float(np.mean(ts))
    return step_s, nsample


# ------------------------------------------------------------------ GPU
def gpu_bench(args, w, rank, world):
    import torch
    dccm = importlib.import_module("dennou-ccm_gb300")
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    dccm.load()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    inp = build_inputs(w, synth)
    N, I, J, nfl = w["N"], w["I"], w["J"], inp["nfl"]
    ncoef = (N + 1) * (N + 2) // 2
    send, recv, coef = remap_table(w, inp, dccm)
    n_ocean = len(inp["ocean"])
    remap = dccm.RemapPlan(I * J, n_ocean, send, recv, coef)
    arrs, fgrid = ocean_columns(inp)
    arrs.update(synth.flux_outputs(fgrid[0], fgrid[1], fill=0.0))
    IA, JA = fgrid[0], fgrid[1]

    def to_dev(a):  # Fortran (IA, JA[, k]) -> contiguous device tensor of the same memory order
        return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)

    # device buffers
    spec_in = torch.from_numpy(inp["spec"].view(np.float64).copy()).to(dev)
    grid = torch.empty((nfl, J, I), dtype=torch.float64, device=dev)
    spec_out = torch.empty_like(spec_in)
    src = torch.from_numpy(np.ascontiguousarray(inp["src"])).to(dev)
    remapped = torch.zeros((6, JA, IA), dtype=torch.float64, device=dev)  # the six remapped inputs
    dflux = {}
    for name in dccm.FLUX_ARGS:
        if name == "a_Sig1Info":
            dflux[name] = arrs[name]
        elif name in REMAP_FIELDS:
            dflux[name] = remapped[REMAP_FIELDS.index(name)]
        else:
            dflux[name] = to_dev(arrs[name])
    # remap writes straight into the interior row (i = 2.., j = 2) of each input
    dst_view = remapped.view(6, -1)[:, IA + 1:]

    plans = {"mixed": dccm.ShtPlan(N, I, J, dccm.SHT_MIXED, nfl), "fp64": dccm.ShtPlan(N, I, J, dccm.SHT_FP64, nfl)}
    steps = {}
    for k, sp in plans.items():
        steps[k] = dccm.Step(sht=sp, nfl=nfl, spec_in=spec_in, grid=grid, spec_out=spec_out, remap=remap,
                             nfields=6, remap_src=src, ld_src=I * J, remap_dst=dst_view, ld_dst=IA * JA,
                             flux=dflux, flux_grid=fgrid)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(int(256 * 2 ** 20 // 4), dtype=torch.float32, device=dev)  # 256 MB > L2

    def timed(step, K, W):
        for _ in range(W):
            step.run(stream)
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(K):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            step.run(stream)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        wall = time.perf_counter() - t0
        return [a.elapsed_time(b) for a, b in evs], wall

    clocks = Clocks()
    clocks.start()
    ms_mixed, wall = timed(steps["mixed"], args.steps, max(3, args.warmup))
    ck = clocks.stop(dev.index or 0)
    ms_fp64, _ = timed(steps["fp64"], args.steps, max(3, args.warmup))
    t_mixed = float(np.mean(ms_mixed)) / 1e3
    t_fp64 = float(np.mean(ms_fp64)) / 1e3
    if world > 1:
        tt = torch.tensor([t_mixed, t_fp64], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_mixed, t_fp64 = (float(x) for x in tt.cpu())

    # accuracy of the timed mixed step against the FP64 step (same inputs)
    steps["fp64"].run(stream)
    torch.cuda.synchronize()
    ref_spec = spec_out.clone()
    ref_grid = grid.clone()
    steps["mixed"].run(stream)
    torch.cuda.synchronize()
    err_spec = float(torch.linalg.norm(spec_out - ref_spec) / torch.linalg.norm(ref_spec))
    err_grid = float(torch.linalg.norm(grid - ref_grid) / torch.linalg.norm(ref_grid))
    err_rt = float(torch.linalg.norm(spec_out - spec_in) / torch.linalg.norm(spec_in))
    st, derr = plans["mixed"].status()
    assert st == 0 and derr == 0, ("device error", st, derr)

    # per-stage device times (stages launched back to back with events)
    stage_ms = np.zeros(4)
    nt = max(3, min(10, args.steps))
    for k in range(nt):
        flush.fill_(float(k))
        stage_ms += np.array(steps["mixed"].run_timed(stream))
    stage_ms /= nt
    hbm, bf16, src_peak = peaks()
    Jh = J // 2
    legendre_flops = 2.0 * J * ncoef * nfl  # per direction, algorithmic
    fft_bytes = nfl * J * I * 8 + nfl * J * (N + 1) * 2 * 4
    nnz = len(coef)
    remap_bytes = 12 * nnz + 4 * (n_ocean + 1) + 8 * 6 * (I * J + n_ocean)
    flux_bytes = 504 * n_ocean
    names = ["sht_inverse", "sht_forward", "remap", "bulk_flux"]
    dom = int(np.argmax(stage_ms))
    roof = {}
    if dom in (0, 1):
        # A transform stage is a Legendre GEMM (tensor) + an FFT (HBM); report
        # the stage as HBM-bound on its dominant memory traffic.
        bytes_ = fft_bytes + nfl * ncoef * 16
        ach = bytes_ / (stage_ms[dom] / 1e3) / 1e9
        roof = {"kernel": names[dom], "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": None, "peak_source": src_peak,
                "algorithmic_bytes": bytes_, "ms": float(stage_ms[dom])}
    else:
        bytes_ = remap_bytes if dom == 2 else flux_bytes
        ach = bytes_ / (stage_ms[dom] / 1e3) / 1e9
        roof = {"kernel": names[dom], "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": None, "peak_source": src_peak,
                "algorithmic_bytes": bytes_, "ms": float(stage_ms[dom])}
    roof["stages_ms"] = {n: float(v) for n, v in zip(names, stage_ms)}
    roof["legendre_tflops_algorithmic"] = legendre_flops / 1e12

    # end to end through the public API with host buffers (pinned)
    h_spec_in = torch.from_numpy(inp["spec"].view(np.float64).copy()).pin_memory()
    h_src = torch.from_numpy(np.ascontiguousarray(inp["src"])).pin_memory()
    h_spec_out = torch.empty_like(h_spec_in).pin_memory()
    out_names = dccm.FLUX_OUT
    h_out = {n: torch.empty_like(dflux[n], device="cpu").pin_memory() for n in out_names}
    h2d = [(h_spec_in, spec_in), (h_src, src)]
    d2h = [(h_spec_out, spec_out)] + [(h_out[n], dflux[n]) for n in out_names]
    h2d_bytes = sum(h.numel() * h.element_size() for h, _ in h2d)
    d2h_bytes = sum(h.numel() * h.element_size() for h, _ in d2h)
    for _ in range(max(3, args.warmup)):
        steps["mixed"].run_host(h2d, d2h, stream)
    if world > 1:
        torch.distributed.barrier()
    te = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        steps["mixed"].run_host(h2d, d2h, stream)
        te.append(time.perf_counter() - t0)
    t_e2e = float(np.mean(te))
    if world > 1:
        tt = torch.tensor([t_e2e], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.cpu()[0])

    res = dict(t_mixed=t_mixed, t_fp64=t_fp64, t_e2e=t_e2e, wall=wall, clocks=ck, roof=roof,
               err=dict(spec_vs_fp64=err_spec, grid_vs_fp64=err_grid, round_trip=err_rt),
               h2d=h2d_bytes, d2h=d2h_bytes, nfl=nfl, nnz=nnz, n_ocean=n_ocean,
               launches=6 if True else 0, table=(send, recv, coef), inp=inp)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    w = WORKLOADS[args.workload]
    nfl = w["lev"] * w["fld"]
    config = {"workload": "%s (%s)" % (args.workload, NAMES[args.workload]), "truncation": w["N"],
              "grid": [w["I"], w["J"]], "field_levels_per_gpu": nfl, "ocean_grid": [w["onx"], w["ony"]],
              "land_fraction": w["land"], "remap_fields": 6, "l2": "flushed between timed steps (256 MB write)"}
    metric = "field-levels/s per coupling step"
    import oracle
    synth = importlib.import_module("dennou-ccm_gb300.synth")

    if args.impl == "reference":
        if rank != 0:
            return
        inp = build_inputs(w, synth)
        # the table is the same Jones-99 table, generated by the oracle
        A, O = inp["A"], inp["O"]
        iD, jD, iS, jS, wts = oracle.j99_gen(A[0], A[1], O[0], O[1], A[3], O[3], 1, w["mode"])
        keep = inp["mask"][(iD - 1) + w["onx"] * (jD - 1)] == 1
        iD, jD, iS, jS, wts = iD[keep], jD[keep], iS[keep], jS[keep], wts[keep]
        send, recv_full = oracle.table_to_index(iD, jD, iS, jS, w["I"], w["onx"])
        rank_ = np.full(w["onx"] * w["ony"], -1, np.int64)
        rank_[inp["ocean"]] = np.arange(len(inp["ocean"]))
        recv = (rank_[recv_full - 1] + 1).astype(np.int32)
        t0 = time.perf_counter()
        step_s, nsample = cpu_measure(oracle, synth, (send, recv, wts), w, inp, args.steps, args.warmup)
        value = nfl / step_s
        cores = oracle.get_threads()
        line = {"impl": "reference", "metric": metric, "value": value, "unit": "field-levels/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": config,
                "cpu_baseline": {"value": value, "unit": "field-levels/s", "cores": cores, "kind": "port",
                                 "sample": "per step: transforms of %d of %d field-levels (scaled), full remap "
                                           "and bulk flux; C FP64 oracle, OpenMP" % (nsample, nfl)},
                "e2e": {"value": value, "unit": "field-levels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "wall_s": time.perf_counter() - t0}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    r = gpu_bench(args, w, rank, world)
    if rank != 0:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    value = world * r["nfl"] / r["t_mixed"]
    cpu = None
    if not args.no_cpu_baseline:
        send, recv, coef = r["table"]
        step_s, nsample = cpu_measure(oracle, synth, (send, recv, coef), w, r["inp"], 3, 1, budget_s=15.0)
        cpu = {"value": r["nfl"] / step_s, "unit": "field-levels/s", "cores": oracle.get_threads(), "kind": "port",
               "sample": "3 steps: transforms of %d of %d field-levels (scaled), full remap and bulk flux; "
                         "C FP64 oracle, OpenMP" % (nsample, r["nfl"])}
    line = {
        "metric": metric, "value": value, "unit": "field-levels/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": r["t_mixed"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3+f32 (Legendre), f32 (FFT), f64 (remap, flux)",
        "data": "synthetic (seeded PCG64; n^-3 spectra, SST-based surface state)", "config": config,
        "fp64_gpu": {"value": world * r["nfl"] / r["t_fp64"], "ms_per_step": r["t_fp64"] * 1e3,
                     "mixed_over_fp64": r["t_fp64"] / r["t_mixed"]},
        "accuracy": r["err"],
        "e2e": {"value": world * r["nfl"] / r["t_e2e"], "unit": "field-levels/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["t_e2e"] * 1e3},
        "gpu_launches": r["launches"] * args.steps,
        "roofline": r["roof"], "clocks": r["clocks"], "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
