"""Coupling-step benchmark: field-levels/s per coupling step on GB300.

Workloads (seeded synthetic data; the reference publishes none):
  c1  T21L16 x 3 fields (48 field-levels), 64x32 grid -> T42 128x64 ocean, no land
  c2  T42L26 x 4 fields (104), 128x64 -> T42 ocean (identity map)
  c3  T85L32 x 4 fields (128), 256x128 -> 1-degree 360x180 ocean, 30 % land  [headline]
  c4  64-member ensemble, truncations from {T21, T42, T63, T85}, 16-32 levels
      x 4 fields (~6,000 field-levels), every member -> T42 ocean
  c5  T341L48 x 4 fields (192), 1024x512 -> 0.25-degree 1440x720 ocean
One step = inverse + forward spherical-harmonic transforms of every
field-level, remap of 6 surface fields (WindU, WindV, SfcAirTemp, SfcPress,
QVap1, LDwRFlx) to the ocean columns, bulk flux on the ocean columns: one
CUDA-graph replay (dccm_step_run).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1..c5]
                  [--impl ours|reference] [--no-cpu-baseline]

--impl reference times the CPU FP64 implementation of the same step on all
host cores (the C oracle: the reference is Fortran and does not build here),
on a bounded sample of field-levels per step.
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GAUSS = {21: (64, 32), 42: (128, 64), 63: (192, 96), 85: (256, 128), 341: (1024, 512)}
WORKLOADS = {
    "c1": dict(N=21, lev=16, fld=3, ocean="gauss", onx=128, ony=64, land=0.0, mode=1),
    "c2": dict(N=42, lev=26, fld=4, ocean="gauss", onx=128, ony=64, land=0.0, mode=0),
    "c3": dict(N=85, lev=32, fld=4, ocean="regular", onx=360, ony=180, land=0.3, mode=1),
    "c4": dict(members=64, truncs=(21, 42, 63, 85), lev=(16, 32), fld=4, ocean="gauss", onx=128, ony=64,
               land=0.0, mode=1),
    "c5": dict(N=341, lev=48, fld=4, ocean="regular", onx=1440, ony=720, land=0.0, mode=1),
}
NAMES = {"c1": "T21L16 -> T42 ocean", "c2": "T42L26 -> T42 ocean", "c3": "T85L32 -> 1deg, 30% land",
         "c4": "64-member ensemble T21-T85 -> T42 ocean", "c5": "T341L48 -> 0.25deg"}
REMAP_FIELDS = ["WindU", "WindV", "SfcAirTemp", "SfcPress", "QVap1", "LDwRFlx"]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# ----------------------------------------------------------------- inputs
class Group:
    """Field-levels of one truncation: spectra, surface fields, remap table."""

    def __init__(self, N, members, levels, fld, synth, seeds):
        self.N = N
        self.I, self.J = GAUSS[N]
        self.members = members
        self.nfl = int(sum(levels) * fld)
        self.spec = np.concatenate([synth.spectra(N, lv * fld, seed=s) for lv, s in zip(levels, seeds)])
        self.axes = synth.gaussian_axes(self.I, self.J)
        src = []
        for s in seeds:
            st, _ = synth.surface_state(self.axes[1], self.I, seed=1000 + s)
            src += [st[n][1:-1, 1:-1].ravel(order="F") for n in REMAP_FIELDS]
        self.src = np.stack(src)  # [member][field] rows of I*J


def build_inputs(w, synth):
    if "members" in w:
        rng = np.random.Generator(np.random.PCG64(0))
        trunc = rng.choice(np.array(w["truncs"]), w["members"])
        lev = rng.integers(w["lev"][0], w["lev"][1] + 1, w["members"])
        groups = []
        for T in w["truncs"]:
            mem = [k for k in range(w["members"]) if trunc[k] == T]
            if mem:
                groups.append(Group(int(T), mem, [int(lev[k]) for k in mem], w["fld"], synth, mem))
    else:
        groups = [Group(w["N"], [0], [w["lev"]], w["fld"], synth, [0])]
    if w["ocean"] == "gauss":
        O = synth.gaussian_axes(w["onx"], w["ony"])
    else:
        O = synth.regular_axes(w["onx"], w["ony"])
    nxo, nyo = w["onx"], w["ony"]
    mask = synth.land_mask(nxo, nyo, w["land"], seed=0) if w["land"] > 0 else np.ones(nxo * nyo, np.uint8)
    ocean = np.flatnonzero(mask)
    socn, _ = synth.surface_state(O[1], nxo, seed=2)
    nmem = sum(len(g.members) for g in groups)
    return dict(groups=groups, O=O, mask=mask, ocean=ocean, socn=socn, nmem=nmem,
                nfl=sum(g.nfl for g in groups))


def ocean_columns(inp):
    """Flux arrays on the list of ocean columns of all members (members in
    group order): Fortran (IA, JA[, k]), IA = n_cols + 2, JA = 3, interior row 2."""
    ocean, nmem = inp["ocean"], inp["nmem"]
    n1 = len(ocean)
    n = n1 * nmem
    IA, JA = n + 2, 3
    out = {}
    for name, a in inp["socn"].items():
        if name == "a_Sig1Info":
            out[name] = a.copy()
            continue
        inner = a[1:-1, 1:-1]
        if inner.ndim == 2:
            arr = np.zeros((IA, JA), order="F")
            arr[1:-1, 1] = np.tile(inner.ravel(order="F")[ocean], nmem)
        else:
            arr = np.zeros((IA, JA, inner.shape[2]), order="F")
            for q in range(inner.shape[2]):
                arr[1:-1, 1, q] = np.tile(inner[:, :, q].ravel(order="F")[ocean], nmem)
        out[name] = arr
    return out, (IA, JA, 2, IA - 1, 2, 2)


def remap_index(w, inp, g, gen):
    """(send, recv, coef) of group g's table, recv over the ocean columns."""
    A, O = g.axes, inp["O"]
    iD, jD, iS, jS, wts = gen(A, O)
    keep = inp["mask"][(iD - 1) + w["onx"] * (jD - 1)] == 1
    iD, jD, iS, jS, wts = iD[keep], jD[keep], iS[keep], jS[keep], wts[keep]
    send = (iS + g.I * (jS - 1)).astype(np.int32)
    rank = np.full(w["onx"] * w["ony"], -1, np.int64)
    rank[inp["ocean"]] = np.arange(len(inp["ocean"]))
    recv = (rank[(iD + w["onx"] * (jD - 1)) - 1] + 1).astype(np.int32)
    assert recv.min() >= 1
    return send, recv, wts


# --------------------------------------------------------------- clocks
# NVML poller run as its own process (so that it takes no time from the
# launching thread): SM clock and clock-event reason bits every 0.1 ms until its
# standard input closes, then one JSON summary line.  argv[1]: the PCI bus id
# of the GPU in use, or "" when NVML sees one GPU.  Read-only NVML queries.
_NVML_POLL = r"""
import ctypes, json, select, sys
lib = ctypes.CDLL("libnvidia-ml.so.1")
assert lib.nvmlInit_v2() == 0
h = ctypes.c_void_p()
n = ctypes.c_uint()
lib.nvmlDeviceGetCount_v2(ctypes.byref(n))
if n.value == 1 or not sys.argv[1]:
    assert lib.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(h)) == 0
else:
    assert lib.nvmlDeviceGetHandleByPciBusId_v2(sys.argv[1].encode(), ctypes.byref(h)) == 0
get_rs = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or lib.nvmlDeviceGetCurrentClocksThrottleReasons
clk, cmax, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(cmax))
for _ in range(3):  # first calls of each query are slow: before the region
    lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))
    get_rs(h, ctypes.byref(rs))
sm, bits = [], 0
print("ready", flush=True)
while not select.select([sys.stdin], [], [], 0.0001)[0]:
    if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and get_rs(h, ctypes.byref(rs)) == 0:
        sm.append(clk.value)
        bits |= rs.value
sm.sort()
print(json.dumps({"n": len(sm), "median": sm[len(sm) // 2] if sm else None, "max": cmax.value, "bits": bits}), flush=True)
"""


class Clocks:
    """SM clock and clock-event reasons sampled from the warm-up through the
    end of the timed region: an NVML poller process (every 0.1 ms), or
    nvidia-smi -lms 20 where NVML cannot be loaded."""

    # NVML clocks event (throttle) reason bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, dev=0):
        self.p = None
        self.poll = None
        self.dev = dev

    def start(self):
        try:
            import torch
            bus = ""
            if torch.cuda.device_count() >= 1:
                pr = torch.cuda.get_device_properties(self.dev)
                bus = "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            self.poll = subprocess.Popen([sys.executable, "-c", _NVML_POLL, bus], stdin=subprocess.PIPE,
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            if self.poll.stdout.readline().strip() == "ready":
                return
            self.poll.wait(timeout=10)
        except Exception:
            pass
        self.poll = None
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # nvidia-smi up before the region starts
        except Exception:
            self.p = None

    def stop(self, dev=0):
        if self.poll is not None:
            try:
                out, _ = self.poll.communicate(input="", timeout=10)
                r = json.loads(out.strip().splitlines()[-1])
            except Exception as e:  # noqa: BLE001
                self.poll.kill()
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvml poller failed: %s" % e]}
            if not r["n"]:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "source": "nvml"}
            return {"sm_mhz": float(r["median"]), "sm_max_mhz": float(r["max"]),
                    "reasons": sorted(nm for bit, nm in self.REASONS.items() if r["bits"] & bit),
                    "samples": r["n"], "source": "nvml, 0.1 ms"}
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
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
                "samples": len(sm), "source": "nvidia-smi, 20 ms"}


# -------------------------------------------------------------- CPU step
def cpu_measure(oracle, synth, w, inp, tables, steps, warmup, budget_s=20.0):
    """The step on the host with the C oracle (all cores): transforms of a
    sample of each group's field-levels (scaled to the full count), every
    remap, the bulk flux.  Returns (seconds per step, sampled field-levels)."""
    arrs, grid = ocean_columns(inp)
    arrs.update(synth.flux_outputs(grid[0], grid[1], fill=0.0))
    n1 = len(inp["ocean"])
    groups = inp["groups"]

    def step(ns):
        t_sht = 0.0
        for g, k in zip(groups, ns):
            t0 = time.perf_counter()
            gr = oracle.sht_inverse(g.N, g.I, g.J, g.spec[:k])
            oracle.sht_forward(g.N, g.I, g.J, gr)
            t_sht += (time.perf_counter() - t0) * g.nfl / k
        t0 = time.perf_counter()
        off = 0
        for g, (send, recv, coef) in zip(groups, tables):
            for mi in range(len(g.members)):
                out = oracle.remap_apply(send, recv, coef, np.asfortranarray(g.src[6 * mi:6 * mi + 6].T), n1)
                for f, name in enumerate(REMAP_FIELDS):
                    arrs[name][1 + off * n1:1 + (off + 1) * n1, 1] = out[:, f]
                off += 1
        oracle.sfc_bulk_flux(arrs, *grid)
        return t_sht + (time.perf_counter() - t0)

    ns = [max(1, min(g.nfl, 8)) for g in groups]
    t = step(ns)  # warm, and size the sample to the time budget
    grow = budget_s / max(1, steps) / max(t, 1e-6)
    ns = [max(1, int(min(g.nfl, k * grow))) for g, k in zip(groups, ns)]
    for _ in range(warmup):
        step(ns)
    ts = [step(ns) for _ in range(steps)]
    return float(np.mean(ts)), sum(ns)


# ------------------------------------------------------------------ GPU
def gpu_setup(w, inp, dccm, synth, torch, dev, keys=("mixed", "fp16", "fp64"), reuse=None):
    """Device buffers, plans and the steps of the given precisions (mixed
    BF16 x 3, FP16 hi + lo, FP64).  reuse: another setup of the same
    workload whose remap tables and plans this one shares (its own device
    buffers and transform plans: a second, independent instance)."""
    groups = inp["groups"]
    n1 = len(inp["ocean"])
    if reuse is not None:
        tables, plans = reuse["tables"], reuse["remap_plans"]
    else:
        tables = []
        for g in groups:
            def gen(A, O):
                t = dccm.gen_gridmapfile_lonlat2lonlat(A[0], A[1], O[0], O[1], A[2], A[3], O[2], O[3],
                                                       accuracy_order=1, weight_mode=w["mode"])
                return t.rows()
            tables.append(remap_index(w, inp, g, gen))
        plans = [dccm.RemapPlan(g.I * g.J, n1, *tb) for g, tb in zip(groups, tables)]
    arrs, fgrid = ocean_columns(inp)
    arrs.update(synth.flux_outputs(fgrid[0], fgrid[1], fill=0.0))
    IA, JA = fgrid[0], fgrid[1]

    def to_dev(a):
        return torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)

    remapped = torch.zeros((6, JA, IA), dtype=torch.float64, device=dev)
    dflux = {}
    for name in dccm.FLUX_ARGS:
        if name == "a_Sig1Info":
            dflux[name] = arrs[name]
        elif name in REMAP_FIELDS:
            dflux[name] = remapped[REMAP_FIELDS.index(name)]
        else:
            dflux[name] = to_dev(arrs[name])
    flat = remapped.view(-1)
    spec_in = [torch.from_numpy(g.spec.view(np.float64).copy()).to(dev) for g in groups]
    grid = [torch.empty((g.nfl, g.J, g.I), dtype=torch.float64, device=dev) for g in groups]
    spec_out = [torch.empty_like(s) for s in spec_in]
    src = [torch.from_numpy(np.ascontiguousarray(g.src)).to(dev) for g in groups]
    remaps, off = [], 0
    for g, p, s in zip(groups, plans, src):
        # member m, field f -> remapped[f] interior row, columns of that member
        remaps.append((p, 6 * len(g.members), s, g.I * g.J, flat[IA + 1 + off * n1:], IA * JA, 6, n1))
        off += len(g.members)
    steps = {}
    keep = {}
    for prec, key in ((dccm.SHT_MIXED, "mixed"), (dccm.SHT_MIXED_FP16, "fp16"), (dccm.SHT_FP64, "fp64")):
        if key not in keys:
            continue
        if len(groups) == 1:
            sp = dccm.ShtPlan(groups[0].N, groups[0].I, groups[0].J, prec, groups[0].nfl)
            steps[key] = dccm.Step(sht=sp, nfl=groups[0].nfl, spec_in=spec_in[0], grid=grid[0],
                                   spec_out=spec_out[0], remaps=remaps, flux=dflux, flux_grid=fgrid)
        else:
            sp = dccm.Ensemble([(g.N, g.I, g.J, g.nfl) for g in groups], prec)
            steps[key] = dccm.Step(ensemble=sp, ens_spec_in=spec_in, ens_grid=grid, ens_spec_out=spec_out,
                                   ens_nfl=[g.nfl for g in groups], remaps=remaps, flux=dflux, flux_grid=fgrid)
        keep[key] = sp
    nnz = sum(len(t[2]) for t in tables)
    return dict(steps=steps, plans=keep, spec_in=spec_in, grid=grid, spec_out=spec_out, src=src, dflux=dflux,
                tables=tables, nnz=nnz, ncol=IA - 2, remap_plans=plans, remaps=remaps, fgrid=fgrid)


def reverse_index(w, inp, g, gen):
    """(send, recv, coef) from the ocean columns to group g's Gaussian grid:
    the table of the ocean grid to the atmosphere grid, rows whose source
    cell is land left out (no surface data there), send over the ocean
    columns."""
    A, O = g.axes, inp["O"]
    iD, jD, iS, jS, wts = gen(O, A)
    lin = (iS - 1) + w["onx"] * (jS - 1)
    keep = inp["mask"][lin] == 1
    rank = np.full(w["onx"] * w["ony"], -1, np.int64)
    rank[inp["ocean"]] = np.arange(len(inp["ocean"]))
    send = (rank[lin[keep]] + 1).astype(np.int32)
    recv = (iD[keep] + g.I * (jD[keep] - 1)).astype(np.int32)
    return send, recv, wts[keep]


def coupled_setup(S, w, inp, dccm, synth, torch, dev, key="mixed"):
    """The step with the implicit surface coupling around the flux, one
    truncation group: the forward sweep on every column of the atmosphere
    grid (the group's levels / fields, one tracer), ImplCplCoef1/2 (4 slots
    each) remapped with the surface fields to the ocean columns, the flux,
    DelVarImplCPL (U, V, T, vapour) remapped back onto level 1 of the
    tendencies (atm/dccm_atm_mod.f90:832-835), the backward sweep."""
    g = inp["groups"][0]
    ncol, kmax = g.I * g.J, max(2, g.nfl // 4)
    IA, JA = S["fgrid"][0], S["fgrid"][1]
    n1 = len(inp["ocean"])
    plan = dccm.ImplCplPlan(ncol, kmax, 1, 1, synth.IMPLCPL_CONSTS)
    prof = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
            for k, v in synth.column_profiles(ncol, kmax, ncmax=1, seed=7).items()}
    shapes = {"DUDt": (kmax, ncol), "DVDt": (kmax, ncol), "DTempDt": (kmax, ncol), "DQMixDt": (1, kmax, ncol),
              "ImplCplCoef1": (4, ncol), "ImplCplCoef2": (4, ncol)}
    out = {k: torch.zeros(v, dtype=torch.float64, device=dev) for k, v in shapes.items()}
    fwd_plan = S["remap_plans"][0]
    df = S["dflux"]
    coef = [(fwd_plan, 4, out[n], ncol, df[n].view(-1)[IA + 1:], IA * JA) for n in ("ImplCplCoef1", "ImplCplCoef2")]

    def gen(A, O):
        t = dccm.gen_gridmapfile_lonlat2lonlat(A[0], A[1], O[0], O[1], A[2], A[3], O[2], O[3],
                                               accuracy_order=1, weight_mode=w["mode"])
        return t.rows()
    rplan = dccm.RemapPlan(n1, ncol, *reverse_index(w, inp, g, gen))
    dv = df["DelVarImplCPL"].view(-1)
    post = [(rplan, 1, dv[q * IA * JA + IA + 1:], IA * JA, (out[n][0] if n != "DQMixDt" else out[n][0, 0]), ncol)
            for q, n in enumerate(("DUDt", "DVDt", "DTempDt", "DQMixDt"))]
    sp = S["plans"][key]
    step = dccm.Step(sht=sp, nfl=g.nfl, spec_in=S["spec_in"][0], grid=S["grid"][0], spec_out=S["spec_out"][0],
                     remaps=list(S["remaps"]) + coef, flux=df, flux_grid=S["fgrid"], implcpl=plan,
                     implcpl_prof=prof, implcpl_out=out, remaps_post=post)
    return dict(step=step, plan=plan, prof=prof, out=out, coef=coef, post=post, rplan=rplan, ncol=ncol, kmax=kmax)


# Flux arrays a coupling step exchanges with the host, with the slots that
# carry data: per-step surface state in, fluxes and coefficients out (slot 3
# of the net/SW-radiation fluxes and their derivative is left untouched; the
# merged surface temperature and albedo land in slot 3).
FLUX_H2D = {"SDwRFlx": (0,), "ImplCplCoef1": (0, 1, 2, 3), "ImplCplCoef2": (0, 1, 2, 3), "SfcTemp": (0, 1),
            "SfcAlbedo": (0, 1), "SIceCon": (0,), "SfcHeight": (0,)}
FLUX_D2H_SLOTS = {"DelVarImplCPL": (0, 1, 2, 3), "SfcHFlx_ns": (0, 1), "SfcHFlx_sr": (0, 1),
                  "DSfcHFlxDTs": (0, 1), "SfcTemp": (2,), "SfcAlbedo": (2,)}


def host_copies(S, groups, dccm, torch):
    """(pinned host, device) pairs of one coupling step's inputs and results:
    spectra and remap sources in, analysed spectra out, and the interior
    ocean columns of the surface arrays (one contiguous run per slot).  The
    surface side lives in one page-locked host allocation per direction
    (remap sources then surface rows), as a host model keeps it."""
    h2d = [(torch.from_numpy(g.spec.view(np.float64).copy()).pin_memory(), s) for g, s in zip(groups, S["spec_in"])]
    d2h = [(torch.empty_like(s, device="cpu").pin_memory(), s) for s in S["spec_out"]]
    df = S["dflux"]

    def run(name, slot):
        a = df[name]
        return a[slot, 1, 1:-1] if a.dim() == 3 else a[1, 1:-1]

    def host_block(devs, fill):
        """One pinned buffer holding a view per device tensor, in order."""
        n = sum(d.numel() for d in devs)
        buf = torch.empty(n, dtype=torch.float64).pin_memory()
        out, off = [], 0
        for d in devs:
            h = buf[off:off + d.numel()].view(d.shape)
            if fill:
                h.copy_(d.cpu())
            out.append((h, d))
            off += d.numel()
        return out

    ins = list(S["src"]) + [run(n, k) for n, slots in FLUX_H2D.items() for k in slots]
    h2d += host_block(ins, True)
    outs = [run(n, k) for n in dccm.FLUX_OUT + ["SfcTemp", "SfcAlbedo"] for k in FLUX_D2H_SLOTS.get(n, (0, 1, 2))]
    d2h += host_block(outs, False)
    return h2d, d2h


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# each stage's kernels in one ncu capture of `bench.py --profile-steps`,
# kept with the profiles of the c3 step; null where not captured.  The c3
# step's working set (about 85 MB) fits the 126 MB L2, so a kernel's
# writes can stay in L2 past its end and its DRAM bytes can fall below its
# algorithmic bytes; the L2 bytes of the same launches (lts__t_bytes.sum,
# every request L2 serves) are reported beside them.
TRAFFIC = {
    "c3": {"legendre_inverse": 7685632 + 12131072, "fft_inverse": 11304192, "fft_forward": 33602304,
           "legendre_forward": 18938368, "remap": 3995904, "bulk_flux": 7722240},
}
L2_BYTES = {
    "c3": {"legendre_inverse": 30760000 + 49978368, "fft_inverse": 85293248, "fft_forward": 79587712,
           "legendre_forward": 43426816, "remap": 20492224, "bulk_flux": 41896288},
}
TRAFFIC_SOURCE = "ncu of bench.py --workload c3 --profile-steps 3, third replay (profiles/step_c3_launches.md)"
# FP64 peak: measured on the device by dccm_fp64_peak (independent DFMA
# chains on every SM) at the start of the run; the nominal figure (2 DFMA
# lanes per SM and clock at the maximum SM clock) is reported beside it.
FP64_NOMINAL_TFLOPS = 152 * 2 * 2 * 2.070e9 / 1e12


def stage_work(S, inp, groups):
    """Algorithmic bytes (minimal HBM traffic) and flops of each stage.
    Legendre synthesis: FP64 spectra in, FP32 Fourier coefficients out, the
    split Legendre table (6 bytes an entry) in; analysis the reverse.  The
    tensor work (six BF16 products of the split operands) is far below the
    byte time, so both Legendre stages are bandwidth-bound.  FFT: FP32
    Fourier coefficients <-> FP64 grid.  Remap: 16 bytes per table entry,
    source fields once and destination rows (the sliced layout's padding
    and slice descriptors are overhead, not counted).  Flux: 504 bytes per
    ocean column (inputs and outputs, FP64)."""
    spec = sum(g.nfl * (g.N + 1) * (g.N + 2) // 2 * 16 for g in groups)
    four = sum(g.nfl * g.J * (g.N + 1) * 2 * 4 for g in groups)
    table = sum((g.N + 1) * (g.N + 2) // 2 * (g.J // 2) * 6 for g in groups)
    grid = sum(g.nfl * g.J * g.I * 8 for g in groups)
    flops = sum(2.0 * g.J * (g.N + 1) * (g.N + 2) / 2 * g.nfl for g in groups)
    n1 = len(inp["ocean"])
    remap = sum(16 * len(tb[2]) + 8 * 6 * len(g.members) * (g.I * g.J + n1)
                for g, tb in zip(groups, S["tables"]))
    return {"legendre_inverse": (spec + four + table, flops), "fft_inverse": (four + grid, None),
            "fft_forward": (grid + four, None), "legendre_forward": (four + spec + table, flops),
            "remap": (remap, None), "bulk_flux": (504 * S["ncol"], None)}


def stage_work_f64(groups):
    """The FP64 path's algorithmic work per stage: Legendre 2 J Ncoef FP64
    flops per field-level (complex x real multiply-adds over the latitude
    pairs, both parities), bytes of the FP64 spectra, the FP64 Fourier
    coefficients (16 J (N+1) per field-level) and the FP64 Pbar table
    (8 Ncoef J/2); FFT 5 I log2(I) flops per row pair (complex FFT of the
    packed pair), bytes of the grid and the Fourier coefficients."""
    out = {}
    spec = sum(g.nfl * (g.N + 1) * (g.N + 2) // 2 * 16 for g in groups)
    four = sum(g.nfl * g.J * (g.N + 1) * 16 for g in groups)
    table = sum((g.N + 1) * (g.N + 2) // 2 * (g.J // 2) * 8 for g in groups)
    grid = sum(g.nfl * g.J * g.I * 8 for g in groups)
    leg = sum(2.0 * g.J * (g.N + 1) * (g.N + 2) / 2 * g.nfl for g in groups)
    fft = sum(5.0 * g.I * np.log2(g.I) * (g.J // 2) * g.nfl for g in groups)
    out["legendre_inverse"] = (spec + four + table, leg)
    out["fft_inverse"] = (four + grid, fft)
    out["fft_forward"] = (grid + four, fft)
    out["legendre_forward"] = (four + spec + table, leg)
    return out


CHAIN = ["legendre_inverse", "fft_inverse", "fft_forward", "legendre_forward"]


def fp64_pipe(ops, ms, fp64_peak):
    """FP64 pipe occupancy of a stage: a DADD, a DMUL and a DFMA each take
    one issue slot of the FP64 pipe (2 lanes per SM and clock), so the
    pipe's operation rate is half the measured DFMA flop rate (TFLOP/s)
    and a kernel of separate multiplies and adds is bound there.  ops: FP64
    operations per launch; ms: the launch's time; floor_ms: the time those
    operations need on the whole GPU's pipe."""
    rate = ops / (ms / 1e3) / 1e12
    return {"ops_per_launch": ops, "achieved": rate, "unit": "T ops/s", "peak": fp64_peak / 2,
            "frac": rate / (fp64_peak / 2), "floor_ms": ops / (fp64_peak / 2 * 1e12) * 1e3}


def remap_pipe_ops(tables, members, fields=6):
    """FP64 operations of the remap apply: one DMUL per table entry and
    field, one DADD per entry and field after each destination row's first
    (the first addition, 0 + p, is done on the integer pipes); tables are
    (send, recv, coef) per group, each applied to fields x members columns."""
    return sum((2.0 * len(t[2]) - len(np.unique(t[1]))) * fields * m for t, m in zip(tables, members))


def roofline(S, inp, groups, stage_ms, workload, fp64_peak, flux_alone=None, products=6):
    """Per-stage roofline against the copy bandwidth, and the headline: the
    transform chain (spectra pack + Legendre synthesis, inverse FFT, forward
    FFT, Legendre analysis), the step's critical path, as one entry (its
    algorithmic bytes over the sum of its stage times).  Legendre stages
    also report their tensor rate against the BF16 peak divided by the
    products per multiply-add (6 for BF16 x 3, 3 for FP16 hi + lo), with
    the raw fraction of the BF16 peak beside it.  The flux kernel, bound by
    the FP64 pipe, reports its FP64 instruction rate (ncu counts per
    column) over the measured FP64 peak.  flux_alone: the flux kernel timed
    alone on its full grid when the step caps its grid; its roofline is then
    taken from that time (the step's time and cap are kept beside it)."""
    hbm, bf16, src_peak = peaks()
    names = dccm_stages()
    work = stage_work(S, inp, groups)
    traffic = TRAFFIC.get(workload, {})
    l2b = L2_BYTES.get(workload, {})
    stages = {}
    stage_ms = list(stage_ms)
    if flux_alone:
        stage_ms[names.index("bulk_flux")] = flux_alone["ms"]
    for n, ms in zip(names, stage_ms):
        q, fl = work[n]
        ach = q / (ms / 1e3) / 1e9
        st = {"ms": float(ms), "bound": "hbm", "achieved": ach, "unit": "GB/s", "peak": hbm, "frac": ach / hbm,
              "algorithmic_bytes": q, "traffic": traffic.get(n), "l2_bytes": l2b.get(n)}
        if fl is not None:
            tf = fl / (ms / 1e3) / 1e12
            st["tensor"] = {"achieved": tf, "unit": "TFLOP/s", "peak": bf16 / products, "frac": tf / (bf16 / products),
                            "products_per_mac": products, "raw_peak": bf16, "raw_frac": tf / bf16,
                            "algorithmic_flops": fl}
        stages[n] = st
    stages["bulk_flux"]["limiter"] = "FP64 pipe, not HBM"
    if flux_alone:
        stages["bulk_flux"]["launch"] = ("full grid, timed alone; in the step its grid is capped at %d CTAs "
                                         "(%.4f ms there)" % (flux_alone["step_cta_cap"], flux_alone["ms_in_step"]))
    f64 = FLUX_FP64_INSTR_PER_COLUMN * S["ncol"]
    tf = f64 / (stages["bulk_flux"]["ms"] / 1e3) / 1e12
    stages["bulk_flux"]["fp64"] = {"achieved": tf, "unit": "TFLOP/s", "peak": fp64_peak,
                                   "peak_source": "measured (dccm_fp64_peak)", "frac": tf / fp64_peak,
                                   "flops_per_launch": f64,
                                   "count": "FP64 pipe work per column from ncu instruction counts (DADD + DMUL "
                                            "+ 2 DFMA), the same for every ice-free column",
                                   "pipe": fp64_pipe(FLUX_FP64_PIPE_OPS_PER_COLUMN * S["ncol"],
                                                     stages["bulk_flux"]["ms"], fp64_peak)}
    # the remap keeps the reference's separately rounded products and sums
    # (bit-exact): one DMUL per table entry and field, and one DADD per
    # entry and field after each row's first (the first addition, 0 + p, is
    # done on the integer pipes), reported beside its bytes
    rf = sum(2.0 * len(t[2]) * 6 * len(g.members) for g, t in zip(groups, S["tables"]))
    rops = remap_pipe_ops(S["tables"], [len(g.members) for g in groups])
    tf = rf / (stages["remap"]["ms"] / 1e3) / 1e12
    stages["remap"]["fp64"] = {"achieved": tf, "unit": "TFLOP/s", "peak": fp64_peak,
                               "peak_source": "measured (dccm_fp64_peak)", "frac": tf / fp64_peak,
                               "flops_per_launch": rf, "pipe": fp64_pipe(rops, stages["remap"]["ms"], fp64_peak)}
    cq = sum(work[n][0] for n in CHAIN)
    cms = sum(stage_ms[names.index(n)] for n in CHAIN)
    ctr = [traffic.get(n) for n in CHAIN]
    cl2 = [l2b.get(n) for n in CHAIN]
    ach = cq / (cms / 1e3) / 1e9
    roof = {"kernel": "transform chain: spectra pack + Legendre synthesis (tcgen05), inverse FFT, forward FFT, "
                      "Legendre analysis (tcgen05)",
            "bound": "hbm", "achieved": ach, "unit": "GB/s", "peak": hbm, "frac": ach / hbm, "ms": cms,
            "algorithmic_bytes": cq, "traffic": sum(ctr) if all(x is not None for x in ctr) else None,
            "l2_bytes": sum(cl2) if all(x is not None for x in cl2) else None,
            "peak_source": src_peak, "critical_path": True,
            "traffic_source": (TRAFFIC_SOURCE if workload in TRAFFIC else None),
            "stages": stages}
    return roof


def roofline_f64(groups, stage_ms, fp64_peak):
    """Stage rooflines of the FP64 step (the denominator of mixed / FP64):
    FP64 flops over the measured FP64 peak, bytes over the copy bandwidth."""
    hbm, _, _ = peaks()
    work = stage_work_f64(groups)
    names = dccm_stages()
    out = {}
    for n in CHAIN:
        ms = float(stage_ms[names.index(n)])
        q, fl = work[n]
        tf = fl / (ms / 1e3) / 1e12
        out[n] = {"ms": ms, "fp64": {"achieved": tf, "unit": "TFLOP/s", "peak": fp64_peak, "frac": tf / fp64_peak,
                                     "algorithmic_flops": fl},
                  "hbm": {"achieved": q / (ms / 1e3) / 1e9, "unit": "GB/s", "peak": hbm,
                          "frac": q / (ms / 1e3) / 1e9 / hbm, "algorithmic_bytes": q}}
    return out


# FP64 pipe work of the flux kernel per ocean column: DADD + DMUL + 2 DFMA
# thread instructions (ncu sass counters, c3, 45,478 columns: 1,182,428
# DADD, 3,137,982 DMUL, 5,002,580 DFMA; the reciprocals, square roots, exp
# and log are the kernel's own, csrc/fp64_fast.cuh).  Every column does the
# same work when there is no sea ice (all workloads here: warps whose
# columns all have SIceCon = 0 skip the ice physics and the merging), so
# the per-column figure carries to every workload.
FLUX_FP64_INSTR_PER_COLUMN = (1182428 + 3137982 + 2 * 5002580) / 45478
# the same counts as FP64 pipe operations (one issue slot each)
FLUX_FP64_PIPE_OPS_PER_COLUMN = (1182428 + 3137982 + 5002580) / 45478


# FP64 flops of the implicit-coupling sweeps per column and level, one
# tracer (DADD + DMUL + 2 DFMA thread instructions, ncu sass counters,
# 32768 columns x 32 levels): per 32-level column forward 3163 (shared
# factors 502 + elimination 2661), backward 1058.
IMPLCPL_FP64_FLOPS = {"forward": 3163 / 32, "backward": 1058 / 32}


def dccm_stages():
    return ["legendre_inverse", "fft_inverse", "fft_forward", "legendre_forward", "remap", "bulk_flux"]


def profile_run(args, w, inp):
    """Graph replays of the mixed-precision step only (default launch
    shapes or --knobs, no autotuning, no host copies): a small, countable
    launch sequence for ncu.  Each replay launches, in order, the spectra
    pack, Legendre synthesis, inverse FFT, forward FFT, Legendre analysis,
    one remap per truncation group and the flux kernel."""
    import torch
    dccm = importlib.import_module("dennou-ccm_gb300")
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    set_knobs(dccm, args.knobs)
    dev = torch.device("cuda", 0)
    S = gpu_setup(w, inp, dccm, synth, torch, dev)
    step = S["steps"]["mixed"]
    for _ in range(args.profile_steps):
        step.run()
    torch.cuda.synchronize()
    st, derr = S["plans"]["mixed"].status()
    # then the implicit surface coupling of the largest group's atmosphere:
    # forward and backward sweep, profile_steps times each, in that order
    g = max(inp["groups"], key=lambda q: q.I * q.J)
    ncol, kmax = g.I * g.J, max(2, g.nfl // 4 if len(inp["groups"]) == 1 else 32)
    d = synth.column_profiles(ncol, kmax, ncmax=1, seed=7)
    plan = dccm.ImplCplPlan(ncol, kmax, 1, 1, synth.IMPLCPL_CONSTS)
    dd = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in d.items()}
    shapes = {"DUDt": (kmax, ncol), "DVDt": (kmax, ncol), "DTempDt": (kmax, ncol), "DQMixDt": (1, kmax, ncol),
              "ImplCplCoef1": (4, ncol), "ImplCplCoef2": (4, ncol)}
    out = {k: torch.empty(v, dtype=torch.float64, device=dev) for k, v in shapes.items()}
    for _ in range(args.profile_steps):
        plan.forward_dev(dd, out)
        plan.backward_dev(out)
    torch.cuda.synchronize()
    print(json.dumps({"profile_steps": args.profile_steps, "workload": args.workload, "status": st,
                      "device_error": derr, "implcpl_columns": ncol, "implcpl_levels": kmax}))


GAUSSIAN_GRIDS = {21: (64, 32), 42: (128, 64), 63: (192, 96), 85: (256, 128), 170: (512, 256), 341: (1024, 512)}


def set_knobs(dccm, knobs):
    """"k=v,k=v" -> dccm_tune_set for each (the profiling modes' launch shapes)."""
    for kv in filter(None, knobs.split(",")):
        k, v = kv.split("=")
        dccm.tune_set(k.strip(), int(v))


def profile_sht(spec, knobs=""):
    """Mixed-precision transforms only, for ncu on a small case: "N:B"
    (truncation, field-levels) on the truncation's Gaussian grid; three
    inverse + forward round trips on the device (each: the spectra pack,
    Legendre synthesis, inverse FFT, forward FFT, Legendre analysis)."""
    import torch
    dccm = importlib.import_module("dennou-ccm_gb300")
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    set_knobs(dccm, knobs)
    N, B = (int(x) for x in spec.split(":"))
    I, J = GAUSSIAN_GRIDS[N]
    plan = dccm.ShtPlan(N, I, J, dccm.SHT_MIXED, max_batch=B)
    s = torch.from_numpy(synth.spectra(N, B, seed=1).view(np.float64).copy()).cuda()
    g = torch.empty((B, J, I), dtype=torch.float64, device="cuda")
    s2 = torch.empty_like(s)
    for _ in range(3):
        plan.inverse_dev(s, g, B)
        plan.forward_dev(g, s2, B)
    torch.cuda.synchronize()
    err = float((s2 - s).norm() / s.norm())
    st = plan.status()
    print(json.dumps({"profile_sht": spec, "grid": [I, J], "round_trip": err, "status": list(st)}))
    assert err < 1e-5 and st == (0, 0)


def max_over_ranks(vals, world, dev):
    """Element-wise maximum of per-rank times over the process group (the
    job's time is its slowest replica); identity on one rank.  dev is where
    the reduction tensor lives (a CUDA device for NCCL, "cpu" for gloo)."""
    if world <= 1:
        return list(vals)
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def job_throughput(world, nfl, t_step):
    """Whole-job field-levels/s: every replica transforms nfl field-levels
    per step (weak scaling), the job's step time is the slowest rank's."""
    return world * nfl / t_step


def gpu_bench(args, w, inp, rank, world):
    import torch
    dccm = importlib.import_module("dennou-ccm_gb300")
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    dccm.load()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    S = gpu_setup(w, inp, dccm, synth, torch, dev)
    # launch shapes from the autotuner (cached per GPU and step shape)
    cache = os.environ.get("DCCM_TUNE_CACHE", os.path.join(ROOT, "dennou-ccm_gb300", "tune_cache.jsonl"))
    tuned = {k: S["steps"][k].autotune(cache) for k in ("fp64", "fp16", "mixed")}
    groups = inp["groups"]
    nfl = inp["nfl"]
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
        for k in range(K):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            step.run(stream)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return [a.elapsed_time(b) for a, b in evs]

    clocks = Clocks(dev.index or 0)
    clocks.start()
    ms_mixed = timed(S["steps"]["mixed"], args.steps, max(3, args.warmup))
    ck = clocks.stop(dev.index or 0)
    ms_fp64 = timed(S["steps"]["fp64"], args.steps, max(3, args.warmup))
    ms_fp16 = timed(S["steps"]["fp16"], args.steps, max(3, args.warmup))
    t_mixed, t_fp64, t_fp16 = max_over_ranks([float(np.mean(ms_mixed)) / 1e3, float(np.mean(ms_fp64)) / 1e3,
                                              float(np.mean(ms_fp16)) / 1e3], world, dev)

    # accuracy of the mixed steps against the FP64 step on the same inputs
    S["steps"]["fp64"].run(stream)
    torch.cuda.synchronize()
    ref_spec = [s.clone() for s in S["spec_out"]]
    ref_grid = [g.clone() for g in S["grid"]]

    def rel(a, b):
        num = sum(float(torch.linalg.norm(x - y)) ** 2 for x, y in zip(a, b))
        den = sum(float(torch.linalg.norm(y)) ** 2 for y in b)
        return (num / den) ** 0.5

    def max_field(a, b):  # the worst field-level's relative L2 error
        return max(float((torch.linalg.norm((x - y).reshape(x.shape[0], -1), dim=1) /
                          torch.linalg.norm(y.reshape(y.shape[0], -1), dim=1)).max()) for x, y in zip(a, b))

    def accuracy(key):
        S["steps"][key].run(stream)
        torch.cuda.synchronize()
        st, derr = S["plans"][key].status()
        assert st == 0 and derr == 0, ("device error", key, st, derr)
        return {"spec_vs_fp64": rel(S["spec_out"], ref_spec), "grid_vs_fp64": rel(S["grid"], ref_grid),
                "round_trip": rel(S["spec_out"], S["spec_in"]),
                "max_field_spec_vs_fp64": max_field(S["spec_out"], ref_spec),
                "max_field_grid_vs_fp64": max_field(S["grid"], ref_grid)}

    err_fp16 = accuracy("fp16")
    err = accuracy("mixed")  # last, so the mixed step's outputs are the ones left in place

    # per-kernel device times (stages launched back to back with events)
    stage_ms = np.zeros(6)
    nt = max(3, min(10, args.steps))
    for k in range(nt):
        flush.fill_(float(k))
        stage_ms += np.array(S["steps"]["mixed"].run_timed(stream))
    stage_ms /= nt
    fp64_peak = dccm.fp64_peak(stream)
    # the FP64 step's stages the same way: the denominator of mixed / FP64
    stage_f64 = np.zeros(6)
    for k in range(nt):
        flush.fill_(float(k))
        stage_f64 += np.array(S["steps"]["fp64"].run_timed(stream))
    stage_f64 /= nt
    roof_f64 = roofline_f64(groups, stage_f64, fp64_peak)
    # The whole-step autotune may cap the flux kernel's grid (it runs beside
    # the transforms and then leaves them issue slots); the kernel's own
    # roofline is taken on its full grid, timed alone the same way.
    flux_alone = None
    cap = tuned["mixed"].get("flux_ctas", 0)
    if cap:
        saved_cap = dccm.tune_get("flux_ctas")
        dccm.tune_set("flux_ctas", 0)
        ts = []
        for k in range(max(3, args.warmup) + nt):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dccm.DSFCM_Util_SfcBulkFlux_Get(S["dflux"], *S["fgrid"], device=True, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= max(3, args.warmup):
                ts.append(e0.elapsed_time(e1))
        dccm.tune_set("flux_ctas", saved_cap)
        flux_alone = {"ms": float(np.mean(ts)), "ms_in_step": float(stage_ms[5]), "step_cta_cap": cap}
    roof = roofline(S, inp, groups, stage_ms, args.workload, fp64_peak, flux_alone)
    roof["fp64_peak"] = {"measured": fp64_peak, "nominal": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s"}

    # end to end through the public API with host buffers (pinned)
    # (the copy lists are prepared once, as a model with persistent host
    # buffers would; every call still copies every byte in and out)
    hc = dccm.HostCopies(*host_copies(S, groups, dccm, torch))
    h2d_bytes, d2h_bytes = hc.nbytes()
    host_tuned = S["steps"]["mixed"].autotune_host(hc, stream=stream)
    cand = host_tuned.pop("candidates_ms")
    host_tuned.update({"ms": cand.get("%d,%d" % (host_tuned["upload_order"], host_tuned["host_path"])),
                       "ms_copy_engines": [cand.get("1,1"), cand.get("2,1")],
                       "ms_all_mapped": [cand.get("1,16"), cand.get("2,16")]})
    for _ in range(max(3, args.warmup)):
        S["steps"]["mixed"].run_host(hc, stream=stream)
    if world > 1:
        torch.distributed.barrier()
    te = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        S["steps"]["mixed"].run_host(hc, stream=stream)
        te.append(time.perf_counter() - t0)
    t_e2e, = max_over_ranks([float(np.mean(te))], world, dev)
    e2e2 = e2e_two_in_flight(args, w, inp, S, hc, host_tuned, dccm, synth, torch, dev, world, cache)
    launches = 5 + len(groups) + 1  # pack + 2 Legendre + 2 FFT + one remap per group + flux
    ic = implcpl_leg(args, groups, dccm, synth, torch, dev, stream, flush, fp64_peak)
    so = spec_ops_leg(args, groups, S, dccm, torch, stream, flush)
    coupled = None
    if len(groups) == 1:  # the step with the implicit coupling around the flux
        C = coupled_setup(S, w, inp, dccm, synth, torch, dev)
        # its own launch shapes: here the surface branch is the longer one
        tuned_c = C["step"].autotune(cache)
        ms_c = timed(C["step"], args.steps, max(3, args.warmup))
        t_c, = max_over_ranks([float(np.mean(ms_c)) / 1e3], world, dev)
        coupled = {"ms_per_step": t_c * 1e3, "plain_ms_per_step": t_mixed * 1e3,
                   "value": job_throughput(world, nfl, t_c), "unit": "field-levels/s",
                   "implcpl_columns": C["ncol"], "levels": C["kmax"], "launch_shapes": tuned_c,
                   "surface_branch": "implicit coupling forward, remaps (+ ImplCplCoef1/2), flux, "
                                     "DelVarImplCPL back to level 1, implicit coupling backward"}
        del C
    return dict(t_mixed=t_mixed, t_fp64=t_fp64, t_fp16=t_fp16, err_fp16=err_fp16, t_e2e=t_e2e, clocks=ck, roof=roof,
                roof_f64=roof_f64, stage_f64=[float(x) for x in stage_f64], err=err, h2d=h2d_bytes,
                d2h=d2h_bytes, nfl=nfl, launches=launches, tables=S["tables"], tuned=dict(tuned, host=host_tuned),
                implcpl=ic, spec_ops=so, coupled=coupled, e2e2=e2e2)


def e2e_two_in_flight(args, w, inp, S, hc, host_tuned, dccm, synth, torch, dev, world, cache):
    """End to end with two independent instances of the step in flight
    (ensemble members or separate runs: each its own device buffers,
    transform plans and page-locked host buffers, the remap plans shared),
    each through dccm_step_launch_host on a stream of its own, the steps
    issued to the two in turn, so one instance's downloads share the host
    link with the other's uploads.  Every step still copies all its inputs
    in and its results out.  Time per step = the span of K steps (CUDA
    events on a stream that waits for both) / K; no L2 flush between steps
    (two are in flight; every step's inputs arrive over the host link).
    Host-copy choices tried (dccm_step_host_choice): each instance's own
    choice from dccm_step_autotune_host, and the copy engines alone under
    either upload order; the fastest is reported, all are listed.  The
    second instance's downloads are compared with the first's (same
    inputs, bit-identical)."""
    groups = inp["groups"]
    S2 = gpu_setup(w, inp, dccm, synth, torch, dev, keys=("mixed",), reuse=S)
    step1, step2 = S["steps"]["mixed"], S2["steps"]["mixed"]
    step2.autotune(cache)
    hc2 = dccm.HostCopies(*host_copies(S2, groups, dccm, torch))
    cur = torch.cuda.current_stream(dev)
    t2 = step2.autotune_host(hc2, stream=cur)
    own = [(host_tuned["upload_order"], host_tuned["host_path"], host_tuned["flux_ctas"]),
           (t2["upload_order"], t2["host_path"], t2["flux_ctas"])]
    cands = {"each instance's own tuned choice": own,
             "copy engines, transforms' inputs first": [(1, 1, c[2]) for c in own],
             "copy engines, surface inputs first": [(2, 1, c[2]) for c in own]}
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    inst = [(step1, hc, streams[0]), (step2, hc2, streams[1])]
    K = max(10, args.steps)

    def issue(n):
        for k in range(n):
            st, h, sx = inst[k % 2]
            st.launch_host(h, stream=sx)

    def span():
        torch.cuda.synchronize()
        issue(2 * max(3, args.warmup))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(cur)
        for sx in streams:
            sx.wait_event(ev0)
        issue(K)
        for sx in streams:
            e = torch.cuda.Event()
            e.record(sx)
            cur.wait_event(e)
        ev1.record(cur)
        torch.cuda.synchronize()
        t, = max_over_ranks([ev0.elapsed_time(ev1) / 1e3 / K], world, dev)
        return t

    times = {}
    for name, ch in cands.items():
        for st, c in zip((step1, step2), ch):
            st.host_choice(*c)
        times[name] = span()
    best = min(times, key=times.get)
    for st, c in zip((step1, step2), cands[best]):
        st.host_choice(*c)
    t = span()
    same = all(torch.equal(a[0], b[0]) for a, b in zip(hc.pairs[1], hc2.pairs[1]))
    step1.host_choice(*own[0])
    h2d, d2h = hc.nbytes()
    del S2
    return {"value": job_throughput(world, inp["nfl"], t), "unit": "field-levels/s", "ms_per_step": t * 1e3,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "instances": 2, "steps": K,
            "downloads_equal": bool(same), "host_copies": best,
            "candidates_ms": {k: v * 1e3 for k, v in times.items()},
            "how": "two independent instances (own device and page-locked host buffers), "
                   "dccm_step_launch_host on two streams in turn; span of K steps / K, no L2 flush"}


def spec_ops_leg(args, groups, S, dccm, torch, stream, flush):
    """The implicit hyperdiffusion step (HDOrder 8, e-folding time 3 hours
    at the truncation wavenumber, 1200 s step, rotation correction) applied
    in place to every group's analysed spectra, as a model does after the
    forward transform; CUDA events, L2 flushed between runs.  Algorithmic
    bytes: every complex coefficient read and written once (32 B)."""
    ops = [dccm.spec_op(dccm.SPEC_HDIFF_IMPLICIT, 6.371e6, 8, 3 * 3600.0, 1200.0, True) for _ in groups]
    outs = S["spec_out"]
    ts = []
    for it in range(max(3, args.warmup) + max(3, min(args.steps, 20))):
        flush.fill_(float(it))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for g, op, o in zip(groups, ops, outs):
            dccm.spec_apply_dev(g.N, op, o, o, g.nfl, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        if it >= max(3, args.warmup):
            ts.append(e0.elapsed_time(e1))
    hbm, _, _ = peaks()
    q = sum(32 * dccm_ncoef(g.N) * g.nfl for g in groups)
    ms = float(np.mean(ts))
    return {"operator": "implicit hyperdiffusion, order 8", "launches": len(groups), "ms": ms,
            "roofline": {"bound": "hbm", "algorithmic_bytes": q, "achieved": q / (ms / 1e3) / 1e9, "unit": "GB/s",
                         "peak": hbm, "frac": q / (ms / 1e3) / 1e9 / hbm}}


def dccm_ncoef(N):
    return (N + 1) * (N + 2) // 2


def implcpl_leg(args, groups, dccm, synth, torch, dev, stream, flush, fp64_peak):
    """The implicit surface coupling of the largest truncation group's
    atmosphere (every Gaussian-grid column, the group's level count, one
    tracer), reported beside the step: forward sweep (ImplCplCoef1/2 for the
    bulk flux) and backward sweep, CUDA events, L2 flushed between runs.
    Algorithmic bytes: 12 input profiles and 4 outputs of kmax+1 levels, the
    module-state matrices written and read back (3 x 3 x kmax), FP64."""
    g = max(groups, key=lambda q: q.I * q.J)
    ncol, kmax = g.I * g.J, max(2, g.nfl // 4 if len(groups) == 1 else 32)
    d = synth.column_profiles(ncol, kmax, ncmax=1, seed=7)
    plan = dccm.ImplCplPlan(ncol, kmax, 1, 1, synth.IMPLCPL_CONSTS)
    dd = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in d.items()}
    out = {"DUDt": (kmax, ncol), "DVDt": (kmax, ncol), "DTempDt": (kmax, ncol), "DQMixDt": (1, kmax, ncol),
           "ImplCplCoef1": (4, ncol), "ImplCplCoef2": (4, ncol)}
    out = {k: torch.empty(v, dtype=torch.float64, device=dev) for k, v in out.items()}
    tf, tb = [], []
    for it in range(max(3, args.warmup) + max(3, min(args.steps, 20))):
        flush.fill_(float(it))
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        plan.forward_dev(dd, out, stream)
        e[1].record(stream)
        for k in ("DUDt", "DVDt", "DTempDt"):
            out[k][0].fill_(1e-3)  # the surface solution at level 1
        out["DQMixDt"][:, 0].fill_(1e-7)
        plan.backward_dev(out, stream)
        e[2].record(stream)
        torch.cuda.synchronize()
        if it >= max(3, args.warmup):
            tf.append(e[0].elapsed_time(e[1]))
            tb.append(e[1].elapsed_time(e[2]))
    hbm, _, _ = peaks()
    fwd_bytes = ncol * 8 * ((kmax + 1) * (9 + 1) + kmax * 2 + kmax * 4 + 8 + 3 * 3 * kmax)
    bwd_bytes = ncol * 8 * (2 * 4 * kmax + 3 * 2 * kmax)
    f, b = float(np.mean(tf)), float(np.mean(tb))

    def fp64(key, ms):
        fl = IMPLCPL_FP64_FLOPS[key] * ncol * kmax
        tfl = fl / (ms / 1e3) / 1e12
        return {"achieved": tfl, "unit": "TFLOP/s", "peak": fp64_peak, "frac": tfl / fp64_peak,
                "flops_per_launch": fl}

    return {"columns": ncol, "levels": kmax, "tracers": 1, "forward_ms": f, "backward_ms": b,
            "columns_per_s": ncol / ((f + b) / 1e3),
            "forward_roofline": {"bound": "hbm", "algorithmic_bytes": fwd_bytes,
                                 "achieved": fwd_bytes / (f / 1e3) / 1e9, "unit": "GB/s", "peak": hbm,
                                 "frac": fwd_bytes / (f / 1e3) / 1e9 / hbm, "limiter": "FP64 pipe, not HBM",
                                 "fp64": fp64("forward", f)},
            "backward_roofline": {"bound": "hbm", "algorithmic_bytes": bwd_bytes,
                                  "achieved": bwd_bytes / (b / 1e3) / 1e9, "unit": "GB/s", "peak": hbm,
                                  "frac": bwd_bytes / (b / 1e3) / 1e9 / hbm, "limiter": "FP64 pipe, not HBM",
                                  "fp64": fp64("backward", b)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only replay the mixed step this many times (for ncu) and exit")
    ap.add_argument("--profile-sht", default=None, metavar="N:B",
                    help="only run 3 mixed SHT round trips of B field-levels at truncation N (for ncu) and exit")
    ap.add_argument("--knobs", default="", metavar="K=V,...",
                    help="launch-shape knobs (dccm_tune_set) for --profile-steps / --profile-sht")
    args = ap.parse_args()
    if args.profile_sht:
        profile_sht(args.profile_sht, args.knobs)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    w = WORKLOADS[args.workload]
    synth = importlib.import_module("dennou-ccm_gb300.synth")
    import oracle
    inp = build_inputs(w, synth)
    nfl = inp["nfl"]
    config = {"workload": "%s (%s)" % (args.workload, NAMES[args.workload]),
              "truncations": sorted({g.N for g in inp["groups"]}), "members": inp["nmem"],
              "field_levels_per_gpu": nfl, "ocean_grid": [w["onx"], w["ony"]], "land_fraction": w["land"],
              "ocean_columns": int(len(inp["ocean"]) * inp["nmem"]), "remap_fields": 6,
              "l2": "flushed between timed steps (256 MB write)"}
    metric = "field-levels/s per coupling step"

    if args.impl == "reference":
        if rank != 0:
            return
        tables = []
        for g in inp["groups"]:
            tables.append(remap_index(w, inp, g, lambda A, O: oracle.j99_gen(A[0], A[1], O[0], O[1], A[3], O[3], 1,
                                                                              w["mode"])))
        t0 = time.perf_counter()
        step_s, nsample = cpu_measure(oracle, synth, w, inp, tables, args.steps, args.warmup)
        value = nfl / step_s
        cores = oracle.get_threads()
        line = {"impl": "reference", "metric": metric, "value": value, "unit": "field-levels/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded)", "config": config,
                "cpu_baseline": {"value": value, "unit": "field-levels/s", "cores": cores, "kind": "port",
                                 "sample": "per step: transforms of %d of %d field-levels (scaled), every remap "
                                           "and the bulk flux; C FP64 oracle, OpenMP" % (nsample, nfl)},
                "e2e": {"value": value, "unit": "field-levels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "wall_s": time.perf_counter() - t0}
        print(json.dumps(line))
        return

    if args.profile_steps > 0:
        profile_run(args, w, inp)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    r = gpu_bench(args, w, inp, rank, world)
    config["launch_shapes"] = r["tuned"]
    if rank != 0:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    cpu = None  # the CPU baseline is a single-GPU figure: measured at N = 1 only
    if not args.no_cpu_baseline and world == 1:
        step_s, nsample = cpu_measure(oracle, synth, w, inp, r["tables"], 3, 1, budget_s=15.0)
        cpu = {"value": nfl / step_s, "unit": "field-levels/s", "cores": oracle.get_threads(), "kind": "port",
               "sample": "3 steps: transforms of %d of %d field-levels (scaled), every remap and the bulk flux; "
                         "C FP64 oracle, OpenMP" % (nsample, nfl)}
    roof = dict(r["roof"])
    stages = roof.pop("stages")
    f64_frac = {n: round(v["fp64"]["frac"], 4) for n, v in r["roof_f64"].items()}
    # Order: the voluminous per-leg detail first, the figures a reader
    # checks first (roofline headline, end to end, FP64 comparison) last,
    # where a truncated tail of the output still shows them.
    line = {
        "metric": metric, "value": job_throughput(world, nfl, r["t_mixed"]), "unit": "field-levels/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": r["t_mixed"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3+f32 (Legendre), f32 (FFT), f64 (remap, flux)",
        "data": "synthetic (seeded PCG64; n^-3 spectra, SST-based surface state)", "config": config,
        "implicit_coupling": r["implcpl"], "spectral_operators": r["spec_ops"], "coupled_step": r["coupled"],
        "roofline_stages": stages, "fp64_gpu_stages": r["roof_f64"],
        "fp16_variant": {"value": job_throughput(world, nfl, r["t_fp16"]), "ms_per_step": r["t_fp16"] * 1e3,
                         "over_fp64": r["t_fp64"] / r["t_fp16"],
                         "legendre": "FP16 hi + lo, per-m and per-field-level power-of-two scales",
                         "accuracy": r["err_fp16"]},
        "accuracy": r["err"],
        "gpu_launches": r["launches"] * args.steps, "clocks": r["clocks"], "cpu_baseline": cpu,
        "roofline": roof,
        "e2e": {"value": job_throughput(world, nfl, r["t_e2e"]), "unit": "field-levels/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["t_e2e"] * 1e3},
        "e2e_two_in_flight": r["e2e2"],
        "stage_ms": {n: round(v["ms"], 5) for n, v in stages.items()},
        "fp64_gpu": {"value": job_throughput(world, nfl, r["t_fp64"]), "ms_per_step": r["t_fp64"] * 1e3,
                     "mixed_over_fp64": r["t_fp64"] / r["t_mixed"],
                     "stage_ms": {n: round(x, 5) for n, x in zip(dccm_stages()[:4], r["stage_f64"][:4])},
                     "stage_fp64_frac": f64_frac},
    }
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
