"""CPU tests of bench.py's work accounting: the algorithmic bytes and flops
of each stage (the roofline's numerators), and the FP64 pipe figures (a
DADD, a DMUL and a DFMA each take one issue slot of the FP64 pipe, so the
pipe's operation rate is half the measured DFMA flop rate; the remap's
count skips each destination row's first addition, done on the integer
pipes)."""
import numpy as np

import bench


def test_fp64_pipe_entry():
    e = bench.fp64_pipe(1.0e9, 2.0, 1.0)  # 1e9 operations in 2 ms at a 1 TFLOP/s DFMA peak
    assert abs(e["achieved"] - 0.5) < 1e-12 and abs(e["peak"] - 0.5) < 1e-12
    assert abs(e["frac"] - 1.0) < 1e-12 and abs(e["floor_ms"] - 2.0) < 1e-12


def test_remap_pipe_ops():
    send = np.array([1, 2, 3, 4, 5])
    recv = np.array([1, 1, 2, 3, 3])  # 5 entries over 3 destination rows
    coef = np.ones(5)
    # (5 DMUL + 2 DADD) per field, 6 fields, 2 members
    assert bench.remap_pipe_ops([(send, recv, coef)], [2]) == 84.0
    assert bench.remap_pipe_ops([(send, recv, coef), (send[:1], recv[:1], coef[:1])], [1, 3]) == 42.0 + 18.0


def test_flux_counts_per_column():
    # ncu counts of the c3 flux launch: 26 DADD, 69 DMUL, 110 DFMA a column
    assert bench.FLUX_FP64_PIPE_OPS_PER_COLUMN == 205.0
    assert bench.FLUX_FP64_INSTR_PER_COLUMN == 315.0


def test_stage_bytes_at_the_c3_workload():
    """The algorithmic bytes the roofline divides by, at c3 (T85 on its
    256 x 128 Gaussian grid, 128 field-levels, 45,478 ocean columns, a
    132,523-entry table): the figures the bench line reports."""
    from types import SimpleNamespace
    g = SimpleNamespace(N=85, I=256, J=128, nfl=128, members=[0])
    tables = [(np.zeros(132523), np.zeros(132523), np.zeros(132523))]
    S = {"tables": tables, "ncol": 45478}
    inp = {"ocean": np.zeros(45478)}
    w = bench.stage_work(S, inp, [g])
    assert w["legendre_inverse"][0] == 20370304 and w["legendre_forward"][0] == 20370304
    assert w["fft_inverse"][0] == 44826624 and w["fft_forward"][0] == 44826624
    assert sum(w[n][0] for n in bench.CHAIN) == 130393856
    assert w["remap"][0] == 5876176
    assert w["bulk_flux"][0] == 22920912
    # 2 J Ncoef flops per field-level (T85: 0.958 MFLOP)
    assert w["legendre_inverse"][1] == 2.0 * 128 * 3741 * 128
