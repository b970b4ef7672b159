"""CPU tests of the C ABI: the library builds and loads, it exports every
function include/dccm_gb300.h declares, and its host-only entry points
(status strings, table file I/O, index conversion) behave.  No call here
touches the GPU."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "dccm_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dccm_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(dccm):
    lib = dccm.load()
    names = header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    # the Python mirror declares a signature for every exported function
    assert set(names) <= set(dccm.exported_symbols()), set(names) - set(dccm.exported_symbols())


def test_status_strings(dccm):
    lib = dccm.load()
    assert lib.dccm_abi_version() == 1
    assert lib.dccm_status_string(0) == b"ok"
    for st in range(-1, -10, -1):
        assert lib.dccm_status_string(st) != b"unknown status"


def test_table_text_round_trip(dccm, oracle, synth, tmp_path):
    """The reference text format written by the oracle rows reads back
    through the library reader (set_mappingTable_interpCoef) exactly."""
    lonS, latS, _, wS = synth.gaussian_axes(64, 32)
    lonD, latD, _, wD = synth.gaussian_axes(128, 64)
    iD, jD, iS, jS, w = oracle.j99_gen(lonS, latS, lonD, latD, wS, wD, 1, 0)
    path = str(tmp_path / "t21_t42.dat")
    with open(path, "w") as f:  # Fortran list-directed style rows
        for r in zip(iD, jD, iS, jS, w):
            f.write("  %10d  %10d  %10d  %10d  %.17E\n" % r)
    send, recv, coef = dccm.set_mappingTable_interpCoef(path, 64, 128)
    s0, r0 = oracle.table_to_index(iD, jD, iS, jS, 64, 128)
    assert np.array_equal(send, s0) and np.array_equal(recv, r0) and np.array_equal(coef, w)
    t = dccm.read_table(path)
    out = str(tmp_path / "again.dat")
    t.write(out)
    rows = dccm.read_table(out).rows()
    assert np.array_equal(rows[4], w) and np.array_equal(rows[2], iS)


def test_table_reader_errors(dccm, tmp_path):
    bad = tmp_path / "bad.dat"
    bad.write_text("1 2 three 4 0.5\n")
    try:
        dccm.read_table(str(bad))
        raise AssertionError("expected an error")
    except dccm.DccmError as e:
        assert e.status == -6
    try:
        dccm.read_table(str(tmp_path / "missing.dat"))
        raise AssertionError("expected an error")
    except dccm.DccmError as e:
        assert e.status == -6
    # Fortran D exponents and comma separators are accepted
    ok = tmp_path / "ok.dat"
    ok.write_text(" 1, 1, 2, 3, 0.5D0\n\n 2 1 2 3 2.5d-1\n")
    rows = dccm.read_table(str(ok)).rows()
    assert list(rows[4]) == [0.5, 0.25] and list(rows[3]) == [3, 3]


def test_null_arguments_rejected(dccm):
    lib = dccm.load()
    h = ctypes.c_void_p()
    assert lib.dccm_remap_plan_create(4, 4, 1, None, None, None, ctypes.byref(h)) == -1
    assert lib.dccm_sfc_bulk_flux_get(None, None) == -1
    assert lib.dccm_remap_table_read(None, ctypes.byref(h)) == -1


def test_failure_path_knobs(dccm):
    """The wait limit and the test-only load withholding are process-wide
    knobs with checked ranges (setting them launches nothing)."""
    saved = {k: dccm.tune_get(k) for k in ("wait_limit_ms", "tc_withhold_loads")}
    try:
        dccm.tune_set("wait_limit_ms", 60000)
        assert dccm.tune_get("wait_limit_ms") == 60000
        for bad in (("wait_limit_ms", 60001), ("wait_limit_ms", -1), ("no_such_knob", 1), ("prio", 3)):
            try:
                dccm.tune_set(*bad)
                raise AssertionError("accepted %r" % (bad,))
            except dccm.DccmError as e:
                assert e.status == -1
        dccm.tune_set("tc_withhold_loads", 5)
        assert dccm.tune_get("tc_withhold_loads") == 1
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)


def test_spml_index_functions(dccm):
    """l_nm / nm_l (SPML's storage rule of its wa arrays) are inverse to each
    other and cover 1..(N+1)^2 exactly once."""
    N = 42
    ls = []
    for n in range(N + 1):
        for m in range(-n, n + 1):
            l = dccm.l_nm(n, m)
            assert tuple(int(x) for x in dccm.nm_l(l)) == (n, m)
            ls.append(l)
    assert sorted(ls) == list(range(1, (N + 1) ** 2 + 1))
    n, m = dccm.nm_l(np.arange(1, (N + 1) ** 2 + 1))
    assert np.array_equal(dccm.l_nm(n, m), np.arange(1, (N + 1) ** 2 + 1))
