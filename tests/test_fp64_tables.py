"""The committed tables of the bulk-flux kernel's FP64 exp and log
(csrc/fp64_tables.cuh) are what their generator writes, and each entry is
the double nearest to its exact value (checked here against mpmath at 200
bits, independently of the generator's own formatting)."""
import os
import re
import subprocess
import sys

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "dennou-ccm_gb300", "csrc")


def test_tables_match_generator():
    pytest.importorskip("mpmath")
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_fp64_tables.py")], check=True,
                         capture_output=True, text=True, cwd=CSRC).stdout
    with open(os.path.join(CSRC, "fp64_tables.cuh")) as f:
        assert f.read() == out


def test_table_entries_are_nearest_doubles():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    text = open(os.path.join(CSRC, "fp64_tables.cuh")).read()

    def block(name):
        body = text[text.index(name):]
        body = body[body.index("{") + 1:body.index("};")]
        return [float.fromhex(x) for x in re.findall(r"-?0x[0-9a-fA-F.]+p[-+]\d+", body)]

    exp2 = block("EXP2_64[64]")
    assert len(exp2) == 64
    for j, v in enumerate(exp2):
        assert v == float(mpmath.power(2, mpmath.mpf(j) / 64)), j
    pairs = block("LOG_F128[129]")
    lo = block("LOG_F128_LO[129]")
    assert len(pairs) == 2 * 129 and len(lo) == 129
    for j in range(129):
        F = 1 + mpmath.mpf(j) / 128
        assert pairs[2 * j] == float(1 / F), j
        assert pairs[2 * j + 1] == float(mpmath.log(F)), j
        assert lo[j] == float(mpmath.log(F) - mpmath.mpf(pairs[2 * j + 1])), j
    consts = dict(re.findall(r"constexpr double (\w+) = (0x[0-9a-fA-F.]+p[-+]\d+);", text))
    ln2 = mpmath.log(2)
    assert float.fromhex(consts["LN2"]) == float(ln2)
    assert float.fromhex(consts["LN2_LO"]) == float(ln2 - mpmath.mpf(float(ln2)))
    assert float.fromhex(consts["INV_LN2_64"]) == float(64 / ln2)
    hi = float.fromhex(consts["LN2_64_HI"])
    assert hi == float(ln2 / 64)
    assert float.fromhex(consts["LN2_64_LO"]) == float(ln2 / 64 - mpmath.mpf(hi))
