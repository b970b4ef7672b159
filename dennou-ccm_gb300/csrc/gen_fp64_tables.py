"""Writes fp64_tables.cuh: the tables and constants of the flux kernel's
FP64 exp and log (fp64_fast.cuh), each value the double nearest to the
exact one (mpmath at 200 bits).  Run from this directory:
    python gen_fp64_tables.py > fp64_tables.cuh
"""
import mpmath

mpmath.mp.prec = 200


def d(v):
    return float(v).hex()


def main():
    ln2 = mpmath.log(2)
    hi = mpmath.mpf(float(ln2 / 64))
    lo = ln2 / 64 - hi
    out = ["// Generated by gen_fp64_tables.py: doubles nearest to the exact values.",
           "#pragma once", "", "namespace dccm {", "namespace fp64 {", "",
           f"constexpr double LN2 = {d(ln2)};  // ln 2 = LN2 + LN2_LO",
           f"constexpr double LN2_LO = {d(ln2 - mpmath.mpf(float(ln2)))};",
           f"constexpr double INV_LN2_64 = {d(64 / ln2)};  // 64 / ln 2",
           f"constexpr double LN2_64_HI = {d(hi)};  // ln 2 / 64 = HI + LO",
           f"constexpr double LN2_64_LO = {d(lo)};", "",
           "// 2^(j / 64), j = 0 .. 63",
           "__device__ const double EXP2_64[64] = {"]
    out += [f"    {d(mpmath.power(2, mpmath.mpf(j) / 64))}," for j in range(64)]
    out += ["};", "",
            "// {1 / F, ln F} for F = 1 + j / 128, j = 0 .. 128, and the rest of ln F",
            "__device__ const double2 LOG_F128[129] = {"]
    lo = []
    for j in range(129):
        F = 1 + mpmath.mpf(j) / 128
        out.append(f"    {{{d(1 / F)}, {d(mpmath.log(F))}}},")
        lo.append(f"    {d(mpmath.log(F) - mpmath.mpf(float(mpmath.log(F))))},")
    out += ["};", "__device__ const double LOG_F128_LO[129] = {"] + lo
    out += ["};", "", "}  // namespace fp64", "}  // namespace dccm", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
