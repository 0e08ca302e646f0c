"""Generate boys_tables.cuh: the constant tables of the analytic ERI kernel's Boys function and
exponential, computed with mpmath at 40 significant digits and rounded once to double.

* Boys function F_n(T) = int_0^1 t^(2n) exp(-T t^2) dt = gamma(n+1/2, T) / (2 T^(n+1/2)).
* BOYS_HI: grid T_k = 1 + k/8 (k = 0..280, T in [1, 36]); row k holds a_j = F_j(T_k)/j!,
  j = 0..8, so that F_0(T_k + d) = sum_j a_j (-d)^j (Taylor series in d, |d| <= 1/16; the first
  omitted term is below 4e-17 relative because F_9 <= F_0).
* BOYS_LO: grid T_k = k/16 (k = 0..16, T in [0, 1]); row k holds F_n(T_k), n = 0..24; the
  kernel sums F_nf(T_k + d) = sum_{j<8} F_{nf+j}(T_k) (-d)^j / j! (|d| <= 1/32, first omitted
  term below 3e-17 relative).
* EXP2: 2^(j/32), j = 0..31, and the Cody-Waite split of ln2/32, for the table-driven
  exponential of P. T. P. Tang (ACM TOMS 15 (1989) 144-157).
* BOYS32 (single precision, for primitive quartets evaluated in FP32): grid T_k = k/8
  (k = 0..240, T in [0, 30]); row k holds F_n(T_k), n = 0..21, rounded to float; the kernel
  sums F_nf(T_k + d) = sum_{j<6} F_{nf+j}(T_k) (-d)^j / j! (|d| <= 1/16, first omitted term
  below 1e-10 relative) and recurs downwards; beyond T = 30 the asymptotic form is exact to
  e^-30.

Run: python slater_stoch_gb300/csrc/gen_boys_tables.py  (rewrites boys_tables.cuh beside it).
"""
from __future__ import annotations

from pathlib import Path

import mpmath as mp

mp.mp.dps = 40

HI_K, HI_H, HI_T0, HI_J = 281, mp.mpf(1) / 8, mp.mpf(1), 9
LO_K, LO_H, LO_N = 17, mp.mpf(1) / 16, 25
B32_K, B32_H, B32_N = 241, mp.mpf(1) / 8, 22


def boys(n: int, T) -> mp.mpf:
    if T == 0:
        return mp.mpf(1) / (2 * n + 1)
    return mp.gammainc(n + mp.mpf(1) / 2, 0, T) / (2 * T ** (n + mp.mpf(1) / 2))


def d(x) -> str:
    return repr(float(x))


def f32(x) -> str:
    import struct
    v = struct.unpack("f", struct.pack("f", float(x)))[0]  # rounded to float
    return repr(v) + "f"


def table(name: str, vals, per_line: int, ctype: str = "double") -> str:
    fmt = d if ctype == "double" else f32
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append("    " + ", ".join(fmt(v) for v in vals[i:i + per_line]) + ",")
    return f"SS_BOYS_TAB {ctype} {name}[{len(vals)}] = {{\n" + "\n".join(lines) + "\n};\n"


def main() -> None:
    hi = []
    for k in range(HI_K):
        T = HI_T0 + k * HI_H
        for j in range(HI_J):
            hi.append(boys(j, T) / mp.factorial(j))
    lo = []
    for k in range(LO_K):
        T = k * LO_H
        for n in range(LO_N):
            lo.append(boys(n, T))
    e2 = [mp.power(2, mp.mpf(j) / 32) for j in range(32)]
    b32 = []
    for k in range(B32_K):
        T = k * B32_H
        for n in range(B32_N):
            b32.append(boys(n, T))
    ln2_32 = mp.log(2) / 32
    hi_part = float(ln2_32)
    lo_part = float(ln2_32 - mp.mpf(hi_part))
    out = [
        "// boys_tables.cuh -- generated by gen_boys_tables.py (mpmath, 40 digits, rounded once to",
        "// double); do not edit by hand.",
        "#pragma once",
        "",
        "#ifdef __CUDACC__",
        "#define SS_BOYS_TAB __device__ const",
        "#else",
        "#define SS_BOYS_TAB static const",
        "#endif",
        "",
        "namespace ss {",
        "",
        f"constexpr int BOYS_HI_K = {HI_K};     // T_k = 1 + k/8",
        f"constexpr int BOYS_HI_J = {HI_J};       // a_j = F_j(T_k) / j!",
        f"constexpr int BOYS_LO_K = {LO_K};      // T_k = k/16",
        f"constexpr int BOYS_LO_N = {LO_N};      // F_n(T_k), n = 0..24",
        f"constexpr int BOYS32_K = {B32_K};     // T_k = k/8, T in [0, 30]",
        f"constexpr int BOYS32_N = {B32_N};      // F_n(T_k), n = 0..21 (float)",
        f"constexpr double EXP_INV_LN2_32 = {d(32 / mp.log(2))};  // 32/ln2",
        f"constexpr double EXP_LN2_32_HI = {d(hi_part)};  // ln2/32 = HI + LO",
        f"constexpr double EXP_LN2_32_LO = {d(lo_part)};",
        "",
        table("boys_hi_tab", hi, HI_J),
        table("boys_lo_tab", lo, 5),
        table("exp2_32_tab", e2, 4),
        table("boys32_tab", b32, 11, "float"),
        "}  // namespace ss",
        "",
    ]
    Path(__file__).with_name("boys_tables.cuh").write_text("\n".join(out))


if __name__ == "__main__":
    main()
