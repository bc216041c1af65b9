"""Generates lean64_tables.h: the lookup tables and constants of the
table-driven FP64 log and exp in lean64.cuh (table methods after
P. T. P. Tang, "Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990, and "... of the exponential
function ...", ACM TOMS 15(2), 1989).  Values are computed with mpmath at 60
digits and rounded once.

    python noa_gb300/csrc/gen_lean64_tables.py > noa_gb300/csrc/lean64_tables.h
"""
import struct

import mpmath

mpmath.mp.dps = 60

LOG_BITS = 8        # 256 bins over the top 8 mantissa bits
LOG_SPLIT = 106     # bins t >= 106 (m >= 1 + 106/256 > sqrt 2) are halved: m in [0.707, 1)
C_BITS = 10         # c_t = C_t / 2^10: m * c_t is exact in 64-bit integers
EXP_N = 128         # 2^(j/128)


def f32(x):
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def ff(x):
    """x as a float pair h + l (h = x rounded to float, l = the rest)."""
    h = f32(x)
    return h, f32(mpmath.mpf(x) - mpmath.mpf(h))


def log_tables():
    """Per bin t: (C_t, F_t, L_t).

    c_t = C_t / 2^10 is 1 / (bin centre) rounded to 10 fractional bits, so
    that r = m c_t - 1 is an exact 64-bit integer multiple of 2^-(62+h);
    |r| < 2^-8.7.  F_t is the number of fractional bits of the bin's
    fixed-point sum L_t + r + d = log m: the largest |log m| of the bin times
    2^F_t is at most 2^62.  L_t = -log(c_t) in units of 2^-F_t, rounded.
    The two bins that touch 1 use c_t = 1, L_t = 0 and F_t = 0 (a marker:
    their scale follows the size of r, so that log m = r + d keeps full
    relative accuracy down to m = 1 +- 2^-53).
    """
    rows = []
    one = 1 << C_BITS
    for t in range(1 << LOG_BITS):
        h = 1 if t >= LOG_SPLIT else 0
        lo = (1 + mpmath.mpf(t) / (1 << LOG_BITS)) / 2 ** h
        hi = (1 + mpmath.mpf(t + 1) / (1 << LOG_BITS)) / 2 ** h
        if t in (0, (1 << LOG_BITS) - 1):
            rows.append((one, 0, 0))
            continue
        C = int(mpmath.nint(one / ((lo + hi) / 2)))
        big = max(abs(mpmath.log(lo)), abs(mpmath.log(hi)))
        F = 62 - int(mpmath.ceil(mpmath.log(big, 2)))
        assert big * mpmath.mpf(2) ** F <= mpmath.mpf(2) ** 62
        assert F >= 62 + h  # the shift of r into the sum is never negative
        for m in (lo, hi):  # |r| stays below 2^-8.7 over the bin
            assert abs(m * C / one - 1) < mpmath.mpf(2) ** -8.7
        L = int(mpmath.nint(-mpmath.log(mpmath.mpf(C) / one) * mpmath.mpf(2) ** F))
        rows.append((C, F, L))
    return rows


def main():
    rows = log_tables()
    T = [float(mpmath.power(2, mpmath.mpf(j) / EXP_N)) for j in range(EXP_N)]
    ln2 = mpmath.log(2)
    ln2n = ln2 / EXP_N
    # hi part with 32 significant bits: k * hi is exact for |k| < 2^21
    e = int(mpmath.floor(mpmath.log(ln2n, 2)))
    hi = mpmath.floor(ln2n / mpmath.power(2, e - 31)) * mpmath.power(2, e - 31)
    lo = ln2n - hi
    lo_h, lo_l = ff(lo)
    third_h, third_l = ff(mpmath.mpf(1) / 3)
    sixth_h, sixth_l = ff(mpmath.mpf(1) / 6)
    out = []
    out.append("/* Generated by gen_lean64_tables.py -- do not edit. */")
    out.append("#pragma once")
    out.append(f"#define LEAN64_LOG_BITS {LOG_BITS}")
    out.append(f"#define LEAN64_LOG_SPLIT {LOG_SPLIT}")
    out.append(f"#define LEAN64_EXP_N {EXP_N}")
    out.append(f"#define LEAN64_LN2 {float(ln2)!r}")
    out.append(f"#define LEAN64_INV_LN2N {float(EXP_N / ln2)!r}")
    out.append(f"#define LEAN64_LN2N_HI {float(hi)!r}")
    out.append(f"#define LEAN64_LN2N_LO {float(lo)!r}")
    out.append(f"#define LEAN64_LN2N_LO_H {lo_h!r}f")
    out.append(f"#define LEAN64_LN2N_LO_L {lo_l!r}f")
    out.append(f"#define LEAN64_THIRD_H {third_h!r}f")
    out.append(f"#define LEAN64_THIRD_L {third_l!r}f")
    out.append(f"#define LEAN64_SIXTH_H {sixth_h!r}f")
    out.append(f"#define LEAN64_SIXTH_L {sixth_l!r}f")
    out.append("/* Per bin t, one 16-byte entry {C_t | F_t << 32, L_t}: the 10-bit")
    out.append("   reciprocal C_t / 2^10 of the bin centre, the number F_t of fractional")
    out.append("   bits of the bin's fixed-point sum (0: the two bins at 1, scaled by")
    out.append("   the size of r) and -log(C_t / 2^10) in units of 2^-F_t. */")
    out.append("#define LEAN64_LOG_TAB_DATA {\\")
    out.append(",\\\n".join("    {%dLL, %dLL}" % (C | (F << 32), L) for C, F, L in rows) + "}")
    out.append("static __device__ const longlong2 lean64_log_tab[%d] = LEAN64_LOG_TAB_DATA;" % len(rows))
    out.append("/* 2^(j/128) rounded to double. */")
    out.append("#define LEAN64_EXP_TAB_DATA {\\")
    out.append(",\\\n".join("    %s" % repr(v) for v in T) + "}")
    out.append("static __device__ const double lean64_exp_t[%d] = LEAN64_EXP_TAB_DATA;" % len(T))
    print("\n".join(out))


if __name__ == "__main__":
    main()
