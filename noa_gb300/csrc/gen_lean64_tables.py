"""Generates lean64_tables.h: the lookup tables of the table-driven FP64 log
and exp in lean64.cuh (methods after P. T. P. Tang, "Table-driven
implementation of the logarithm function in IEEE floating-point arithmetic",
ACM TOMS 16(4), 1990, and "... of the exponential function ...", ACM TOMS
15(2), 1989).  Values are computed with mpmath at 60 digits and rounded once.

    python noa_gb300/csrc/gen_lean64_tables.py > noa_gb300/csrc/lean64_tables.h
"""
import struct

import mpmath

mpmath.mp.dps = 60

LOG_BITS = 8        # 256 bins over the top 8 mantissa bits
LOG_SPLIT = 106     # bins t >= 106 (m >= 1 + 106/256 > sqrt 2) are halved: m in [0.707, 1)
EXP_N = 128         # 2^(j/128)


def f32(x):
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def log_tables():
    c, L = [], []
    for t in range(1 << LOG_BITS):
        if t in (0, (1 << LOG_BITS) - 1):
            ct = 1.0    # the bins that touch 1: r = m - 1 exactly, log exact near 1
        else:
            mt = 1 + (mpmath.mpf(t) + mpmath.mpf("0.5")) / (1 << LOG_BITS)
            if t >= LOG_SPLIT:
                mt /= 2
            ct = f32(1 / mt)
        c.append(ct)
        L.append(float(-mpmath.log(mpmath.mpf(ct))))
    return c, L


def main():
    c, L = log_tables()
    T = [float(mpmath.power(2, mpmath.mpf(j) / EXP_N)) for j in range(EXP_N)]
    ln2 = mpmath.log(2)
    ln2n = ln2 / EXP_N
    # hi part with 32 significant bits: k * hi is exact for |k| < 2^21
    e = int(mpmath.floor(mpmath.log(ln2n, 2)))
    hi = mpmath.floor(ln2n / mpmath.power(2, e - 31)) * mpmath.power(2, e - 31)
    lo = ln2n - hi
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
    out.append("/* Per bin t, {c_t, L_t}: c_t = 1/m_t rounded to float (1 for the two")
    out.append("   bins touching 1), stored as double so that no float -> double")
    out.append("   conversion is needed, and L_t = -log(c_t) rounded to double.  The")
    out.append("   pair is one 16-byte entry: a single load per logarithm. */")
    out.append("static __device__ const double2 lean64_log_cl[%d] = {" % len(c))
    out.append(",\n".join("    {%r, %s}" % (a, repr(b)) for a, b in zip(c, L)) + "};")
    out.append("/* 2^(j/128) rounded to double. */")
    out.append("static __device__ const double lean64_exp_t[%d] = {" % len(T))
    out.append(",\n".join("    %s" % repr(v) for v in T) + "};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
