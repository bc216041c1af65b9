/*
 * FP64-accurate elementary functions that issue few FP64 instructions.
 *
 * On GB300 the FP64 pipe retires 2 lanes per clock per SM: one FP64 warp
 * instruction occupies it for 16 clocks, while the SM issues 4 warp
 * instructions per clock to its integer (ALU, 64 lanes) and FP32 (128 lanes)
 * pipes.  A DCS kernel built on FP64 arithmetic is therefore bound by its
 * FP64 instruction count with issue ~80% idle (ncu: FP64 pipe 86%, issue
 * 12%), and replacing one FP64 instruction by up to ~30 integer or FP32
 * instructions still shortens it.  The functions here keep double accuracy
 * (about 1 ulp; tests compare them with CUDA's functions and numpy) and do
 * their work in exact 64-bit integer arithmetic (range reduction, products
 * with short table constants, fixed-point sums rounded once to double) and
 * in float-float arithmetic (the small correction terms, which need 2^-47
 * relative), leaving FP64 only where a double is the natural operand:
 *
 *   lean_log   1 FP64 op.  Tang's table method (P. T. P. Tang, ACM TOMS
 *              16(4), 1990): x = 2^e m, c_t = C_t / 2^10 ~ 1/m from the top
 *              8 mantissa bits; r = m c_t - 1 exact in 64-bit integers;
 *              log x = e ln2 + [-log c_t + r + (log1p(r) - r)], the bracket
 *              a fixed-point sum at the bin's scale, the final e ln2 one
 *              FMA.  The two bins next to 1 use c_t = 1 with a scale that
 *              follows r: full relative accuracy near 1.
 *   lean_exp   2 FP64 ops.  Tang's table method (ACM TOMS 15(2), 1989):
 *              k = round(x 128 / ln2), r = x - k hi (one exact FMA), the
 *              rest of exp(r) - 1 in float-float and a fixed-point sum;
 *              exp x = 2^k' fma(T_j, p, T_j), 2^k' added to the exponent.
 *   lean_rcp   0 FP64 ops.  MUFU seed, exact float-float residual 1 - m y0
 *              on the mantissa split into three floats, y0 (1 + e + e^2)
 *              summed in fixed point and rounded once.
 *   lean_div   1 FP64 op: a * lean_rcp(b).
 *   lean_sqrt  6 FP64 ops.  MUFU rsqrt, then two Newton steps on s = x y.
 *
 * Arguments outside the fast range (zero, negative, subnormal, |x| > 700
 * for exp, |b| >= 2^1022 for rcp, values outside float range for sqrt,
 * inf, NaN) take CUDA's IEEE function, so special values behave exactly as
 * in IEEE arithmetic.  The double <-> float and int -> double conversions go
 * through the integer pipe (fpconv.cuh), because the hardware conversions
 * would occupy the FP64 pipe too.
 */
#pragma once

#include "fpconv.cuh"
#include "lean64_tables.h"

#include <cstring>

#include <cuda_runtime.h>

namespace lean64 {

#ifndef LEAN64_FN
#define LEAN64_FN __device__ __forceinline__
#endif

LEAN64_FN float rcp_approx(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    // host builds: a stand-in seed 1 - 3 ulp off the rounded 1/x, as far off
    // as the MUFU approximation may be, so that host checks cover that error
    float r = 1.f / x;
    unsigned u;
    memcpy(&u, &r, 4);
    u ^= 3u;
    memcpy(&r, &u, 4);
    return r;
#endif
}

__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// x >= 0 finite double compared with a positive constant through the bit
// pattern (integer pipe); NaN compares as larger than every constant.
__device__ __forceinline__ bool bits_ge(double x, double c) {
    return __double_as_longlong(x) >= __double_as_longlong(c);
}

// ------------------------------------------------------------ lean_log / lean_exp
// Host builds of lean_log / lean_exp / lean_rcp (for checking them on a CPU)
// define LEAN64_FN as __host__ __device__ and LEAN64_HOST_TABLES before
// including this header; the product builds them for the device only.

#if defined(LEAN64_HOST_TABLES) && !defined(__CUDA_ARCH__)
static const longlong2 lean64_log_tab_host[1 << LEAN64_LOG_BITS] = LEAN64_LOG_TAB_DATA;
static const double lean64_exp_t_host[LEAN64_EXP_N] = LEAN64_EXP_TAB_DATA;
#endif

namespace detail {

#if defined(__CUDA_ARCH__) || !defined(LEAN64_HOST_TABLES)
__device__ __forceinline__ long long d2ll(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double ll2d(long long b) { return __longlong_as_double(b); }
__device__ __forceinline__ unsigned f2u(float x) { return __float_as_uint(x); }
__device__ __forceinline__ float u2f(unsigned b) { return __uint_as_float(b); }
__device__ __forceinline__ int clz64(unsigned long long x) { return __clzll((long long)x); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ int f2i_rn(float x) { return __float2int_rn(x); }
__device__ __forceinline__ longlong2 log_entry(int t) { return __ldg(&lean64_log_tab[t]); }
__device__ __forceinline__ double exp_entry(int j) { return __ldg(&lean64_exp_t[j]); }
#elif defined(LEAN64_HOST_TABLES)
inline long long d2ll(double x) { long long b; memcpy(&b, &x, 8); return b; }
inline double ll2d(long long b) { double x; memcpy(&x, &b, 8); return x; }
inline unsigned f2u(float x) { unsigned b; memcpy(&b, &x, 4); return b; }
inline float u2f(unsigned b) { float x; memcpy(&x, &b, 4); return x; }
inline int clz64(unsigned long long x) { return __builtin_clzll(x); }
inline float fadd(float a, float b) { return a + b; }  // host code is built with -ffp-contract=off
inline float fmul(float a, float b) { return a * b; }
inline int f2i_rn(float x) { return (int)nearbyintf(x); }
inline longlong2 log_entry(int t) { return lean64_log_tab_host[t]; }
inline double exp_entry(int j) { return lean64_exp_t_host[j]; }
#endif

// f 2^F as a signed 64-bit integer, truncated toward zero; 0 for zero and
// float subnormals.  Callers keep |f| 2^F below 2^55 (a left shift <= 31).
LEAN64_FN long long fix_from_float(float f, int F) {
    const unsigned u = f2u(f);
    const unsigned ef = (u >> 23) & 0xFFu;
    // the significand (implicit bit set) at bits 40..63: the float's
    // exponent and sign bits fall off the top of the word
    const unsigned long long m = (unsigned long long)(u | 0x800000u) << 40;
    const int t = 190 - (int)ef - F;  // bit 0 of the significand weighs 2^(ef - 150); t >= 9
    const unsigned long long v = (ef != 0u && t < 64) ? (m >> t) : 0ull;
    return (u >> 31) ? -(long long)v : (long long)v;
}

// S 2^-F as a double, rounded to nearest even; S != 0, 1 <= 1086 - F - clz.
LEAN64_FN double fix_to_double(long long S, int F) {
    const unsigned long long sign = (unsigned long long)S & 0x8000000000000000ull;
    const unsigned long long U = S < 0 ? 0ull - (unsigned long long)S : (unsigned long long)S;
    const int lz = clz64(U);
    const unsigned long long N = U << lz;  // leading bit at 63
    unsigned long long m = N >> 11;        // 53 bits, leading bit at 52
    const unsigned long long rest = N & 0x7FFull;
    m += (rest > 0x400ull || (rest == 0x400ull && (m & 1ull))) ? 1ull : 0ull;
    // biased exponent 1086 - lz - F; the leading bit of m adds the last 1
    // (and a carry out of rounding moves to the next binade by itself)
    return ll2d((long long)(sign | (((unsigned long long)(1085 - lz - F) << 52) + m)));
}

} // namespace detail

// log x with one FP64 instruction.  x = 2^e m, m in [0.707, 1.414) (bin t of
// the top 8 mantissa bits, halved above sqrt 2), c = C_t / 2^10 ~ 1/m:
//   r = m c - 1 = R 2^-(62+h)      exact, one 64-bit integer multiply
//   d = log1p(r) - r               float-float, ~2^-47 relative
//   T = -log c + r + d             64-bit fixed point at the bin's scale
//                                  2^-F_t, rounded once to double
//   log x = fma(e, ln2, T)         the one FP64 instruction
// |T| <= 0.347 < ln2 / 2, so the fma never cancels; in the two bins next to
// 1 the scale follows r (log x = r + d there), so log x keeps full relative
// accuracy at x = 1 +- 2^-53.
LEAN64_FN double lean_log(double x) {
    using namespace detail;
    const long long b = d2ll(x);
    // positive, normal and finite?
    if ((unsigned long long)(b - 0x0010000000000000LL) >= 0x7FE0000000000000ULL)
        return log(x);
    const int hi = (int)(b >> 32);
    const int t = (hi >> 12) & 0xFF;
    const int h = t >= LEAN64_LOG_SPLIT ? 1 : 0;
    const int e = (hi >> 20) - 1023 + h;
    const unsigned long long M = ((unsigned long long)b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
    const longlong2 ent = log_entry(t);  // {C_t | F_t << 32, L_t}, one 16-byte load
    const unsigned long long C = (unsigned long long)ent.x & 0xFFFFull;
    const int Ft = (int)(ent.x >> 32);
    const long long R = (long long)(M * C - (1ull << (62 + h)));
    if (R == 0)  // m = 1: x = 2^e
        return fpconv::f64i(e) * LEAN64_LN2;
    const unsigned long long A = R < 0 ? 0ull - (unsigned long long)R : (unsigned long long)R;
    const int lz = clz64(A);              // 8 <= lz <= 63
    const unsigned long long N = A << lz;  // |r| = N 2^-(62+h+lz), N in [2^63, 2^64)
    // r = rh + rl: the top 24 bits of N exactly, then the next 23
    const unsigned sgn = R < 0 ? 0x80000000u : 0u;
    const float rh = u2f(sgn | ((unsigned)(128 - h - lz) << 23) | ((unsigned)(N >> 40) & 0x7FFFFFu));
    const float v = fadd(u2f(0x4B000000u | ((unsigned)(N >> 17) & 0x7FFFFFu)), -8388608.f);  // exact
    const float rl = fmul(u2f(sgn | ((unsigned)(82 - h - lz) << 23)), v);                   // +- v 2^(-45-h-lz)
    // d = -r^2/2 + r^3 w,  w = 1/3 - r/4 + r^2 (1/5 - r/6 + r^2/7)
    const float sh = fmul(rh, rh);
    const float sl = fmaf(fmul(2.f, rh), rl, fmaf(rh, rh, -sh));
    const float zt = fmul(sh, fmaf(rh, fmaf(rh, 1.f / 7.f, -1.f / 6.f), 0.2f));
    const float qa = fmul(-0.25f, rh);
    const float zh = fadd(qa, zt);
    const float zl = fmaf(-0.25f, rl, fadd(zt, -fadd(zh, -qa)));
    const float wh = fadd(LEAN64_THIRD_H, zh);
    const float wl = fadd(fadd(zh, -fadd(wh, -LEAN64_THIRD_H)), fadd(zl, LEAN64_THIRD_L));
    const float ch = fmul(sh, rh);
    const float cl = fmaf(sh, rl, fmaf(sl, rh, fmaf(sh, rh, -ch)));
    const float uh = fmul(ch, wh);
    const float ul = fmaf(ch, wl, fmaf(cl, wh, fmaf(ch, wh, -uh)));
    const float hs = fmul(-0.5f, sh);
    const float dh = fadd(hs, uh);
    const float dl = fadd(fadd(uh, -fadd(dh, -hs)), fmaf(-0.5f, sl, ul));
    // T = L_t + r + d in units of 2^-F
    const int F = Ft != 0 ? Ft : 60 + h + lz;
    const long long Sr = (long long)(A << (F - 62 - h));  // shift 1..7, or lz - 2 at 1
    const long long S = ent.y + (R < 0 ? -Sr : Sr) + fix_from_float(dh, F) + fix_from_float(dl, F);
    return fma(fpconv::f64i(e), LEAN64_LN2, fix_to_double(S, F));
}

// exp x with two FP64 instructions.  k = round(x 128 / ln2), 2^(k/128) =
// 2^k' T_j:
//   r = x - k hi                   exact (hi has 32 bits), the first FMA
//   rt = r - k lo                  float-float (the reduced argument)
//   d = expm1(rt) - rt             float-float, ~2^-47 relative
//   p = r + (d - k lo)             64-bit fixed point, 2^-70, rounded once
//   exp x = 2^k' fma(T_j, p, T_j)  the second FMA; 2^k' on the exponent bits
LEAN64_FN double lean_exp(double x) {
    using namespace detail;
    if ((d2ll(x) & 0x7FFFFFFFFFFFFFFFLL) >= 0x4085E00000000000LL)  // |x| >= 700, inf, NaN
        return exp(x);
    const int k = f2i_rn(fmul(fpconv::f32(x), (float)LEAN64_INV_LN2N));
    const double r = fma(-fpconv::f64i(k), LEAN64_LN2N_HI, x);
    const unsigned long long br = (unsigned long long)d2ll(r);
    const unsigned er = (unsigned)(br >> 52) & 0x7FFu;
    const unsigned rs = (unsigned)(br >> 32) & 0x80000000u;
    // r = rh + rl to 2^-47 (the top 24 bits, then 23); zero below 2^-80,
    // where r only enters linearly
    const bool big = er >= 943u;
    const float rh = big ? u2f(rs | ((er - 896u) << 23) | ((unsigned)(br >> 29) & 0x7FFFFFu)) : 0.f;
    const float rv = fadd(u2f(0x4B000000u | ((unsigned)(br >> 6) & 0x7FFFFFu)), -8388608.f);
    const float rl = big ? fmul(u2f(rs | ((er - 942u) << 23)), rv) : 0.f;
    // k lo and rt = r - k lo
    const float kf = fadd(u2f(0x4B400000u + (unsigned)k), -12582912.f);  // exact, |k| < 2^22
    const float kh = fmul(kf, LEAN64_LN2N_LO_H);
    const float kl = fmaf(kf, LEAN64_LN2N_LO_L, fmaf(kf, LEAN64_LN2N_LO_H, -kh));
    const float th = fadd(rh, -kh);
    const float tb = fadd(th, -rh);
    const float te = fadd(fadd(rh, -fadd(th, -tb)), fadd(-kh, -tb));
    const float tl = fadd(te, fadd(rl, -kl));
    // d = rt^2 (1/2 + rt w),  w = 1/6 + rt (1/24 + rt (1/120 + rt/720))
    const float sh = fmul(th, th);
    const float sl = fmaf(fmul(2.f, th), tl, fmaf(th, th, -sh));
    const float g = fmul(th, fmaf(th, fmaf(th, 1.f / 720.f, 1.f / 120.f), 1.f / 24.f));
    const float wh = fadd(LEAN64_SIXTH_H, g);
    const float wl = fadd(fadd(g, -fadd(wh, -LEAN64_SIXTH_H)), LEAN64_SIXTH_L);
    const float vh = fmul(th, wh);
    const float vl = fmaf(th, wl, fmaf(tl, wh, fmaf(th, wh, -vh)));
    const float qh = fadd(0.5f, vh);
    const float ql = fadd(fadd(vh, -fadd(qh, -0.5f)), vl);
    const float dh = fmul(sh, qh);
    const float dl = fmaf(sh, ql, fmaf(sl, qh, fmaf(sh, qh, -dh)));
    // p = r + d - k lo in units of 2^-70
    const unsigned long long Mr = (br & 0x000FFFFFFFFFFFFFull) | (er ? 0x0010000000000000ull : 0ull);
    const int shr = 1005 - (int)(er ? er : 1u);  // the weight of bit 0 of Mr is 2^(er - 1075)
    const long long Pr = (long long)(shr <= 0 ? Mr << (-shr < 10 ? -shr : 10) : Mr >> (shr > 63 ? 63 : shr));
    // d - k lo as one float pair (two-sum), then into the fixed-point sum
    const float xs = fadd(dh, -kh);
    const float xb = fadd(xs, -dh);
    const float xl = fadd(fadd(fadd(dh, -fadd(xs, -xb)), fadd(-kh, -xb)), fadd(dl, -kl));
    const long long S = (rs ? -Pr : Pr) + fix_from_float(xs, 70) + fix_from_float(xl, 70);
    const double p = S == 0 ? 0.0 : fix_to_double(S, 70);
    const double tj = exp_entry(k & (LEAN64_EXP_N - 1));
    const double y = fma(tj, p, tj);
    return ll2d((long long)((unsigned long long)d2ll(y) + ((unsigned long long)(long long)(k >> 7) << 52)));
}

// 1/b with no FP64 instruction.  b = +-2^E m, m in [1, 2) split exactly into
// floats m1 + m2 + m3 (24 + 23 + 6 bits); y0 = MUFU rcp(m1) ~ 1/m to 2^-22;
// the residual e = 1 - m y0 in float-float (exact products by FMA, 1 - m1 y0
// exact by Sterbenz); 1/m = y0 (1 + e + e^2) to ~2^-64, summed in 64-bit fixed
// point (2^-62) and rounded once; 2^-E and the sign go on the bits.  Zero,
// subnormal, |b| >= 2^1022 (a subnormal result), inf and NaN take IEEE 1/b.
// a / b is a * lean_rcp(b): one FP64 multiply.
LEAN64_FN double lean_rcp(double b) {
    using namespace detail;
    const unsigned long long bb = (unsigned long long)d2ll(b);
    const unsigned eb = (unsigned)(bb >> 52) & 0x7FFu;
    if (eb - 1u >= 2044u)
        return 1.0 / b;
    const unsigned long long M = bb & 0x000FFFFFFFFFFFFFull;
    const float m1 = u2f((127u << 23) | (unsigned)(M >> 29));                                     // [1, 2)
    const float m2 = fmul(fadd(u2f(0x4B000000u | ((unsigned)(M >> 6) & 0x7FFFFFu)), -8388608.f), 0x1p-46f);
    const float m3 = fmul(fadd(u2f(0x4B000000u | ((unsigned)M & 0x3Fu)), -8388608.f), 0x1p-52f);
    const float y0 = rcp_approx(m1);
    const float p1 = fmul(m1, y0);
    const float p1e = fmaf(m1, y0, -p1);
    const float a = fadd(1.f, -p1);  // exact
    const float p2 = fmul(m2, y0);
    const float p2e = fmaf(m2, y0, -p2);
    // e = a - p1e - p2 - (p2e + m3 y0), |e| < 2^-21
    const float s1 = fadd(a, -p1e);
    const float s1b = fadd(s1, -a);
    const float s1e = fadd(fadd(a, -fadd(s1, -s1b)), fadd(-p1e, -s1b));
    const float eh = fadd(s1, -p2);
    const float eb2 = fadd(eh, -s1);
    const float e1 = fadd(fadd(s1, -fadd(eh, -eb2)), fadd(-p2, -eb2));
    const float el = fadd(fadd(e1, s1e), -fmaf(m3, y0, p2e));
    // y0 (e + e^2) as a float pair
    const float ch = fmul(y0, eh);
    const float cl = fmaf(y0, fmaf(eh, eh, el), fmaf(y0, eh, -ch));
    const long long S = fix_from_float(y0, 62) + fix_from_float(ch, 62) + fix_from_float(cl, 62);
    const double ym = fix_to_double(S, 62);  // 1/m in (0.5, 1]
    return ll2d((long long)(((unsigned long long)d2ll(ym) - ((unsigned long long)(long long)((int)eb - 1023) << 52)) |
                            (bb & 0x8000000000000000ull)));
}

LEAN64_FN double lean_div(double a, double b) { return a * lean_rcp(b); }

__device__ __forceinline__ double lean_sqrt(double x) {
    const float xf = fpconv::f32(x);
    if (!(xf >= 2e-38f && xf <= 1e38f))
        return sqrt(x);
    const double y = fpconv::f64(rsqrt_approx(xf));
    const double h = 0.5 * y;
    double s = x * y;
    double r = fma(-s, s, x);
    s = fma(r, h, s);
    r = fma(-s, s, x);
    return fma(r, h, s);
}

} // namespace lean64
