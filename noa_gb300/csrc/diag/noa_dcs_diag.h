/*
 * libnoa_dcs_diag.so -- test and benchmark instruments of the muon DCS
 * library.  Not part of the drop-in surface (include/noa_dcs.h) and not
 * linked into libnoa_dcs.so; no counterpart in the reference.  Status codes
 * are those of noa_dcs.h.
 */
#ifndef NOA_DCS_DIAG_H
#define NOA_DCS_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic-throughput probe: launches `blocks` x 256 threads of independent
 * FMA chains in FP64 (fp64 != 0) or FP32 on `stream`, writing one value per
 * thread to the device buffer `out`, and stores the launch's flop count in
 * *flops.  Timing it gives the measured FP64 / FP32 pipe peaks that the DCS
 * kernels' rooflines are quoted against. */
int noa_dcs_probe_fma(int fp64, void *out, int blocks, int iters, double *flops, void *stream);

/* out[i] = f(x[i]) (or f(x[i], y[i])) for one of the DCS library's FP64
 * elementary functions -- fn 0 log, 1 exp, 2 reciprocal, 3 division x/y,
 * 4 sqrt -- of its integer-pipe conversions -- fn 5 (double)(float)x,
 * 6 (double)(int)x for x in int range -- or of its float-float functions on x
 * split into a float pair -- fn 7 exp (-87 < x < 88), 8 log (x > 0, normal
 * float range) -- or fn 9 the normal-range conversion (double)(float)x, NaN
 * outside the normal float range, on device buffers, so that their error can
 * be measured against a reference libm and the conversions checked against
 * the casts. */
int noa_dcs_lean64_eval(int fn, const double *x, const double *y, double *out, int64_t n, void *stream);

/* out[i] for the pair (K[i], q[i]) of process proc (0 bremsstrahlung, 1 pair
 * production, 2 photonuclear, 3 ionisation) on element (A, I, Z) and mass: the
 * decision the DCS kernels take first in float or lean arithmetic --
 * bremsstrahlung's electron term (q < qe_max), pair production's and
 * photonuclear's open / closed, ionisation's first exit -- as 1 or 0 when it
 * equals the reference's exact IEEE decision, -2 when it does not, and -1
 * where ionisation's float test leaves the decision to the exact one.
 * Device buffers; enqueued on `stream`. */
int noa_dcs_decision_check(int proc, const double *K, const double *q, double *out, int64_t n, double A, double I,
                           int32_t Z, double mass, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NOA_DCS_DIAG_H */
