// Host build of the FP32C bodies and float-float primitives (noa_gb300/csrc/
// dcs_fp32c.cuh is written for host and device), for the CPU tests: the
// calibration of the error estimates against the oracle and the accuracy of
// ff_exp / ff_log.  Compiled by tests/test_fp32c_host.py.
#include "dcs_fp32c.cuh"

#include <cstdint>

using namespace noa_dcs;

// mode 0: the float form; mode 1 (pair production): the float-float
// screening-log form.  Closed pairs (the exact bounds) give 0 with est 0.
extern "C" int fp32c_host_eval(int proc, int mode, const double *K, const double *q, double *out, float *est,
                               int64_t n, double A, double I, int Z, double mass) {
    noa_dcs_consts c;
    noa_dcs_fill_consts(&c, A, I, Z, mass);
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) {
        float r = 0.f;
        double v = 0.;
        if (proc == 0) {
            v = brems_fp32c(K[i], q[i], c, r);
        } else if (proc == 1) {
            const double a = (q[i] <= 4. * ME || q[i] >= K[i] + c.pp_kmax_shift) ? 2.
                                                                                  : pprod_argmin_exact(K[i], q[i], c);
            if (!(a >= 1. || a <= 0.))
                v = mode ? pprod_fp32c<false, true>(K[i], q[i], c, r) : pprod_fp32c<false>(K[i], q[i], c, r);
        } else if (proc == 2) {
            double q2min, q2max;
            if (photo_window(K[i], q[i], c, q2min, q2max))
                v = photo_fp32c<false>(K[i], q[i], c, r);
        } else {
            v = ion_fp32c(K[i], q[i], c, r);
        }
        out[i] = v;
        est[i] = r;
    }
    return 0;
}

// fn 0: ff_exp, 1: ff_log, of x split into a float pair
extern "C" void ff_host_eval(int fn, const double *x, double *out, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        const FF a = ff_from(x[i]);
        const FF r = fn == 0 ? ff_exp(a) : ff_log(a);
        out[i] = (double)r.h + (double)r.l;
    }
}
