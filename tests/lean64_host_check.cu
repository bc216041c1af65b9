// Host build of lean64's log, exp and reciprocal (the device source compiled
// for the CPU: integer and float operations give the same results there), run
// against long double libm.  Prints one line per input set:
//   <set> <count> <max ulp> <mean ulp>
// and one line per special value: special <fn> <x> <got> <expected>.
// Built and run by tests/test_lean64_host.py.  With arguments
// `values <in> <out>` it instead reads n doubles (raw) from <in> and writes
// lean_log(x) then lean_exp(x) for each (2n raw doubles) to <out>, for the
// device-equals-host test in tests/test_gpu_lean64.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#define LEAN64_FN __host__ __device__ __forceinline__
#define LEAN64_HOST_TABLES
#include "../noa_gb300/csrc/lean64.cuh"

namespace {

double ulp_of(double v) {
    int e;
    std::frexp(std::fabs(v), &e);
    return std::ldexp(1.0, e - 53);
}

struct Stat {
    const char *name;
    double max = 0, sum = 0;
    long n = 0;
    void add(double got, long double ref) {
        if (!std::isfinite((double)ref) || std::fabs((double)ref) < 0x1p-1000)
            return;  // outside the range the bars are stated for
        const double u = (double)(fabsl((long double)got - ref) / ulp_of((double)ref));
        max = u > max || std::isnan(u) ? u : max;
        sum += u;
        n++;
    }
    void print() const { std::printf("%s %ld %.6g %.6g\n", name, n, max, n ? sum / n : 0.0); }
};

double from_bits(uint64_t b) {
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}

} // namespace

int values(const char *in, const char *out) {
    FILE *f = std::fopen(in, "rb");
    if (!f)
        return 1;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f) / 8;
    std::fseek(f, 0, SEEK_SET);
    double *x = new double[n], *y = new double[2 * n];
    const long got = (long)std::fread(x, 8, n, f);
    std::fclose(f);
    if (got != n)
        return 1;
    for (long i = 0; i < n; i++) {
        y[i] = lean64::lean_log(x[i]);
        y[n + i] = lean64::lean_exp(x[i]);
    }
    FILE *o = std::fopen(out, "wb");
    if (!o)
        return 1;
    const long put = (long)std::fwrite(y, 8, 2 * n, o);
    std::fclose(o);
    delete[] x;
    delete[] y;
    return put == 2 * n ? 0 : 1;
}

int main(int argc, char **argv) {
    if (argc == 4 && std::strcmp(argv[1], "values") == 0)
        return values(argv[2], argv[3]);
    const long n = argc > 1 ? std::atol(argv[1]) : 200000;
    std::mt19937_64 g(20240613);
    std::uniform_real_distribution<double> U(0, 1);
    Stat log_bits{"log_random_bits"}, log_edges{"log_bin_edges"}, log_one{"log_near_one"}, log_split{"log_sqrt2_split"};
    Stat exp_wide{"exp_wide"}, exp_half{"exp_half_way"}, exp_small{"exp_small"};
    Stat rcp_bits{"rcp_random_bits"}, rcp_edges{"rcp_mantissa_edges"};
    for (long i = 0; i < n; i++) {
        const double xb = from_bits(g() & 0x7FFFFFFFFFFFFFFFull);
        if (xb > 0 && std::isfinite(xb))
            log_bits.add(lean64::lean_log(xb), logl((long double)xb));
        const int t = (int)(U(g) * 256), ex = (int)(U(g) * 2000) - 1000;
        const long long k = (long long)(U(g) * 64) - 32;
        const double xe = std::ldexp(1 + t / 256.0 + k * 0x1p-52, ex);
        log_edges.add(lean64::lean_log(xe), logl((long double)xe));
        const long long kk = (long long)(U(g) * 1e6) + 1;
        const double x1 = 1 + kk * 0x1p-52, x2 = 1 - kk * 0x1p-53;
        log_one.add(lean64::lean_log(x1), logl((long double)x1));
        log_one.add(lean64::lean_log(x2), logl((long double)x2));
        const double xs = std::ldexp(std::sqrt(2.0) + k * 0x1p-50, ex);
        log_split.add(lean64::lean_log(xs), logl((long double)xs));

        const double yw = U(g) * 1398 - 699;
        exp_wide.add(lean64::lean_exp(yw), expl((long double)yw));
        const long long kx = (long long)(U(g) * 258000) - 129000;
        const double yh = std::nextafter((kx + 0.5) * (0.6931471805599453 / 128), U(g) < 0.5 ? 0.0 : 1000.0);
        if (std::fabs(yh) < 700)
            exp_half.add(lean64::lean_exp(yh), expl((long double)yh));
        const double ys = (U(g) * 2 - 1) * std::pow(10.0, -(U(g) * 15));
        exp_small.add(lean64::lean_exp(ys), expl((long double)ys));

        const double zb = from_bits(g());
        if (std::isfinite(zb) && std::fabs(zb) > 0x1p-1021 && std::fabs(zb) < 0x1p1021)
            rcp_bits.add(lean64::lean_rcp(zb), 1.0L / (long double)zb);
        const double ze = std::ldexp((U(g) < 0.5 ? 1.0 : 2.0) + k * 0x1p-52, ex) * (U(g) < 0.5 ? -1 : 1);
        rcp_edges.add(lean64::lean_rcp(ze), 1.0L / (long double)ze);
    }
    for (const Stat *s : {&log_bits, &log_edges, &log_one, &log_split, &exp_wide, &exp_half, &exp_small, &rcp_bits,
                          &rcp_edges})
        s->print();
    const double lsp[] = {1.0, 2.0, 0.5, 0x1p-1022, 0x1.fffffffffffffp+1023, 0.0, -0.0, -1.0, INFINITY, NAN, 5e-324};
    for (double x : lsp)
        std::printf("special log %a %a %a\n", x, lean64::lean_log(x), std::log(x));
    const double esp[] = {0.0, -0.0, 1e-300, -1e-300, 5e-324, 700.0, 710.0, -745.0, -800.0, INFINITY, -INFINITY, NAN};
    for (double x : esp)
        std::printf("special exp %a %a %a\n", x, lean64::lean_exp(x), std::exp(x));
    const double rsp[] = {0.0, -0.0, 1.0, -1.0, 0.5, 4.0, 5e-324, 1e-310, 0x1p1022, 0x1p-1022, INFINITY, -INFINITY, NAN};
    for (double x : rsp)
        std::printf("special rcp %a %a %a\n", x, lean64::lean_rcp(x), 1.0 / x);
    return 0;
}
