/*
 * Thin C wrapper around the UNMODIFIED reference header src/noa/pms/dcs.hh of
 * grinisrit/noa -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiled by oracle/build_ref.sh against the reference sources where they
 * lie (include path <noa checkout>/src) and the pip LibTorch, into
 * oracle/_ref/libnoa_ref_dcs.so.  It calls the reference's own dcs::vmap /
 * dcs::pvmap (dcs.hh:35-75) and dcs::vmap_integral(dcs::recoil_integral(...))
 * (dcs.hh:89-130), the elastic-scattering functions coulomb_data,
 * coulomb_transport and hard_scattering (dcs.hh:604-872) and soft_scattering
 * (dcs.hh:941-952) on tensors that wrap the caller's buffers, so the golden
 * vectors under tests/golden come from the reference code path itself.
 */
#include <noa/pms/dcs.hh>
#include <noa/pms/physics.hh>

#include <torch/torch.h>

#include <cstdint>
#include <vector>

using namespace noa::pms;

namespace {

torch::Tensor wrap(const double *p, int64_t n) {
    return torch::from_blob(const_cast<double *>(p), {n}, torch::TensorOptions().dtype(torch::kFloat64));
}

template <typename F>
void run_map(const F &f, bool parallel, const double *K, const double *q, double *out, int64_t n,
             const AtomicElement &el, double mass) {
    auto tk = wrap(K, n), tq = wrap(q, n), tr = wrap(out, n);
    if (parallel)
        dcs::pvmap(f)(tr, tk, tq, el, mass);
    else
        dcs::vmap(f)(tr, tk, tq, el, mass);
}

template <typename F, typename G>
void run_integral(const F &f, const G &g, const double *K, double *out, int64_t n, double xlow,
                  const AtomicElement &el, double mass, int32_t min_points) {
    auto tk = wrap(K, n), tr = wrap(out, n);
    dcs::vmap_integral(dcs::recoil_integral(f, g))(tr, tk, xlow, el, mass, min_points);
}

} // namespace

extern "C" {

int ref_dcs_vmap(int process, int parallel, const double *K, const double *q, double *out, int64_t n, double A,
                 double I, int32_t Z, double mass) {
    const AtomicElement el{A, I, Z};
    switch (process) {
    case 0:
        run_map(dcs::bremsstrahlung, parallel, K, q, out, n, el, mass);
        return 0;
    case 1:
        run_map(dcs::pair_production, parallel, K, q, out, n, el, mass);
        return 0;
    case 2:
        run_map(dcs::photonuclear, parallel, K, q, out, n, el, mass);
        return 0;
    case 3:
        run_map(dcs::ionisation, parallel, K, q, out, n, el, mass);
        return 0;
    default:
        return -1;
    }
}

int ref_recoil_integral_vmap(int process, int moment, const double *K, double *out, int64_t n, double xlow, double A,
                             double I, int32_t Z, double mass, int32_t min_points) {
    const AtomicElement el{A, I, Z};
    const bool del = (moment == 0);
    switch (process) {
    case 0:
        del ? run_integral(dcs::bremsstrahlung, dcs::del_integrand, K, out, n, xlow, el, mass, min_points)
            : run_integral(dcs::bremsstrahlung, dcs::cel_integrand, K, out, n, xlow, el, mass, min_points);
        return 0;
    case 1:
        del ? run_integral(dcs::pair_production, dcs::del_integrand, K, out, n, xlow, el, mass, min_points)
            : run_integral(dcs::pair_production, dcs::cel_integrand, K, out, n, xlow, el, mass, min_points);
        return 0;
    case 2:
        del ? run_integral(dcs::photonuclear, dcs::del_integrand, K, out, n, xlow, el, mass, min_points)
            : run_integral(dcs::photonuclear, dcs::cel_integrand, K, out, n, xlow, el, mass, min_points);
        return 0;
    case 3:
        del ? run_integral(dcs::ionisation, dcs::del_integrand, K, out, n, xlow, el, mass, min_points)
            : run_integral(dcs::ionisation, dcs::cel_integrand, K, out, n, xlow, el, mass, min_points);
        return 0;
    default:
        return -1;
    }
}

int ref_coulomb_data(const double *K, int64_t n, double A, double I, int32_t Z, double mass, double *fCM,
                     double *screen, double *fspin, double *invlambda) {
    const AtomicElement el{A, I, Z};
    auto o = torch::TensorOptions().dtype(torch::kFloat64);
    dcs::coulomb_data(torch::from_blob(fCM, {n, 2}, o), torch::from_blob(screen, {n, 9}, o), wrap(fspin, n),
                      wrap(invlambda, n), wrap(K, n), el, mass);
    return 0;
}

int ref_coulomb_transport(const double *screen, const double *fspin, const double *mu, int64_t n_mu, int64_t n,
                          double *coefs) {
    auto o = torch::TensorOptions().dtype(torch::kFloat64);
    auto tmu = n_mu == 1 ? torch::from_blob(const_cast<double *>(mu), {}, o) : wrap(mu, n);
    dcs::coulomb_transport(torch::from_blob(coefs, {n, 2}, o),
                           torch::from_blob(const_cast<double *>(screen), {n, 9}, o), wrap(fspin, n), tmu);
    return 0;
}

int ref_hard_scattering(const double *G, const double *fCM, const double *screen, const double *invlambda,
                        const double *fspin, int64_t nel, int64_t nkin, double *mu0, double *lb_h) {
    auto o = torch::TensorOptions().dtype(torch::kFloat64);
    auto blob = [&](const double *p, std::vector<int64_t> shape) {
        return torch::from_blob(const_cast<double *>(p), shape, o);
    };
    dcs::hard_scattering(wrap(mu0, nkin), wrap(lb_h, nkin), blob(G, {nel, nkin, 2}), blob(fCM, {nel, nkin, 2}),
                         blob(screen, {nel, nkin, 9}), blob(invlambda, {nel, nkin}), blob(fspin, {nel, nkin}));
    return 0;
}

int ref_soft_scattering(const double *K, double *out, int64_t n, double A, double I, int32_t Z, double mass) {
    const AtomicElement el{A, I, Z};
    dcs::soft_scattering(wrap(out, n), wrap(K, n), el, mass);
    return 0;
}
}

