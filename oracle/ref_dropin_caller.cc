/*
 * A program written against the REFERENCE's declarations -- the link-level
 * proof of the drop-in.  TEST INFRASTRUCTURE ONLY.
 *
 * It includes only the reference's own src/noa/pms/dcs.hh, whose
 * noa::pms::dcs::cuda namespace declares vmap_bremsstrahlung and
 * map_bremsstrahlung (dcs.hh:1004-1019), and calls them the way the
 * reference's CUDA benchmark and test do (benchmark/measure-dcs-calc-cuda.cc:
 * 10-30, test/unit/test-dcs-calc-cuda.cc:12-19).  oracle/build_ref.sh links it
 * with noa_gb300/libnoa_dcs_torch.so instead of compiling the reference's
 * dcs.cuh, with no header of this repository on the include path: the link
 * succeeds only if the library exports the reference's mangled names.
 *
 * Usage: ref_dropin_caller IN OUT
 *   IN:  int64 n, then n float64 K (GeV), then n float64 q (GeV)
 *   OUT: n float64 from vmap_bremsstrahlung (result tensor zero-filled first),
 *        then n float64 from map_bremsstrahlung; both for standard rock and
 *        the muon mass, computed on cuda:0.
 * Exit status 0 on success, 1 on a usage or I/O error, 2 on a c10::Error.
 */
#include <noa/pms/dcs.hh>

#include <torch/torch.h>

#include <cstdint>
#include <cstdio>
#include <vector>

int main(int argc, char **argv) {
    using namespace noa::pms;
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 1;
    }
    std::FILE *fin = std::fopen(argv[1], "rb");
    if (!fin)
        return 1;
    int64_t n = 0;
    if (std::fread(&n, sizeof n, 1, fin) != 1 || n < 0) {
        std::fclose(fin);
        return 1;
    }
    std::vector<double> K(static_cast<size_t>(n)), q(static_cast<size_t>(n));
    const bool ok = std::fread(K.data(), sizeof(double), K.size(), fin) == K.size() &&
                    std::fread(q.data(), sizeof(double), q.size(), fin) == q.size();
    std::fclose(fin);
    if (!ok)
        return 1;
    try {
        const auto cpu = torch::TensorOptions().dtype(torch::kFloat64);
        const auto kinetic = torch::from_blob(K.data(), {n}, cpu).to(torch::kCUDA);
        const auto recoil = torch::from_blob(q.data(), {n}, cpu).to(torch::kCUDA);
        const auto result = torch::zeros_like(kinetic);
        dcs::cuda::vmap_bremsstrahlung(result, kinetic, recoil, STANDARD_ROCK, MUON_MASS);
        const auto mapped = dcs::cuda::map_bremsstrahlung(kinetic, recoil, STANDARD_ROCK, MUON_MASS);
        const auto both = torch::cat({result, mapped}).to(torch::kCPU).contiguous();
        std::FILE *fout = std::fopen(argv[2], "wb");
        if (!fout)
            return 1;
        const size_t m = static_cast<size_t>(2 * n);
        const bool wrote = std::fwrite(both.data_ptr<double>(), sizeof(double), m, fout) == m;
        std::fclose(fout);
        return wrote ? 0 : 1;
    } catch (const c10::Error &e) {
        std::fprintf(stderr, "c10::Error: %s\n", e.what());
        return 2;
    }
}
