// The C++ continuation binding (mpmc_hnu_gb300/cpp/gpu_pr76_pt_continuation.hpp)
// run on the CPU (test infrastructure only): the three C-ABI functions it
// calls are provided here by the host build of the device code
// (flash_host.cpp, linked beside this file).  Reads the paths from a binary
// file (npath, npoint, then p, t [npath * npoint] and z [3 * npath]) of the
// three-component fixture mixture and prints each point's max3 status and
// each path's brackets, for tests/test_continuation_hints.py.
#include "gpu_pr76_pt_continuation.hpp"

#include <cstdio>

extern "C" int host_hinted_batch(int n, const double* tc, const double* pc, const double* omega, const double* kij,
                                 int64_t ncell, const double* p, const double* t, const double* z,
                                 const int32_t* hint_count, const double* hint_x, const int32_t* three,
                                 const double* fraction, int32_t* published, int32_t* max3, double* x, double* y,
                                 double* x3, double* f3);

struct mpmc_gpu_flash {
    int n;
    std::vector<double> tc, pc, omega, kij;
};

extern "C" {
int mpmc_gpu_flash_components(const mpmc_gpu_flash* h) { return h ? h->n : 0; }
const char* mpmc_gpu_flash_last_error(void) { return "host build"; }
int mpmc_gpu_flash_solve_hinted(mpmc_gpu_flash* h, int64_t ncell, const double* p, const double* t, const double* z,
                                const mpmc_start_hints* hints, const mpmc_flash_outputs* out,
                                const mpmc_three_phase_outputs* out3) {
    return host_hinted_batch(h->n, h->tc.data(), h->pc.data(), h->omega.data(), h->kij.data(), ncell, p, t, z,
                             hints->count, hints->composition, hints->three_phase, hints->fraction, out->status,
                             out3->max3_status, out->liquid, out->vapor, out3->composition, out3->phase_fraction);
}
}

int main(int argc, char** argv) {
    if (argc != 2) return 1;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 1;
    int64_t dims[2];
    if (std::fread(dims, 8, 2, f) != 2) return 1;
    const int64_t npath = dims[0], npoint = dims[1];
    std::vector<double> p(npath * npoint), t(npath * npoint), z(3 * npath);
    if (std::fread(p.data(), 8, p.size(), f) != p.size() || std::fread(t.data(), 8, t.size(), f) != t.size() ||
        std::fread(z.data(), 8, z.size(), f) != z.size())
        return 1;
    std::fclose(f);
    // the three-phase fixture mixture of the reference's tests
    mpmc_gpu_flash h{3, {190.6, 500.0, 500.0}, {4.6e6, 5.0e6, 5.0e6}, {0.01, 0.10, 0.10},
                     {0.0, 0.05, 0.05, 0.05, 0.0, 0.20, 0.05, 0.20, 0.0}};
    std::vector<std::vector<mpmc::flash::Pr76PtPathState>> paths(npath);
    std::vector<std::vector<double>> feeds(npath);
    for (int64_t k = 0; k < npath; ++k) {
        for (int64_t j = 0; j < npoint; ++j) paths[k].push_back({p[k * npoint + j], t[k * npoint + j]});
        for (int i = 0; i < 3; ++i) feeds[k].push_back(z[i * npath + k]);
    }
    const auto res = mpmc::flash::solve_gpu_pr76_pt_continuation(&h, paths, feeds);
    for (const auto& r : res) {
        for (const auto& pt : r.points) std::printf("%d ", static_cast<int>(pt.status));
        std::printf("| %zu", r.transition_brackets.size());
        for (const auto& b : r.transition_brackets) std::printf(" %zu-%zu", b.left_index, b.right_index);
        std::printf("\n");
    }
    return 0;
}
