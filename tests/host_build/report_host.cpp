// The GB300 backend binding's transition report, exported for a test
// (test infrastructure only): GpuPr76PtFlashBackend::transition_report of
// mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp for a published status and
// max3 status, encoded as ref_transition_reports encodes the reference's
// (oracle/ref_harness.cpp).  Compiled against the reference's flash headers;
// no C ABI call is made, so nothing is linked.
#include "gpu_pr76_pt_flash_backend.hpp"

extern "C" int our_transition_report(int32_t status, int32_t max3_status, int32_t* evidence) {
    const auto report = mpmc::flash::GpuPr76PtFlashBackend::transition_report(status, max3_status);
    const int count = static_cast<int>(std::min<std::size_t>(report.evidence.size(), 8));
    for (int k = 0; k < count; ++k) {
        const auto& e = report.evidence[k];
        int32_t* row = evidence + k * 6;
        row[0] = static_cast<int32_t>(e.source_phase_count);
        row[1] = e.target_phase_count ? static_cast<int32_t>(*e.target_phase_count) : 0;
        row[2] = static_cast<int32_t>(e.trigger);
        row[3] = static_cast<int32_t>(e.resolution);
        row[4] = e.fresh_target_solve_attempted ? 1 : 0;
        row[5] = e.target_topology_closed ? 1 : 0;
    }
    return count;
}
