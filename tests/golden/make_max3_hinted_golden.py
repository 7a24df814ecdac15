"""Record the reference's max-3-phase orchestration with caller starts and
split options (solve_pr76_pt_max3 with Pr76PtMax3Options and initial /
final starts, modules/flash/include/mpmc/flash/pr76_three_phase.hpp:328-341).

Runs only where the MPMC_HNU reference sources are present and the harness
oracle/_ref/libpr76_ref.so is built (`make -C oracle ref`).  The fixtures come
out of the reference tests themselves: a small C++ program that includes
tests/flash/pr76_three_phase/pr76_max3_robustness_test.cpp (its main renamed)
prints the parameters of its recovery_model() and of the synthetic fixture
model(), recovery_phases(), the fixture's equal_feed(), starts() and
reference_phases(); the metastable witness, a literal local to the test
function, is read from the test source.  Nothing is transcribed by hand.

Cases (one row each in tests/golden/max3_hinted_reference.npz):
  recovery   the test's 3 -> 2 recovery (pr76_max3_robustness_test.cpp:275-356):
             recovery model, 1 MPa, 250 K, feed 0.25 phase 0 + 0.75 phase 2,
             initial starts {witness}, final starts the three recovery phases,
             one three-phase start (the recovery phases, fraction seed
             {0, 0.75}), initial automatic starts off, 2 split attempts;
  three      the 3 -> 3 continuation base (:171-183): fixture model, equal
             feed, starts() as initial and final starts, the fixture's
             reference phases as three-phase start;
  budget     recovery with max_split_attempts = 0 (the quota test of
             pr76_near_dew_backend_test.cpp:302-331 on this mixture);
  no_starts  recovery with automatic starts off and no initial start (an
             empty search: a length_error in the reference);
  support    a final start off the feed's support (a domain_error before
             any property call, pt_split.hpp:436-443).
"""

from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mpmc_hnu_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402

REFERENCE = pyoracle.REFERENCE_ROOT
TEST = os.path.join(REFERENCE, "tests", "flash", "pr76_three_phase", "pr76_max3_robustness_test.cpp")

DUMP = r"""
#include <cstdio>
#define main robustness_test_main
#include "%s"
#undef main
static void vec(const char* key, const std::vector<double>& v, bool comma = true) {
    std::printf("\"%%s\": [", key);
    for (std::size_t i = 0; i < v.size(); ++i) std::printf("%%s%%.17g", i ? ", " : "", v[i]);
    std::printf("]%%s", comma ? ", " : "");
}
static void model_params(const char* key, const mpmc::thermodynamics::Pr76Phase<double>& m) {
    const auto& ps = m.parameters();
    const auto tc = ps.critical_temperatures_k(), pc = ps.critical_pressures_pa(), om = ps.acentric_factors();
    const auto kij = ps.kij_matrix();
    std::printf("\"%%s\": {", key);
    vec("tc", std::vector<double>(tc.begin(), tc.end()));
    vec("pc", std::vector<double>(pc.begin(), pc.end()));
    vec("omega", std::vector<double>(om.begin(), om.end()));
    vec("kij", std::vector<double>(kij.begin(), kij.end()), false);
    std::printf("}, ");
}
int main() {
    std::printf("{");
    model_params("recovery_model", recovery_model());
    model_params("fixture_model", pr76_max3_test::model());
    const auto& rp = recovery_phases();
    for (int k = 0; k < 3; ++k) { char key[32]; std::snprintf(key, 32, "recovery_phase%%d", k); vec(key, rp[k]); }
    const auto& fp = pr76_max3_test::reference_phases();
    for (int k = 0; k < 3; ++k) { char key[32]; std::snprintf(key, 32, "fixture_phase%%d", k); vec(key, fp[k]); }
    const auto st = pr76_max3_test::starts();
    std::printf("\"fixture_starts\": [");
    for (std::size_t k = 0; k < st.size(); ++k) {
        std::printf("%%s[", k ? ", " : "");
        for (std::size_t i = 0; i < st[k].size(); ++i) std::printf("%%s%%.17g", i ? ", " : "", st[k][i]);
        std::printf("]");
    }
    std::printf("], ");
    vec("fixture_feed", pr76_max3_test::equal_feed(), false);
    std::printf("}\n");
    return 0;
}
"""


def fixture_data() -> dict:
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dump.cpp")
        exe = os.path.join(tmp, "dump")
        with open(src, "w") as f:
            f.write(DUMP % TEST)
        inc = [f"-I{os.path.join(REFERENCE, 'modules', m, 'include')}" for m in ("ad", "thermodynamics", "flash")]
        subprocess.check_call(["g++", "-std=c++20", "-O1", *inc, src, "-o", exe])
        data = json.loads(subprocess.check_output([exe]).decode())
    text = open(TEST).read()
    m = re.search(r"const Vec metastable_witness\{([^}]*)\}", text)
    data["witness"] = [float(v) for v in m.group(1).replace("\n", " ").split(",")]
    return data


def mixture(d: dict) -> synth.Mixture:
    n = len(d["tc"])
    return synth.Mixture(np.array(d["tc"]), np.array(d["pc"]), np.array(d["omega"]), np.array(d["kij"]).reshape(n, n))


def main() -> None:
    pyoracle.build()
    if not pyoracle.reference_available() or not os.path.exists(TEST):
        raise SystemExit("reference harness or test source not available")
    d = fixture_data()
    rec = [np.array(d[f"recovery_phase{k}"]) for k in range(3)]
    fix = [np.array(d[f"fixture_phase{k}"]) for k in range(3)]
    rec_feed = 0.25 * rec[0] + 0.75 * rec[2]
    off_support = np.array([0.5, 0.5, 0.0])
    cases = {
        "recovery": dict(model="recovery", feed=rec_feed, initial=[d["witness"]], final=rec, three=rec,
                         fraction=(0.0, 0.75), auto=False, attempts=2),
        "three": dict(model="fixture", feed=np.array(d["fixture_feed"]), initial=d["fixture_starts"],
                      final=d["fixture_starts"], three=fix, fraction=(1.0 / 3.0, 1.0 / 3.0), auto=True, attempts=16),
        "budget": dict(model="recovery", feed=rec_feed, initial=[d["witness"]], final=rec, three=rec,
                       fraction=(0.0, 0.75), auto=False, attempts=0),
        "no_starts": dict(model="recovery", feed=rec_feed, initial=[], final=rec, three=None, fraction=None,
                          auto=False, attempts=2),
        "support": dict(model="recovery", feed=rec_feed, initial=[d["witness"]], final=[off_support], three=None,
                        fraction=None, auto=True, attempts=16),
    }
    out = {"recovery_tc": d["recovery_model"]["tc"], "recovery_pc": d["recovery_model"]["pc"],
           "recovery_omega": d["recovery_model"]["omega"], "recovery_kij": d["recovery_model"]["kij"],
           "fixture_tc": d["fixture_model"]["tc"], "fixture_pc": d["fixture_model"]["pc"],
           "fixture_omega": d["fixture_model"]["omega"], "fixture_kij": d["fixture_model"]["kij"],
           "cases": np.array(list(cases))}
    for name, c in cases.items():
        mix = mixture(d[f"{c['model']}_model"])
        feed = np.asarray(c["feed"], dtype=np.float64)[:, None]
        h = pyoracle.start_hints(3, 1, initial=[c["initial"]], final=[c["final"]],
                                 three_phase=[c["three"]] if c["three"] is not None else None,
                                 fraction=[c["fraction"]] if c["fraction"] is not None else None,
                                 initial_automatic_starts=c["auto"], max_split_attempts=c["attempts"])
        ref = pyoracle.reference_max3_hinted(mix, np.array([1e6]), np.array([250.0]), feed, h, threads=1)
        out[f"{name}_model"] = c["model"]
        out[f"{name}_z"] = feed
        for k, v in h.items():
            out[f"{name}_hint_{k}"] = np.asarray(v)
        for k, v in ref.items():
            out[f"{name}_ref_{k}"] = np.asarray(v)
        print(name, "max3", int(np.asarray(ref["max3_status"]).ravel()[0]), "published",
              int(np.asarray(ref["published"]).ravel()[0]), "attempts", int(np.asarray(ref["attempts"]).ravel()[0]))
    np.savez_compressed(os.path.join(HERE, "max3_hinted_reference.npz"), **out)


if __name__ == "__main__":
    main()
