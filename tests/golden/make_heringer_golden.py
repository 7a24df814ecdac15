"""Record the reference's max-3-phase orchestration on a six-component
sour-gas mixture.

Runs only where the MPMC_HNU reference sources are present.  The mixture is
the reference tests' own Heringer-2026 sour-gas fixture
(tests/flash/pr76_three_phase/heringer_2026_sour_gas_fixture.hpp: PR76 Tc,
Pc, omega and kij of its six components, and the Table-B1 feed): a small
C++ program compiled against that header prints them, so nothing is
transcribed by hand.  The states follow the reference's own P-Z path
(pr76_heringer_2026_boundary_test.cpp:27-53): CO2 mole fraction
0.60-0.85 with the other components in their Table-B1 proportions, p 20-50 bar,
T in {170, 178.8, 190} K.  Writes tests/golden/max3_heringer_reference.npz with
the mixture, the states and the outputs of solve_pr76_pt_max3 through the
harness's ref_max3_batch.
"""

from __future__ import annotations

import json
import os
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
FIXTURE = os.path.join(REFERENCE, "tests", "flash", "pr76_three_phase", "heringer_2026_sour_gas_fixture.hpp")

DUMP = r"""
#include <cstdio>
#include "%s"
namespace fx = pr76_heringer_2026_sour_gas_test;
int main() {
    const std::size_t n = fx::critical_temperatures_k.size();
    std::printf("{\"tc\": [");
    for (std::size_t i = 0; i < n; ++i) std::printf("%%s%%.17g", i ? ", " : "", fx::critical_temperatures_k[i]);
    std::printf("], \"pc\": [");
    for (std::size_t i = 0; i < n; ++i) std::printf("%%s%%.17g", i ? ", " : "", fx::critical_pressures_pa[i]);
    std::printf("], \"omega\": [");
    for (std::size_t i = 0; i < n; ++i) std::printf("%%s%%.17g", i ? ", " : "", fx::acentric_factors[i]);
    std::printf("], \"kij\": [");
    for (std::size_t i = 0; i < n; ++i)
        for (std::size_t j = 0; j < n; ++j) std::printf("%%s%%.17g", i + j ? ", " : "", i == j ? 0.0 : fx::kij(i, j));
    std::printf("], \"feed\": [");
    for (std::size_t i = 0; i < n; ++i) std::printf("%%s%%.17g", i ? ", " : "", fx::table_b1_mole_percent[i]);
    std::printf("]}\n");
    return 0;
}
"""


def fixture_data() -> dict:
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "dump.cpp")
        exe = os.path.join(tmp, "dump")
        with open(src, "w") as f:
            f.write(DUMP % FIXTURE)
        inc = [f"-I{os.path.join(REFERENCE, 'modules', m, 'include')}" for m in ("ad", "thermodynamics", "flash")]
        subprocess.check_call(["g++", "-std=c++20", "-O1", *inc, src, "-o", exe])
        return json.loads(subprocess.check_output([exe]).decode())


def main() -> None:
    pyoracle.build()
    if not pyoracle.reference_available() or not os.path.exists(FIXTURE):
        raise SystemExit("reference harness or fixture not available")
    data = fixture_data()
    n = len(data["tc"])
    mix = synth.Mixture(np.array(data["tc"]), np.array(data["pc"]), np.array(data["omega"]),
                        np.array(data["kij"]).reshape(n, n))
    b1 = np.array(data["feed"])
    rest = b1[1:] / b1[1:].sum()
    cells = []
    for zc in np.round(np.arange(0.60, 0.851, 0.025), 3):
        feed = np.concatenate([[zc], (1.0 - zc) * rest])
        for pb in np.arange(20.0, 50.1, 2.5):
            for t in (170.0, 178.8, 190.0):
                cells.append((pb * 1e5, t, feed))
    p = np.array([c[0] for c in cells])
    t = np.array([c[1] for c in cells])
    z = np.ascontiguousarray(np.array([c[2] for c in cells]).T)
    ref = pyoracle.reference_max3(mix, p, t, z, threads=16)
    np.savez_compressed(os.path.join(HERE, "max3_heringer_reference.npz"), tc=mix.tc, pc=mix.pc, omega=mix.omega,
                        kij=mix.kij, p=p, t=t, z=z, **{f"ref_{k}": v for k, v in ref.items()})
    counts = np.bincount(ref["max3_status"] + 1, minlength=7)
    print(len(cells), "cells; max3 status counts (invalid, single, two, three, boundary, higher, indeterminate):",
          counts)


if __name__ == "__main__":
    main()
