"""Record the reference's selected-phase property chart on fixture cells.

Runs only where the MPMC_HNU reference sources were present to build
oracle/_ref/libpr76_ref.so (`make -C oracle ref`).  Writes
tests/golden/property_chart_reference.npz: for every case of
tests/chart_cases.golden_cases() (the reference closure test's own charts,
seeded synthetic charts with random pivots at 2, 4, 10 and 20 components and
one to three phases, and cells that fail in each reported class) the inputs
and the outputs of mpmc::flow::evaluate_pr76_selected_phase_property_chart
(modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533)
through the harness's ref_property_chart_batch.  Keys are <case>/<field>.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from tests import chart_cases  # noqa: E402


def main() -> None:
    pyoracle.build()
    if not pyoracle.reference_available():
        raise SystemExit("reference harness not built (make -C oracle ref)")
    data = {}
    for name, mix, spec, q, dep in chart_cases.golden_cases():
        r = pyoracle.reference_property_chart(mix, spec.phases, spec.root_index, spec.molar_mass, spec.viscosity,
                                              spec.enthalpy, q, dep, threads=1)
        tc, pc, omega, kij = mix.as_tuple()
        fields = {"tc": tc, "pc": pc, "omega": omega, "kij": kij, "phases": np.int32(spec.phases),
                  "root_index": np.array(spec.root_index, np.int32), "molar_mass": spec.molar_mass,
                  "viscosity": spec.viscosity, "enthalpy": spec.enthalpy, "q": q,
                  "dependent": dep if dep is not None else np.zeros((0, 0), np.int32),
                  "status": r["status"], "values": r["values"], "jacobian": r["jacobian"]}
        for k, v in fields.items():
            data[f"{name}/{k}"] = v
        print(name, "statuses", np.bincount(r["status"], minlength=8))
    path = os.path.join(HERE, "property_chart_reference.npz")
    np.savez_compressed(path, **data)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
