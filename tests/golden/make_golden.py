"""Generate the golden fixtures of tests/golden from the MPMC_HNU reference.

Runs only where the reference sources exist (default /root/reference, or the
MPMC_REFERENCE_ROOT environment variable) and oracle/_ref/libpr76_ref.so has
been built from them (`make -C oracle ref`).  Writes:

kat.json
    The reference's own independent golden vectors (Decimal-precision PR76
    scripts in its test tree), parsed from its C++ reference headers, with the
    mixtures, states and tolerance budgets that its tests apply:
      tests/flash/pt_split/ternary_references.hpp     (ternary_test.cpp:24-46)
      tests/flash/pt_split/sensitivity_references.hpp (sensitivity_test.cpp:49-55, 220-260)
      tests/flash/pt_split/boundary_references.hpp    (boundary_test.cpp:28-34, 161-196, 240-300)
      tests/physics/thermodynamic_closure/closure_references.hpp (closure_test.cpp:35-48, 230-260)
reference_outputs.npz
    Outputs of the reference flash itself (solve_pr76_pt_vle,
    differentiate_pr76_pt_vle, build_pr76_pt_vle_closure, Pr76PhaseAdWorkspace)
    compiled from the unmodified headers, on (a) every KAT state above plus the
    dew-limit edge states of tests/flash/pt_split/dew_limit_references.hpp and
    (b) seeded synthetic cells for N in {3, 4, 6, 10, 12, 20}.

Machines without the reference sources run the tests against the committed
outputs of this script.
"""

from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mpmc_hnu_gb300 import synth  # noqa: E402
from oracle import pyoracle  # noqa: E402

REF = pyoracle.REFERENCE_ROOT
SPLIT = os.path.join(REF, "tests", "flash", "pt_split")
CLOSURE = os.path.join(REF, "tests", "physics", "thermodynamic_closure")

# ---------------------------------------------------------------------------
# A small tokenizer for C++ brace initialisers (decimal with L suffix, hex
# floats, strings, nested braces).
_TOKEN = re.compile(r'\s*(\{|\}|,|"[^"]*"|[-+]?0[xX][0-9a-fA-Fp.+-]+|[-+]?[0-9.]+(?:[eE][-+]?[0-9]+)?L?)')


def _parse_braces(text: str):
    pos = 0
    stack = [[]]
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            pos += 1
            continue
        tok = m.group(1)
        pos = m.end()
        if tok == "{":
            stack.append([])
        elif tok == "}":
            done = stack.pop()
            stack[-1].append(done)
        elif tok == ",":
            continue
        elif tok.startswith('"'):
            stack[-1].append(tok.strip('"'))
        elif tok.lower().startswith(("0x", "-0x", "+0x")):
            stack[-1].append(float.fromhex(tok))
        else:
            stack[-1].append(float(tok.rstrip("L")))
    return stack[0][0]


def _unwrap(x):
    """Remove the extra nesting of std::array double-brace initialisers."""
    while isinstance(x, list) and len(x) == 1 and isinstance(x[0], list):
        x = x[0]
    if isinstance(x, list):
        return [_unwrap(v) for v in x]
    return x


def parse_header(path: str) -> dict:
    text = open(path).read()
    out = {}
    for m in re.finditer(r"inline constexpr [^\n=]*?\b(\w+)(?:\[\])?\s*(?:=\s*)?(\{.*?\});", text, re.S):
        out[m.group(1)] = _unwrap(_parse_braces(m.group(2)))
    return out


# ---------------------------------------------------------------------------
# Mixtures of the reference tests (component data cited per use).
def mixture(specs, kij):
    n = len(specs)
    k = np.zeros((n, n))
    for (i, j), v in kij.items():
        k[i, j] = k[j, i] = v
    return {"tc": [s[0] for s in specs], "pc": [s[1] for s in specs], "omega": [s[2] for s in specs],
            "kij": k.tolist()}


# methane/ethane/propane, zero kij: ternary_test.cpp:94-99, sensitivity_test.cpp:126-132
TERNARY = mixture([(190.555, 4.595e6, 0.0), (305.4, 4.88e6, 0.099), (369.825, 4.248e6, 0.15308)], {})
# nitrogen/ethane, kij 0.08: sensitivity_test.cpp:76-100, boundary_test.cpp:64-78
N2_C2 = mixture([(126.2, 3.39e6, 0.04), (305.4, 4.88e6, 0.098)], {(0, 1): 0.08})
# carbon dioxide/methane, kij 0.095: boundary_test.cpp:64-78, dew_limit_test.cpp:62-72
CO2_C1 = mixture([(304.2, 7.38e6, 0.225), (190.6, 4.60e6, 0.008)], {(0, 1): 0.095})


def build_kat() -> dict:
    ter = parse_header(os.path.join(SPLIT, "ternary_references.hpp"))["ternary_references"]
    sens = parse_header(os.path.join(SPLIT, "sensitivity_references.hpp"))
    bnd = parse_header(os.path.join(SPLIT, "boundary_references.hpp"))
    clo = parse_header(os.path.join(CLOSURE, "closure_references.hpp"))
    dew = parse_header(os.path.join(SPLIT, "dew_limit_references.hpp"))

    flash_cases = []
    # ternary split anchors: 2e-9 * (1 + |e|), ternary_test.cpp:28, 40-46
    for k, (feed, x, y, beta, zl, zv) in enumerate(ter):
        flash_cases.append({"name": f"ternary_{k}", "mixture": "ternary", "p": 4.0e6, "t": 220.0, "feed": feed,
                            "must": "two", "x": x, "y": y, "beta": beta, "zl": zl, "zv": zv,
                            "abs_tol": 2e-9, "rel_scale": True, "beta_tol": 2e-9})
    # boundary pressure paths, z = {0.3, 0.7}: boundary_test.cpp:283-300, budgets :32-33
    for (carbon, coord, p, t, feed, x, y, beta, zl, zv, feed_z, tpd) in bnd["pressure_path"]:
        must = "two" if 0.1 <= coord <= 0.9 else ("not_two" if coord <= 0 or coord >= 1 else "any")
        flash_cases.append({"name": f"pressure_{'co2' if carbon else 'n2'}_{coord:g}",
                            "mixture": "co2_c1" if carbon else "n2_c2", "p": p, "t": t, "feed": [0.3, 0.7],
                            "must": must, "x": [x, 1 - x], "y": [y, 1 - y], "beta": beta, "zl": zl, "zv": zv,
                            "abs_tol": 2e-9, "rel_scale": False, "beta_tol": 1e-8, "first_only": True})
    # boundary composition paths along the tie lines: boundary_test.cpp:240-262
    coords = [-1e-3, -1e-6, -1e-10, 0.0, 1e-10, 1e-8, 1e-6, 1e-4, .01, .1, .25, .5, .75, .9, .99,
              .9999, .999999, .99999999, .9999999999, 1.0, 1.0000000001, 1.000001, 1.001]
    for (carbon, p, t, x, y, zl, zv) in bnd["ties"]:
        for q in coords:
            z0 = float((1 - q) * x + q * y)
            beta = (z0 - x) / (y - x)
            must = "two" if 0.01 <= q <= 0.99 else ("not_two" if q <= 0 or q >= 1 else "any")
            flash_cases.append({"name": f"composition_{'co2' if carbon else 'n2'}_{q:g}",
                                "mixture": "co2_c1" if carbon else "n2_c2", "p": p, "t": t, "feed": [z0, 1 - z0],
                                "must": must, "x": [x, 1 - x], "y": [y, 1 - y], "beta": beta, "zl": zl, "zv": zv,
                                "abs_tol": 2e-9, "rel_scale": False, "beta_tol": 1e-8, "first_only": True})
    # dew-limit audit states, CO2/methane at 220 K, z = {0.3, 0.7}: dew_limit_test.cpp:47-49, 160-170
    edge_cases = [{"name": f"dew_{name}", "mixture": "co2_c1", "p": p, "t": 220.0, "feed": [0.3, 0.7],
                   "region": region} for (name, p, region, *_rest) in dew["states"]]

    sens_cases = [
        # sensitivity_test.cpp:224-240, budget 2e-8 * max(1e-7, |e|) (:49-55)
        {"name": "binary", "mixture": "n2_c2", "p": 7.6e6, "t": 270.0, "feed": [0.3, 0.7],
         "dbeta": sens["binary_vapor_fraction"], "dlnk": sens["binary_log_k"], "dx": sens["binary_liquid"],
         "dy": sens["binary_vapor"], "tol": 2e-8},
        {"name": "ternary", "mixture": "ternary", "p": 4.0e6, "t": 220.0, "feed": ter[1][0],
         "dbeta": sens["ternary_vapor_fraction"], "dlnk": sens["ternary_log_k"], "dx": sens["ternary_liquid"],
         "dy": sens["ternary_vapor"], "tol": 2e-8},
    ]
    closure_cases = [
        # closure_test.cpp:35-48 budgets; states :234-256
        {"name": "binary", "mixture": "n2_c2", "p": 7.6e6, "t": 270.0, "feed": [0.3, 0.7],
         "primal": clo["binary_primal"], "dzl": clo["binary_liquid_z_gradient"],
         "dzv": clo["binary_vapor_z_gradient"], "drhol": clo["binary_liquid_density_gradient"],
         "drhov": clo["binary_vapor_density_gradient"], "primal_tol": 5e-11, "tol": 3e-8},
        {"name": "ternary", "mixture": "ternary", "p": 4.0e6, "t": 220.0,
         "feed": [0.69717974137952967145, 0.21360224237319418100, 0.08921801624727614754],
         "primal": clo["ternary_primal"], "dzl": clo["ternary_liquid_z_gradient"],
         "dzv": clo["ternary_vapor_z_gradient"], "drhol": clo["ternary_liquid_density_gradient"],
         "drhov": clo["ternary_vapor_density_gradient"], "primal_tol": 5e-11, "tol": 3e-8},
    ]
    return {"source": "MPMC_HNU test-tree Decimal references (see tests/golden/make_golden.py)",
            "mixtures": {"ternary": TERNARY, "n2_c2": N2_C2, "co2_c1": CO2_C1},
            "flash": flash_cases, "edge": edge_cases, "sensitivity": sens_cases, "closure": closure_cases}


class _Mix:
    def __init__(self, d):
        self.tc = np.array(d["tc"], float)
        self.pc = np.array(d["pc"], float)
        self.omega = np.array(d["omega"], float)
        self.kij = np.array(d["kij"], float)
        self.n = len(self.tc)

    def as_tuple(self):
        return self.tc, self.pc, self.omega, self.kij


SYNTH_CASES = [(3, 96, 5), (4, 96, 6), (6, 128, 1), (10, 96, 2), (12, 48, 3), (20, 32, 4)]
SENS_MAX_N = 10
KEEP = ["status", "beta", "x", "y", "ln_k", "ln_phi_l", "ln_phi_v", "z_l", "z_v", "counters"]
KEEP_SENS = ["sens_status", "dlnk", "dbeta", "dx", "dy", "dzl", "dzv", "drhol", "drhov", "jl", "jv"]


def build_reference_outputs(kat: dict) -> dict:
    arrays = {}
    # KAT and edge states grouped per mixture
    groups: dict[str, list] = {}
    for case in kat["flash"] + kat["edge"] + kat["sensitivity"] + kat["closure"]:
        groups.setdefault(case["mixture"], []).append(case)
    for name, cases in groups.items():
        mix = _Mix(kat["mixtures"][name])
        p = np.array([c["p"] for c in cases], float)
        t = np.array([c["t"] for c in cases], float)
        z = np.array([c["feed"] for c in cases], float).T.copy()
        out = pyoracle.reference_flash(mix, p, t, z, threads=8, sens=True)
        arrays[f"kat_{name}_p"] = p
        arrays[f"kat_{name}_t"] = t
        arrays[f"kat_{name}_z"] = z
        arrays[f"kat_{name}_names"] = np.array([c["name"] for c in cases])
        for k in KEEP + KEEP_SENS:
            arrays[f"kat_{name}_{k}"] = out[k]
    for n, ncell, seed in SYNTH_CASES:
        mix = synth.make_mixture(n, seed)
        p, t, z = synth.make_cells(n, ncell, seed)
        sens = n <= SENS_MAX_N
        out = pyoracle.reference_flash(mix, p, t, z, threads=8, sens=sens)
        arrays[f"synth_n{n}_seed"] = np.array([seed, ncell])
        for k in KEEP + (KEEP_SENS if sens else []):
            arrays[f"synth_n{n}_{k}"] = out[k]
    return arrays


def main() -> None:
    if not os.path.isdir(os.path.join(REF, "modules")):
        raise SystemExit(f"reference sources not found at {REF}")
    pyoracle.build()
    kat = build_kat()
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    arrays = build_reference_outputs(kat)
    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **arrays)
    print(f"wrote kat.json ({len(kat['flash'])} flash, {len(kat['edge'])} edge, "
          f"{len(kat['sensitivity'])} sensitivity, {len(kat['closure'])} closure cases) and "
          f"reference_outputs.npz ({len(arrays)} arrays)")


if __name__ == "__main__":
    main()
