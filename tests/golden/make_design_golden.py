#!/usr/bin/env python3
"""Extract the reference's IIR-design known answers into tests/golden/design_zpk.json.

Run in a container where the reference checkout is present:

    python tests/golden/make_design_golden.py /path/to/scir-reference

The reference's ``crates/scir-iir-filters/src/filter_design.rs`` tests check
``butter_internal(N, <band>(Wn...), None)`` (Wn normalised to Nyquist = 1)
against zeros / poles / gain that SciPy produced, with a tolerance each.  This
script reads those test bodies as text and writes, per test: the order, the
band type, the edges, the expected zeros and poles as [re, im] pairs, the gain
and the tolerance.  The test suite only reads the JSON file.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = "crates/scir-iir-filters/src/filter_design.rs"

NUM = r"-?[0-9][0-9_]*(?:\.[0-9_]*)?(?:[eE][-+]?[0-9]+)?"
PAIR = re.compile(r"\(\s*(" + NUM + r")\s*,\s*(" + NUM + r")\s*\)")


def _num(s: str) -> float:
    return float(s.replace("_", ""))


def _complex_list(body: str) -> list:
    """[re, im] pairs of a `vec_cplx![...]` or `vec![Complex::one(); n]` field."""
    m = re.search(r"vec!\[\s*Complex::<f64>::one\(\);\s*(\d+)\s*\]", body)
    if m:
        return [[1.0, 0.0]] * int(m.group(1))
    return [[_num(a), _num(b)] for a, b in PAIR.findall(body)]


def extract(text: str) -> list:
    cases = []
    for m in re.finditer(r"fn (test_butter_\w+)\(\)\s*\{(.*?)\n    \}\n", text, re.S):
        name, body = m.group(1), m.group(2)
        call = re.search(r"butter_internal\(\s*(\d+)\s*,\s*(\w+)\(([^)]*)\)\s*,\s*None\s*\)", body)
        exp = re.search(r"ZPKCoeffs\s*\{(.*?)\n\s*\};", body, re.S)
        tol = re.search(r"assert_approx_equal_to_with_sort\(&zpk_expected,\s*(" + NUM + ")", body)
        if not (call and exp and tol):
            continue
        fields = exp.group(1)
        z_part = fields[fields.index("z:"):fields.index("p:")]
        p_part = fields[fields.index("p:"):fields.index("k:")]
        k = _num(re.search(r"k:\s*(" + NUM + ")", fields).group(1))
        cases.append({
            "name": name,
            "order": int(call.group(1)),
            "btype": call.group(2),
            "wn": [_num(v) for v in call.group(3).split(",")],
            "z": _complex_list(z_part),
            "p": _complex_list(p_part),
            "k": k,
            "tol": _num(tol.group(1)),
            "source": f"{SRC} ({name})",
        })
    return cases


def main(argv: list) -> int:
    if len(argv) != 2:
        print(__doc__)
        return 2
    with open(os.path.join(argv[1], SRC)) as f:
        cases = extract(f.read())
    out = os.path.join(HERE, "design_zpk.json")
    with open(out, "w") as f:
        json.dump(cases, f, indent=1)
    print(f"{len(cases)} cases -> {out}")
    for c in cases:
        print(f"  {c['name']}: N={c['order']} {c['btype']}{tuple(c['wn'])} "
              f"{len(c['z'])} zeros {len(c['p'])} poles tol {c['tol']}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
