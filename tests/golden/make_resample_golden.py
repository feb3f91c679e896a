#!/usr/bin/env python3
"""Extract the reference's baked resample_poly(2, 3) filter into
tests/golden/resample23_table.json.

Run in a container where the reference checkout is present:

    python tests/golden/make_resample_golden.py /path/to/scir-reference

``scir_signal::resample_poly`` (crates/scir-signal/src/lib.rs:313-362) uses a
31-value table ``const H: [f64; 31]`` written as decimal literals.  Rust and C
both round a decimal literal to the nearest double, so the literal text
defines the taps bit for bit.  This script reads the table as text and writes
the literals (underscores removed) together with the IEEE-754 bit pattern of
each parsed value; the test suite compares the library's table with both and
never reads the reference tree.
"""
from __future__ import annotations

import json
import os
import re
import struct
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = "crates/scir-signal/src/lib.rs"
NUM = r"-?[0-9][0-9_]*(?:\.[0-9_]*)?(?:[eE][-+]?[0-9]+)?"


def extract(text: str) -> list:
    fn = text.index("pub fn resample_poly(")
    m = re.search(r"const H: \[f64; (\d+)\] = \[(.*?)\];", text[fn:], re.S)
    if not m:
        raise SystemExit("table H not found after resample_poly")
    lits = [s.replace("_", "") for s in re.findall(NUM, m.group(2))]
    if len(lits) != int(m.group(1)):
        raise SystemExit(f"expected {m.group(1)} literals, found {len(lits)}")
    line = text[:fn + m.start()].count("\n") + 1
    return lits, line


def main(argv):
    ref = argv[1] if len(argv) > 1 else "/root/reference"
    with open(os.path.join(ref, SRC)) as f:
        lits, line = extract(f.read())
    out = {
        "source": f"{SRC}:{line}",
        "up": 2, "down": 3,
        "literals": lits,
        "bits": [struct.unpack("<Q", struct.pack("<d", float(s)))[0] for s in lits],
    }
    path = os.path.join(HERE, "resample23_table.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(f"wrote {path}: {len(lits)} taps from {out['source']}")


if __name__ == "__main__":
    main(sys.argv)
