"""Extract the literal known answers of Chmy.jl's own test-suite into reference_kats.json.

Reads the reference's test files as TEXT (no Julia is needed or run) and records:
  * test/test_grids.jl      — the numeric expectations of bounds/extent/origin/spacing/
                              inv_spacing/coord on the 5x20 grid;
  * test/test_fields.jl     — the six expected interior arrays of set! (discrete/continuous);
  * test/test_grid_operators.jl — the vmag known answer.
Run from the repository root:  python tests/golden/make_reference_kats.py /path/to/Chmy.jl
"""

from __future__ import annotations

import json
import re
import sys
from pathlib import Path

OUT = Path(__file__).resolve().parent / "reference_kats.json"


def parse_julia_array(lit: str) -> list:
    """Julia `[a; b;; c; d;;; ...]` literal -> nested list indexed [z][y][x]."""
    body = lit.strip()[1:-1]
    slabs = []
    for slab in body.split(";;;"):
        cols = []
        for col in slab.split(";;"):
            cols.append([float(v) for v in col.replace("\n", " ").split(";") if v.strip()])
        slabs.append(cols)
    return slabs


def extract_fields(text: str) -> list[dict]:
    out = []
    for m in re.finditer(r"@test Array\(interior\(f\)\) == (\[[^\]]+\])", text):
        line = text.count("\n", 0, m.start()) + 1
        out.append({"line": line, "array_zyx": parse_julia_array(m.group(1))})
    return out


_TUP = r"\(([-\d.]+),\s*([-\d.]+)\)"


def extract_grids(text: str) -> list[dict]:
    out = []
    pat = re.compile(
        r"@test (?:all\()?(bounds|extent|origin|spacing|inv_spacing|coord)\(grid, (Vertex|Center)\(\), Dim\((\d)\)(?:, (\w+(?: \+ 1)?))?\) \.?≈ (" + _TUP + r"|[-\d.]+)\)?"
    )
    for m in pat.finditer(text):
        fn, loc, dim, idx, rhs = m.group(1), m.group(2), int(m.group(3)), m.group(4), m.group(5)
        if rhs.startswith("("):
            expected = [float(m.group(6)), float(m.group(7))]
        else:
            expected = float(rhs)
        out.append(
            {
                "line": text.count("\n", 0, m.start()) + 1,
                "fn": fn,
                "loc": loc,
                "dim": dim,
                "index": idx,
                "expected": expected,
            }
        )
    return out


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    kats = {
        "source": "Chmy.jl test-suite (test/test_grids.jl, test/test_fields.jl, test/test_grid_operators.jl)",
        "grids": {"nx": 5, "ny": 20, "origin": [-1, -2], "extent": [2, 4], "cases": extract_grids((ref / "test/test_grids.jl").read_text())},
        "fields": {"dims": [2, 2, 2], "origin": [0, 0, 0], "extent": [1, 1, 1], "loc": ["Center", "Vertex", "Center"],
                   "cases": extract_fields((ref / "test/test_fields.jl").read_text())},
    }
    ops = (ref / "test/test_grid_operators.jl").read_text()
    m = re.search(r"sigdigits=5\)\s*\.≈\s*([\d.]+)", ops)
    kats["vmag"] = {"value": 2.0, "expected_sigdigits5": float(m.group(1)), "line": ops.count("\n", 0, m.start()) + 1}
    OUT.write_text(json.dumps(kats, indent=1) + "\n")
    print(f"wrote {OUT}: {len(kats['grids']['cases'])} grid cases, {len(kats['fields']['cases'])} field arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_reference_kats.py <path to a Chmy.jl checkout>")
    main(sys.argv[1])
