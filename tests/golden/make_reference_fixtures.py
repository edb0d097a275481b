"""Writes the reference-input fixtures of the CPU tests from a GeodesicODIS checkout.

    ODIS_REFERENCE_ROOT=<checkout> python tests/golden/make_reference_fixtures.py

The reference ships no golden outputs; its inputs are the fixtures of its own
operator tests (src/tests.cpp runs over input_files/grid_l*.txt).  The two
smallest shipped grids (grid_l3.txt: 162 cells, grid_l4.txt: 642 cells) and
the shipped input.in are stored here gzip-compressed, byte for byte, with their
SHA-256 in MANIFEST.txt, so that the tests that pin the oracle and the host
mesh build on the reference's own grids run without the checkout.  The larger
grids (2562 cells and up) stay in the checkout; their tests run when
ODIS_REFERENCE_ROOT names it.
"""
from __future__ import annotations

import gzip
import hashlib
import os
import sys
from pathlib import Path

FILES = ("input_files/grid_l3.txt", "input_files/grid_l4.txt", "input.in")


def main() -> int:
    root = os.environ.get("ODIS_REFERENCE_ROOT")
    if not root:
        print("set ODIS_REFERENCE_ROOT to a GeodesicODIS checkout", file=sys.stderr)
        return 2
    here = Path(__file__).resolve().parent
    lines = []
    for rel in FILES:
        data = (Path(root) / rel).read_bytes()
        name = Path(rel).name
        with gzip.GzipFile(here / f"{name}.gz", "wb", compresslevel=9, mtime=0) as f:
            f.write(data)
        lines.append(f"{hashlib.sha256(data).hexdigest()}  {rel}")
    (here / "MANIFEST.txt").write_text("\n".join(lines) + "\n")
    print("\n".join(lines))
    return 0


if __name__ == "__main__":
    sys.exit(main())
