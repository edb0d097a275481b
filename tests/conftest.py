"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

# A GeodesicODIS checkout (its shipped grids and input.in serve as fixtures), named by the
# environment variable ODIS_REFERENCE_ROOT.  Without it the tests use the byte-exact copies of
# the smallest shipped files in tests/golden (make_reference_fixtures.py) and skip the rest.
REF_ROOT = Path(os.environ["ODIS_REFERENCE_ROOT"]) if os.environ.get("ODIS_REFERENCE_ROOT") else None
REF_INPUT = (REF_ROOT / "input_files") if REF_ROOT else Path("__no_reference_checkout__")
REF_SKIP = "set ODIS_REFERENCE_ROOT to a GeodesicODIS checkout to run the tests on its shipped files"
GOLDEN = ROOT / "tests" / "golden"
_unpacked: dict[str, Path] = {}

# Enceladus-like body of the benchmark configurations
RADIUS = 252.1e3
GRAV = 0.113
ANGVEL_IN = 5.307e-5


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libodis_gpu.so")


@pytest.fixture(scope="session")
def built():
    """Build the product library and the oracle once per session (idempotent)."""
    from geodesicodis_gb300 import build_ext
    from oracle import pyoracle
    build_ext.build()
    pyoracle.build()
    return True


@pytest.fixture(scope="session")
def grid_dir(tmp_path_factory, built):
    import geodesicodis_gb300 as g
    d = tmp_path_factory.mktemp("grids")
    for lvl in range(0, 6):
        g.generate_grid_file(lvl, d / f"grid_{lvl}.txt")
    return d


def _golden_copy(rel: str) -> Path | None:
    """The fixture copy of the reference file `rel`, unpacked once per process and checked against the
    SHA-256 of the shipped file; None when tests/golden holds no copy of it."""
    import atexit
    import gzip
    import hashlib
    import shutil
    import tempfile
    if rel in _unpacked:
        return _unpacked[rel]
    gz = GOLDEN / (Path(rel).name + ".gz")
    if not gz.exists():
        return None
    sums = dict(line.split()[::-1] for line in (GOLDEN / "MANIFEST.txt").read_text().splitlines() if line.strip())
    data = gzip.decompress(gz.read_bytes())
    assert hashlib.sha256(data).hexdigest() == sums[rel], f"{gz} does not match the shipped {rel}"
    if "dir" not in _unpacked:
        d = Path(tempfile.mkdtemp(prefix="odis_ref_"))
        atexit.register(shutil.rmtree, d, True)
        _unpacked["dir"] = d
    out = _unpacked["dir"] / Path(rel).name
    out.write_bytes(data)
    _unpacked[rel] = out
    return out


def ref_file(rel: str) -> Path:
    """A file of the reference checkout (path relative to its root), else its fixture copy; skips the
    calling test when neither exists."""
    if REF_ROOT is not None and (REF_ROOT / rel).exists():
        return REF_ROOT / rel
    p = _golden_copy(rel)
    if p is None:
        pytest.skip(REF_SKIP)
    return p


def ref_grid(level_baseline: int) -> Path:
    """The reference's shipped grid with 10*4^level+2 cells (its file is named one level higher)."""
    return ref_file(f"input_files/grid_l{level_baseline + 1}.txt")


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    s = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / s)


def ecc_case_params(**over):
    """The reference's own CPU-sized case: h = 10 km, alpha = 1e-5, ECC e = 0.0047, 2000 steps/orbit."""
    from oracle import pyoracle as O
    angvel, P, dt, n = O.derive_time(ANGVEL_IN, 59.197)
    p = dict(radius=RADIUS, g=GRAV, angvel=angvel, h=1e4, alpha=1e-5, ecc=0.0047, obliq=0.0, love_reduct=1.0,
             dt=dt, potential=O.ECC, init_load=0)
    p.update(over)
    return p


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
