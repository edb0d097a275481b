"""DATA/data.h5 output (src/outFiles.cpp:138-823) without the HDF5 library.

The image has no HDF5 library, so the checker is tests/h5read.py, a reader
written from the HDF5 file-format specification.  It is pinned first against
HDF5 files that the HDF5 library itself wrote (the reference's shipped
input_files/*.h5, and a MATLAB v7.3 file that scipy ships as test data), where
those files exist; then the library's writer (odis_h5_*) is read back through it.
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np
import pytest

import h5read
from conftest import REF_INPUT

SCIPY_MAT = None
try:
    import scipy
    SCIPY_MAT = Path(scipy.__file__).parent / "io" / "matlab" / "tests" / "data" / "testhdf5_7.4_GLNX86.mat"
except ImportError:      # pragma: no cover
    pass

# the reference's dataset names and creation order (CreateHDF5Framework, DumpGridData)
REF_NAMES = ["east velocity", "north velocity", "x velocity", "y velocity", "z velocity", "displacement",
             "dissipated energy", "dissipation avg output", "kinetic avg output", "dummy1 output",
             "face longitude", "face latitude"]


def test_reader_on_library_written_csr_file():
    """The reference's regridding weights (written by the HDF5 library): a CSR matrix whose row
    pointer is non-decreasing and ends at the number of non-zeros."""
    path = REF_INPUT / "grid_l4_6x6_weights.h5"
    if not path.exists():
        pytest.skip("reference input files not mounted")
    f = h5read.H5File(path)
    assert f.superblock_version == 0 and (f.leaf_k, f.internal_k) == (4, 16)
    ds = f.datasets()
    assert sorted(ds) == ["column index", "row index", "weights"]
    r, c, w = ds["row index"].read(), ds["column index"].read(), ds["weights"].read()
    assert r.dtype == np.int32 and w.dtype == np.float64
    assert r[0] == 0 and r[-1] == c.size == w.size and np.all(np.diff(r) >= 0)
    sums = np.add.reduceat(w, r[:-1][np.diff(r) > 0])
    assert np.median(sums) == pytest.approx(1.0)


def test_reader_on_matlab_file():
    """A MATLAB v7.3 file (HDF5 with a 512-byte user block) that scipy ships: `testdouble` is
    0:pi/4:2*pi, stored with a version-2 layout message."""
    if SCIPY_MAT is None or not SCIPY_MAT.exists():
        pytest.skip("scipy's MATLAB test data not installed")
    f = h5read.H5File(SCIPY_MAT)
    assert f.base == 512
    x = f.datasets()["testdouble"].read()
    np.testing.assert_array_equal(x.ravel(), np.arange(9) * (np.pi / 4))


def _reference_like(tmp_path, T=5, N=42, E=120):
    import geodesicodis_gb300 as g
    shapes = {"east velocity": (T, E), "north velocity": (T, E), "x velocity": (T, N), "y velocity": (T, N),
              "z velocity": (T, N), "displacement": (T, N), "dissipated energy": (T, E),
              "dissipation avg output": (T,), "kinetic avg output": (T,), "dummy1 output": (T, N),
              "face longitude": (E,), "face latitude": (E,)}
    path = tmp_path / "data.h5"
    w = g.H5Writer(path, [(n, shapes[n]) for n in REF_NAMES])
    return w, path, shapes


def test_writer_round_trip(built, tmp_path):
    """Every dataset of the reference's layout: extents, float32, contiguous storage, rows written
    in place out of order, unwritten rows read as the fill value 0, and the group structure
    (12 links over two symbol nodes, keys bounding them) valid."""
    T = 5
    w, path, shapes = _reference_like(tmp_path, T)
    rng = np.random.default_rng(0)
    expect = {n: np.zeros(s, np.float32) for n, s in shapes.items()}
    for t in (3, 0, 1):           # row 2 and 4 stay unwritten
        for n, s in shapes.items():
            if len(s) == 2:
                row = rng.standard_normal(s[1]).astype(np.float32)
                w.write_rows(n, t, row)
                expect[n][t] = row
            elif n in ("dissipation avg output", "kinetic avg output"):
                v = np.float32(rng.standard_normal())
                w.write_rows(n, t, [v])
                expect[n][t] = v
    lon = rng.uniform(-180, 180, shapes["face longitude"]).astype(np.float32)
    w.write_rows("face longitude", 0, lon)
    expect["face longitude"] = lon
    w.close()
    f = h5read.H5File(path)
    assert f.eof == path.stat().st_size
    ds = f.datasets()
    assert sorted(ds) == sorted(REF_NAMES)
    for n, s in shapes.items():
        d = ds[n]
        assert d.shape == s and d.maxshape == s and d.dtype == np.dtype("<f4") and d.layout[0] == "contiguous"
        assert d.messages == [0x0001, 0x0003, 0x0005, 0x0008, 0x0012, 0x0000]
        np.testing.assert_array_equal(d.read(), expect[n])
    # the B-tree has one leaf node over two symbol nodes (8 + 4 links)
    btree = struct.unpack_from("<Q", f.root_messages()[0][1])[0]
    assert f.buf[btree:btree + 4] == b"TREE" and struct.unpack_from("<H", f.buf, btree + 6)[0] == 2


def test_writer_checks_arguments(built, tmp_path):
    import geodesicodis_gb300 as g
    with pytest.raises(g.OdisError):
        g.H5Writer(tmp_path / "a.h5", [("x", (2, 3)), ("x", (4,))])          # duplicate name
    with pytest.raises(g.OdisError):
        g.H5Writer(tmp_path / "b.h5", [("", (2,))])                          # empty name
    with pytest.raises(g.OdisError):
        g.H5Writer(tmp_path / "c.h5", [("x", (2, 3, 4))])                    # rank 3
    with pytest.raises(g.OdisError):
        g.H5Writer(tmp_path / "missing" / "d.h5", [("x", (2,))])             # no directory
    w = g.H5Writer(tmp_path / "e.h5", [("x", (2, 3))])
    with pytest.raises(g.OdisError):
        w.write_rows("x", 1, np.zeros(6))                                    # past the extent
    with pytest.raises(g.OdisError):
        w.write_rows("x", 0, np.zeros(4))                                    # not whole rows
    w.write_rows("x", 1, np.ones(3))
    w.close()
    np.testing.assert_array_equal(h5read.H5File(tmp_path / "e.h5").datasets()["x"].read(), [[0, 0, 0], [1, 1, 1]])


def test_writer_many_datasets(built, tmp_path):
    """More links than one symbol node holds: 100 datasets over 13 symbol nodes, all readable."""
    import geodesicodis_gb300 as g
    names = [f"field {k:03d}" for k in range(100)][::-1]
    with g.H5Writer(tmp_path / "m.h5", [(n, (2,)) for n in names]) as w:
        for k, n in enumerate(names):
            w.write_rows(n, 0, [k, -k])
    ds = h5read.H5File(tmp_path / "m.h5").datasets()
    assert len(ds) == 100
    for k, n in enumerate(names):
        np.testing.assert_array_equal(ds[n].read(), [k, -k])
