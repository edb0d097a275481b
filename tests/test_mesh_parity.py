"""The product's host-side mesh builder (libodis_gpu.so, no GPU needed) against the oracle:
geometry and TRiSK weights must be bit-identical, since both follow the reference's formulas."""
import numpy as np
import pytest

from conftest import RADIUS, ref_grid
from test_grid import read_grid


def _compare(path):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    om = O.OracleMesh(path, RADIUS)
    pm = g.Mesh.from_file(path, RADIUS)
    assert (om.n_cells, om.n_edges, om.n_vertices) == (pm.n_cells, pm.n_edges, pm.n_vertices)
    for w in range(12):
        np.testing.assert_array_equal(om.field(w), pm.field(w), err_msg=f"field {w}")
    ta, tb = om.topology(), pm.topology()
    for k in ta:
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)
    # vertex geometry of the nonlinear terms; a face's two vertices are an
    # unordered pair (the reference's order there depends on its face loop and
    # enters no result)
    for w in range(5):
        np.testing.assert_array_equal(om.vertex_field(w), pm.vertex_field(w), err_msg=f"vertex field {w}")
    va, vb = om.vertex_topology(), pm.vertex_topology()
    for k in ("vert_nodes", "vert_faces", "vert_face_dir"):
        np.testing.assert_array_equal(va[k], vb[k], err_msg=k)
    np.testing.assert_array_equal(np.sort(va["face_verts"], axis=1), np.sort(vb["face_verts"], axis=1))
    return om, pm


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
def test_generated_grids(grid_dir, level):
    _compare(grid_dir / f"grid_{level}.txt")


@pytest.mark.parametrize("level", [2, 3, 4, 5])
def test_reference_grids(built, level):
    _compare(ref_grid(level))


def test_generate_in_memory_equals_file(grid_dir):
    import geodesicodis_gb300 as g
    a = g.Mesh.generate(3, RADIUS)
    b = g.Mesh.from_file(grid_dir / "grid_3.txt", RADIUS)
    for w in range(12):
        np.testing.assert_array_equal(a.field(w), b.field(w))


def test_bad_grid_is_rejected(tmp_path, built):
    import geodesicodis_gb300 as g
    p = tmp_path / "bad.txt"
    p.write_text("header\n0 0.0 0.0 {1, 2, 3, 4, 5, 99}, {(0,0), (0,0), (0,0), (0,0), (0,0), (0,0)}\n")
    with pytest.raises(g.OdisError):
        g.Mesh.from_file(p, RADIUS)
    with pytest.raises(g.OdisError):
        g.Mesh.from_file(tmp_path / "missing.txt", RADIUS)


def test_array_api_matches_file_path(grid_dir, built):
    """generate_grid (arrays) holds what generate_grid_file writes; Mesh.from_arrays builds the same mesh as
    Mesh.from_file; malformed friend lists are rejected (the checks the device build shares)."""
    import geodesicodis_gb300 as g
    nd, fr, cd = g.generate_grid(3)
    lat, lon, fr2, cent = read_grid(grid_dir / "grid_3.txt")
    np.testing.assert_array_equal(fr, fr2)
    rc = np.pi / 180                                   # read_grid returns radians
    np.testing.assert_array_equal(nd[:, 0] * rc, lat)
    np.testing.assert_array_equal(nd[:, 1] * rc, lon)
    np.testing.assert_array_equal(cd * rc, cent)
    a = g.Mesh.from_arrays(nd * (np.pi / 180), fr, cd * (np.pi / 180), 252.1e3)
    assert a.compare(g.Mesh.from_file(grid_dir / "grid_3.txt", 252.1e3)) == (0.0, 0)
    for k in range(3):
        bad = fr.copy()
        if k == 0:
            bad[9, 1] = len(nd)
        elif k == 1:
            bad[9, 1] = bad[9, 2]
        else:
            bad[9, 1], bad[9, 2] = bad[9, 2], bad[9, 1]
        with pytest.raises(g.OdisError):
            g.Mesh.from_arrays(nd * (np.pi / 180), bad, cd * (np.pi / 180), 252.1e3)


@pytest.mark.parametrize("level", [2, 4])
def test_reference_formulas_conditioning(built, level):
    """The reference's geometry formulas (acos arc lengths, cosine-law spherical excess of the kite areas)
    amplify last-bit input changes: one ulp on a random half of the coordinates moves the TRiSK weights and
    kite fractions far more than one ulp.  So a build with another math library (CUDA's, on the device) can
    match the reference's bits only in its integers; its geometry agrees to this conditioning."""
    import geodesicodis_gb300 as g
    nd, fr, cd = g.generate_grid(level)
    ns, cs = nd * (np.pi / 180), cd * (np.pi / 180)
    rng = np.random.default_rng(level)

    def bump(x):
        pick = (rng.random(x.shape) < 0.5) & (x != -np.pi / 180)
        return np.where(pick, np.nextafter(x, np.where(rng.random(x.shape) < 0.5, np.inf, -np.inf)), x)
    a = g.Mesh.from_arrays(ns, fr, cs, RADIUS)
    rel, bad = g.Mesh.from_arrays(bump(ns), fr, bump(cs), RADIUS).compare(a)
    print(f"level {level}: one-ulp input change moves the geometry by {rel:.1e} (relative)")
    assert bad == 0
    assert 1e-14 < rel < {2: 1e-11, 4: 1e-8}[level]
