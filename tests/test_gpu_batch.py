"""Batched sweep (odis_batch_*) against the FP64 oracle, member by member.

Members differ in mesh level, thickness, drag, eccentricity, obliquity and
steps per orbit (FULL potential: eccentricity + obliquity tide).  The batch
runs FP32 state with double-float accumulation, so the bar is the FP32-variant
bar: dissipated power within 1e-4 of the FP64 oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ANGVEL_IN, GRAV, RADIUS, rel_err

pytestmark = pytest.mark.gpu


def _setup(grid_dir, count=11, seed=7, spo=(2000, 2400), levels=(2, 3)):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    angvel, P, _, _ = O.derive_time(ANGVEL_IN, 59.197)
    paths = [grid_dir / f"grid_{lv}.txt" for lv in levels]
    meshes = [g.Mesh.from_file(p, RADIUS) for p in paths]
    rng = np.random.default_rng(seed)
    members = []
    for i in range(count):
        members.append(dict(mesh=i % len(levels), steps_per_orbit=int(rng.choice(spo)),
                            h=float(10 ** rng.uniform(3.0, 4.3)), alpha=float(10 ** rng.uniform(-7, -4)),
                            ecc=float(rng.uniform(0.001, 0.01)), obliq=float(np.deg2rad(rng.uniform(0.0, 0.5)))))
    common = g.make_params(radius=RADIUS, g=GRAV, angvel=angvel, h=1.0, alpha=0.0, dt=1.0, potential=g.POT_FULL)
    return g, O, angvel, P, paths, meshes, members, common


def _oracle(O, path, angvel, P, m):
    om = O.OracleMesh(path, RADIUS)
    return O.OracleSolver(om, radius=RADIUS, g=GRAV, angvel=angvel, h=m["h"], alpha=m["alpha"], ecc=m["ecc"],
                          obliq=m["obliq"], dt=P / m["steps_per_orbit"], potential=O.FULL)


def test_batch_members_match_oracle(grid_dir):
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir)
    b = g.Batch(common, meshes, members)
    steps = 600
    op, sp = b.run(steps=steps, step_power=True)
    assert sp.shape == (len(members), steps)
    for i, m in enumerate(members):
        orc = _oracle(O, paths[m["mesh"]], angvel, P, m)
        po = orc.run(steps)
        _, vo, eo, _, _ = orc.get_state()
        it, vg, eg = b.get_member(i)
        assert it == steps
        assert rel_err(sp[i, steps // 2:], po[steps // 2:]) < 1e-4, i
        assert abs(sp[i, steps // 2:].mean() / po[steps // 2:].mean() - 1) < 1e-4, i
        assert rel_err(eg, eo) < 1e-3 and rel_err(vg, vo) < 1e-3, i
    b.close()


@pytest.mark.parametrize("rows", ["1", "2", "4"])
def test_batch_kernel_variants_match_oracle(grid_dir, monkeypatch, rows):
    """Each kernel variant forced by ODIS_BATCH_ROWS (face/cell rows per thread and tile): the same members
    against the FP64 oracle."""
    monkeypatch.setenv("ODIS_BATCH_ROWS", rows)
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=6, seed=11)
    b = g.Batch(common, meshes, members)
    assert b.info()["rows_per_thread"] == int(rows)
    steps = 400
    _, sp = b.run(steps=steps, step_power=True)
    for i, m in enumerate(members):
        orc = _oracle(O, paths[m["mesh"]], angvel, P, m)
        po = orc.run(steps)
        _, vo, eo, _, _ = orc.get_state()
        it, vg, eg = b.get_member(i)
        assert it == steps
        assert rel_err(sp[i, steps // 2:], po[steps // 2:]) < 1e-4, i
        assert rel_err(eg, eo) < 1e-3 and rel_err(vg, vo) < 1e-3, i
    b.close()


def test_batch_orbit_power_and_retirement(grid_dir, monkeypatch):
    """Members with fewer steps per orbit stop first; nothing about them depends on the others."""
    monkeypatch.setenv("ODIS_BATCH_ROWS", "2")      # both batches run the same kernel variant
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=9, seed=3)
    a = g.Batch(common, meshes, members)
    op, sp = a.run(orbits=1, step_power=True)
    spo = np.array([m["steps_per_orbit"] for m in members])
    assert op.shape == (len(members), 1)
    for i in range(len(members)):
        n = spo[i]
        assert np.all(sp[i, n:] == 0.0)
        assert abs(op[i, 0] / sp[i, :n].mean() - 1) < 1e-12
        assert a.get_member(i)[0] == n
    # the same members run for exactly 2000 steps each: the 2000-step members end bit-identical
    b = g.Batch(common, meshes, members)
    b.run(steps=2000)
    for i in np.flatnonzero(spo == 2000):
        _, va, ea = a.get_member(int(i))
        _, vb, eb = b.get_member(int(i))
        np.testing.assert_array_equal(va, vb)
        np.testing.assert_array_equal(ea, eb)
    a.close()
    b.close()


def test_batch_chunking_and_split_runs_are_bitwise(grid_dir, monkeypatch):
    monkeypatch.setenv("ODIS_BATCH_ROWS", "2")      # both batches run the same kernel variant
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=6, seed=5)
    a = g.Batch(common, meshes, members)
    b = g.Batch(common, meshes, members)
    _, pa = a.run(steps=400, step_power=True)
    _, pb1 = b.run(steps=100, step_power=True, chunk=30)
    _, pb2 = b.run(steps=300, step_power=True, chunk=64)
    np.testing.assert_array_equal(pa, np.concatenate([pb1, pb2], axis=1))
    for i in range(len(members)):
        np.testing.assert_array_equal(a.get_member(i)[1], b.get_member(i)[1])
        np.testing.assert_array_equal(a.get_member(i)[2], b.get_member(i)[2])
    assert a.info()["launches"] >= 1 and b.info()["launches"] > a.info()["launches"]
    a.close()
    b.close()


def test_batch_warm_start_entry_point(grid_dir):
    """set_member = state at orbital phase 0 with a fresh (forward-Euler) start, as the oracle's set_state(0, ...)."""
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=4, seed=11, spo=(2000,))
    b = g.Batch(common, meshes, members)
    warm = {}
    for i, m in enumerate(members):
        orc = _oracle(O, paths[m["mesh"]], angvel, P, m)
        orc.run(m["steps_per_orbit"])                      # one orbit: back at phase 0
        _, v, eta, _, _ = orc.get_state()
        warm[i] = (v, eta)
        b.set_member(i, v, eta)
        assert rel_err(b.get_member(i)[1], v) < 1e-12
    _, sp = b.run(steps=300, step_power=True)
    for i, m in enumerate(members):
        orc = _oracle(O, paths[m["mesh"]], angvel, P, m)
        E, N = orc.E, orc.N
        orc.set_state(0, warm[i][0], warm[i][1], np.zeros((E, 3)), np.zeros((N, 3)))
        po = orc.run(300)
        assert rel_err(sp[i], po) < 1e-4, i
    b.close()


def test_batch_nonfinite_member_is_reported(grid_dir):
    import geodesicodis_gb300 as g
    g_, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=3, seed=2)
    members[1] = dict(members[1], steps_per_orbit=20, h=1e5)   # far past the stability limit
    b = g.Batch(common, meshes, members)
    with pytest.raises(g.OdisError) as ex:
        b.run(steps=400)
    assert ex.value.code == g.ERR_NONFINITE
    # the other members are unaffected
    orc = _oracle(O, paths[members[0]["mesh"]], angvel, P, members[0])
    orc.run(400)
    assert rel_err(b.get_member(0)[2], orc.get_state()[2]) < 1e-3
    b.close()


def test_batch_bulk_state_and_projection(grid_dir):
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=10, seed=13)
    b = g.Batch(common, meshes, members)
    b.run(steps=200)
    for mesh in (0, 1):
        idx = b.mesh_members(mesh)
        v, eta = b.get_mesh_members(mesh)
        for k, i in enumerate(idx):
            _, vi, ei = b.get_member(int(i))
            np.testing.assert_array_equal(v[k], vi)
            np.testing.assert_array_equal(eta[k], ei)
        rng = np.random.default_rng(mesh)
        bv = rng.standard_normal((13, v.shape[1])).astype(np.float32)
        be = rng.standard_normal((9, eta.shape[1])).astype(np.float32)
        pr = b.project(mesh, bv, be)
        ref = np.concatenate([v @ bv.T.astype(np.float64), eta @ be.T.astype(np.float64)], axis=1)
        assert np.max(np.abs(pr - ref)) / np.max(np.abs(ref)) < 1e-5
        # bulk set: a scaled copy, then the members restart from step 0
        b.set_mesh_members(mesh, 2 * v, 3 * eta)
        v2, eta2 = b.get_mesh_members(mesh)
        assert rel_err(v2, 2 * v) < 1e-12 and rel_err(eta2, 3 * eta) < 1e-12
        assert all(b.get_member(int(i))[0] == 0 for i in idx)
    b.close()


def test_batch_run_is_one_graph_launch(grid_dir, monkeypatch):
    """Every run replays its chunks' cooperative launches from one CUDA graph; chunking changes nothing."""
    monkeypatch.setenv("ODIS_BATCH_ROWS", "2")      # both batches run the same kernel variant
    g, O, angvel, P, paths, meshes, members, common = _setup(grid_dir, count=6, seed=9)
    b = g.Batch(common, meshes, members)
    i0 = b.info()                                  # creation times the row variants with short runs
    b.run(steps=500, chunk=64)                     # 8 chunks
    info = b.info()
    assert info["graph_runs"] - i0["graph_runs"] == 1 and info["launches"] - i0["launches"] == 8
    c = g.Batch(common, meshes, members)
    c.run(steps=500, chunk=1000)
    for i in range(len(members)):
        np.testing.assert_array_equal(b.get_member(i)[1], c.get_member(i)[1])
    b.close()
    c.close()
