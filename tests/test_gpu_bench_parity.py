"""GPU parity at the benchmarked sizes: the workloads bench.py times, against the FP64 oracle.

* Level 6 (40962 cells), ECC tide, self-gravity/loading to l_max = 16, 4200 steps per orbit: one whole orbit
  in FP64 and DF64 within 1e-10 (max-abs normalised) on eta, v, both AB3 histories and the power series; the
  FP32-state variant's power within 1e-4, its per-field errors printed.
* Every tile shape of the self-gravity transforms (ODIS_SH_TILES: degrees per analysis tile, cell chunks,
  synthesis lanes or the dense synthesis's warps, cells per synthesis thread), each a different code path,
  over 300 steps.
* Level 8 (655362 cells), FULL tide, l_max = 32, h = 20 km, drag 1e-6: 200 steps at the stable step.
* Batch members on levels 4, 5 and 6, thick oceans included at their stable step counts.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ANGVEL_IN, GRAV, RADIUS, rel_err

pytestmark = pytest.mark.gpu

L6_STEPS = 4200          # one orbit at 4200 steps per orbit (dt = 28.189 s)
L6_SHORT = 300


def _cmp(gpu_state, orc_state, tol):
    _, vg, eg, dvg, deg = gpu_state
    _, vo, eo, dvo, deo = orc_state
    errs = dict(eta=rel_err(eg, eo), v=rel_err(vg, vo), dvdt=rel_err(dvg, dvo), detadt=rel_err(deg, deo))
    for k, e in errs.items():
        assert e < tol, (k, e)
    return errs


@pytest.fixture(scope="module")
def level6(tmp_path_factory, built):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    path = tmp_path_factory.mktemp("l6") / "grid_6.txt"
    g.generate_grid_file(6, path)
    angvel, P, dt, n = O.derive_time(ANGVEL_IN, 28.19)
    assert n == L6_STEPS
    fac = O.benchmark_sh_factors(GRAV, RADIUS, 16, seed=1)
    p = dict(radius=RADIUS, g=GRAV, angvel=angvel, h=1e4, alpha=1e-5, ecc=0.0047, dt=dt, potential=O.ECC,
             sh_lmax=16, sh_factors=fac)
    orc = O.OracleSolver(O.OracleMesh(path, RADIUS), **p)
    p_short = orc.run(L6_SHORT)
    s_short = orc.get_state()
    p_full = np.concatenate([p_short, orc.run(L6_STEPS - L6_SHORT)])
    s_full = orc.get_state()
    return dict(p=p, mesh=g.Mesh.from_file(path, RADIUS), short=(p_short, s_short), full=(p_full, s_full))


def _solver(level6, precision):
    import geodesicodis_gb300 as g
    return g.Solver(g.make_params(precision=precision, **level6["p"]), level6["mesh"])


@pytest.mark.parametrize("precision", [0, 2])
def test_level6_sh16_one_orbit(level6, precision):
    """The benchmark workload, one orbit, with the tiles the setup-time timing picks on this GPU."""
    sol = _solver(level6, precision)
    pg = sol.run(L6_STEPS)
    po, so = level6["full"]
    errs = _cmp(sol.get_state(), so, 1e-10)
    errs["power"] = rel_err(pg, po)
    print(f"level 6 l_max 16 precision {precision} tiles {sol.sh_tiles()}: {errs}")
    assert errs["power"] < 1e-10
    assert po[-1] > 0
    sol.close()


def test_level6_sh16_fp32_variant(level6):
    """FP32 state and stencils: power within 1e-4 of the FP64 oracle over the orbit's second half; the state
    errors are reported (relative, max-abs normalised)."""
    sol = _solver(level6, 1)
    pg = sol.run(L6_STEPS)
    po, so = level6["full"]
    _, vg, eg, _, _ = sol.get_state()
    _, vo, eo, _, _ = so
    e = dict(power=rel_err(pg[L6_STEPS // 2:], po[L6_STEPS // 2:]), eta=rel_err(eg, eo), v=rel_err(vg, vo))
    print(f"level 6 l_max 16 FP32 tiles {sol.sh_tiles()}: {e}")
    assert e["power"] < 1e-4
    assert e["eta"] < 1e-3 and e["v"] < 1e-3
    sol.close()


# (degrees per analysis tile, cell chunks, synthesis lanes (16, 32, 48: a warp per order pair, 1-3 cell
# groups per block; -4, -8, -16: the dense synthesis Z t with that many warps per block), cells per
# synthesis thread, analysis from precomputed trig-weighted values): every value of each parameter appears
TILES = [(2, 8, 1, 1, 0), (4, 16, 2, 2, 1), (8, 32, 4, 1, 0), (2, 64, 8, 2, 1), (4, 8, 16, 1, 1),
         (8, 64, 16, 2, 0), (2, 16, 16, 2, 1), (4, 4, 32, 1, 1), (2, 2, 48, 2, 0),
         (2, 8, -8, 1, 1), (4, 16, -16, 2, 0), (8, 32, -4, 2, 1), (2, 4, -4, 1, 0),
         (2, 7, 16, 1, 1), (4, 13, -8, 1, 0)]          # chunk counts that fill whole waves are not powers of two


@pytest.mark.parametrize("precision", [0, 2, 1])
@pytest.mark.parametrize("tiles", TILES, ids=lambda t: "x".join(map(str, t)))
def test_level6_sh_tile_paths(level6, monkeypatch, precision, tiles):
    monkeypatch.setenv("ODIS_SH_TILES", ",".join(map(str, tiles)))
    monkeypatch.setenv("ODIS_SH_TC", "0")
    sol = _solver(level6, precision)
    assert tuple(sol.sh_tuning()) == tiles
    pg = sol.run(L6_SHORT)
    po, so = level6["short"]
    if precision == 1:
        assert rel_err(pg[L6_SHORT // 2:], po[L6_SHORT // 2:]) < 1e-4
        _cmp(sol.get_state(), so, 1e-3)
    else:
        _cmp(sol.get_state(), so, 1e-10)
        assert rel_err(pg, po) < 1e-10
    sol.close()


@pytest.mark.parametrize("precision", [0, 2, 1])
def test_level6_half_and_full_basis(level6, monkeypatch, precision):
    """The antipodal half basis (the default on these centrally symmetric meshes) and the full basis
    (ODIS_SH_HALF=0) give the same run: to rounding in FP64/DF64, and both against the oracle."""
    half = _solver(level6, precision)
    lay = half.sh_layout()
    assert lay["half"] and lay["cells"] == 40962 // 2
    monkeypatch.setenv("ODIS_SH_HALF", "0")
    full = _solver(level6, precision)
    assert not full.sh_layout()["half"] and full.sh_layout()["cells"] == 40962
    assert full.sh_layout()["basis_bytes"] == 2 * lay["basis_bytes"]
    ph, pf = half.run(L6_SHORT), full.run(L6_SHORT)
    po, so = level6["short"]
    # FP64: the two bases differ by rounding only; double-float carries its 48-bit rounding along
    tol = {0: 1e-12, 2: 1e-11, 1: 1e-4}[precision]
    assert rel_err(ph, pf) < tol
    for x, y in zip(half.get_state()[1:], full.get_state()[1:]):
        assert rel_err(x, y) < (1e-3 if precision == 1 else tol)
    if precision != 1:
        _cmp(full.get_state(), so, 1e-10)
    half.close()
    full.close()


def test_level6_sh16_tensor_core_path(level6, monkeypatch):
    """The FP32 method's tcgen05 transforms at the benchmark size."""
    monkeypatch.setenv("ODIS_SH_TC", "1")
    sol = _solver(level6, 1)
    assert sol.sh_tiles()[0] == 0
    pg = sol.run(L6_SHORT)
    po, so = level6["short"]
    assert rel_err(pg[L6_SHORT // 2:], po[L6_SHORT // 2:]) < 1e-4
    _cmp(sol.get_state(), so, 1e-3)
    sol.close()


def test_level8_sh32_sample(tmp_path, built):
    """The level-8 workload: FULL tide (e 0.0047, obliquity 0.2 deg), h 20 km, drag 1e-6,
    l_max 32, at the stable step count; 200 steps in FP64 and DF64 (1e-10) and FP32 (power 1e-4)."""
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    path = tmp_path / "grid_8.txt"
    g.generate_grid_file(8, path)
    mesh = g.Mesh.from_file(path, RADIUS)
    angvel, P, _, _ = O.derive_time(ANGVEL_IN, 118394.0 / 8000)
    n = g.stable_steps_per_orbit(P, mesh.gravity_wave_omega(GRAV, 2e4), 0.95)
    fac = O.benchmark_sh_factors(GRAV, RADIUS, 32, seed=1)
    p = dict(radius=RADIUS, g=GRAV, angvel=angvel, h=2e4, alpha=1e-6, ecc=0.0047, obliq=np.deg2rad(0.2),
             dt=P / n, potential=O.FULL, sh_lmax=32, sh_factors=fac)
    steps = 200
    orc = O.OracleSolver(O.OracleMesh(path, RADIUS), **p)
    po = orc.run(steps)
    so = orc.get_state()
    del orc
    for prec, tol in ((0, 1e-10), (2, 1e-10), (1, 1e-4)):
        sol = g.Solver(g.make_params(precision=prec, **p), mesh)
        pg = sol.run(steps)
        if prec == 1:
            assert rel_err(pg[steps // 2:], po[steps // 2:]) < tol
            errs = _cmp(sol.get_state(), so, 1e-3)
        else:
            errs = _cmp(sol.get_state(), so, tol)
            assert rel_err(pg, po) < tol
        print(f"level 8 l_max 32 precision {prec} ({n} steps/orbit) tiles {sol.sh_tiles()}: {errs}")
        sol.close()


def test_batch_members_levels_4_to_6(tmp_path, built):
    """Batch members on levels 4, 5 and 6 from the sweep's distribution, thick oceans (up to 100 km) at their
    stable step counts, against the FP64 oracle member by member: power within 1e-4, state within 1e-3."""
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    angvel, P, _, _ = O.derive_time(ANGVEL_IN, 59.197)
    levels = (4, 5, 6)
    paths, meshes = [], []
    for lv in levels:
        paths.append(tmp_path / f"grid_{lv}.txt")
        g.generate_grid_file(lv, paths[-1])
        meshes.append(g.Mesh.from_file(paths[-1], RADIUS))
    rng = np.random.default_rng(21)
    members = []
    for k in range(9):
        mi = k % 3
        h = float(10 ** rng.uniform(2.0, 5.0)) if k < 6 else 1e5          # the last three: 100 km
        spo = max(2000, g.stable_steps_per_orbit(P, meshes[mi].gravity_wave_omega(GRAV, h), 0.95))
        spo += spo % 2
        members.append(dict(mesh=mi, steps_per_orbit=int(spo), h=h, alpha=float(10 ** rng.uniform(-7, -4)),
                            ecc=float(rng.uniform(0.001, 0.01)), obliq=float(np.deg2rad(rng.uniform(0.0, 0.5)))))
    common = g.make_params(radius=RADIUS, g=GRAV, angvel=angvel, h=1.0, alpha=0.0, dt=1.0, potential=g.POT_FULL)
    b = g.Batch(common, meshes, members)
    steps = 800
    _, sp = b.run(steps=steps, step_power=True)
    omeshes = [O.OracleMesh(pth, RADIUS) for pth in paths]
    for i, m in enumerate(members):
        orc = O.OracleSolver(omeshes[m["mesh"]], radius=RADIUS, g=GRAV, angvel=angvel, h=m["h"],
                             alpha=m["alpha"], ecc=m["ecc"], obliq=m["obliq"], dt=P / m["steps_per_orbit"],
                             potential=O.FULL)
        po = orc.run(steps)
        _, vo, eo, _, _ = orc.get_state()
        it, vg, eg = b.get_member(i)
        assert it == steps
        assert rel_err(sp[i, steps // 2:], po[steps // 2:]) < 1e-4, (i, m)
        assert rel_err(eg, eo) < 1e-3 and rel_err(vg, vo) < 1e-3, (i, m)
    b.close()
