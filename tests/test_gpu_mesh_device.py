"""Grid generation and mesh build on the GPU (odis_mesh_generate_device, odis_mesh_from_*_device,
odis_grid_generate_arrays) against the host build, which the CPU tests pin bit for bit to the oracle.

* Integer arrays (numbering, friends, faces, TRiSK stencils, vertex topology): identical.
* Floating-point arrays: they differ only where CUDA's sin/cos/acos/asin/atan2 round differently from the
  C library's in the last bit, and the reference's formulas amplify that: the cosine-law spherical excess
  behind the kite fractions and TRiSK weights moves by ~1e-10 (level 4), 3e-8 (level 6) and 1e-5 (level 8)
  when the host build's inputs move by one ulp.  The bound is ten times that host-side sensitivity,
  measured in the test itself.
* A run on the device-built mesh against the FP64 oracle on the host-generated grid file: 1e-10 at level 4.
* Malformed input is rejected with ODIS_ERR_MESH before any kernel indexes it.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import RADIUS, rel_err

pytestmark = pytest.mark.gpu


def _ulp_sensitivity(level, seed=0):
    """Largest relative change of the host-built geometry when a random half of the input coordinates moves
    by one ulp: the conditioning of the reference's formulas at this level."""
    import geodesicodis_gb300 as g
    nd, fr, cd = g.generate_grid(level)
    ns, cs = nd * (np.pi / 180), cd * (np.pi / 180)
    rng = np.random.default_rng(seed)

    def bump(x):
        pick = (rng.random(x.shape) < 0.5) & (x != -np.pi / 180)
        return np.where(pick, np.nextafter(x, np.where(rng.random(x.shape) < 0.5, np.inf, -np.inf)), x)
    a = g.Mesh.from_arrays(ns, fr, cs, RADIUS)
    rel, bad = g.Mesh.from_arrays(bump(ns), fr, bump(cs), RADIUS).compare(a)
    assert bad == 0
    return rel


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5, 6, 7])
def test_device_grid_matches_host(built, level):
    import geodesicodis_gb300 as g
    nh, fh, ch = g.generate_grid(level)
    nd, fd, cd = g.generate_grid(level, device=True)
    np.testing.assert_array_equal(fd, fh)
    # degrees; atan2's last bit at 360 degrees is 6e-14
    dn, dc = np.abs(nd - nh), np.abs(cd - ch)
    dn[:, 1] = np.minimum(dn[:, 1], np.abs(dn[:, 1] - 360.0))
    dc[..., 1] = np.minimum(dc[..., 1], np.abs(dc[..., 1] - 360.0))
    same = float(np.mean(nd == nh)), float(np.mean(cd == ch))
    print(f"level {level}: coordinates bit-identical: nodes {same[0]:.4f}, vertices {same[1]:.4f}; "
          f"largest difference {max(dn.max(), dc.max()):.1e} deg")
    assert dn.max() < 1e-12 and dc.max() < 1e-12


@pytest.mark.parametrize("level", [2, 4, 6])
def test_device_build_matches_host(built, tmp_path, level):
    import geodesicodis_gb300 as g
    path = tmp_path / f"grid_{level}.txt"
    g.generate_grid_file(level, path)
    host = g.Mesh.from_file(path, RADIUS)
    dev = g.Mesh.from_file(path, RADIUS, device=True)
    bound = 10 * _ulp_sensitivity(level) + 1e-14
    rel, bad = dev.compare(host)
    print(f"level {level} build on the device vs host: integer mismatches {bad}, geometry {rel:.2e} (bound {bound:.1e})")
    assert bad == 0 and rel < bound
    gen = g.Mesh.generate(level, RADIUS, device=True)
    rel, bad = gen.compare(host)
    print(f"level {level} generate + build on the device vs host file: integer mismatches {bad}, geometry {rel:.2e}")
    assert bad == 0 and rel < bound


def test_level8_device_setup_time(built):
    """Level 8 (655362 cells): device generate + build against the host's, same mesh; times printed."""
    import geodesicodis_gb300 as g
    g.Mesh.generate(2, RADIUS, device=True)                 # context and module load outside the timing
    t = time.perf_counter()
    dev = g.Mesh.generate(8, RADIUS, device=True)
    td = time.perf_counter() - t
    t = time.perf_counter()
    host = g.Mesh.generate(8, RADIUS)
    th = time.perf_counter() - t
    rel, bad = dev.compare(host)
    bound = 10 * _ulp_sensitivity(8)
    print(f"level 8 generate + build: device {td:.3f} s, host {th:.3f} s; integer mismatches {bad}, "
          f"geometry {rel:.2e} (bound {bound:.1e})")
    assert bad == 0 and rel < bound


def test_run_on_device_mesh_against_oracle(built, tmp_path):
    """FP64 LTE run (ECC tide, SH l_max 8) on the device-built level-4 mesh against the oracle on the file:
    1e-10 after 1500 steps (the TRiSK weights differ from the host's by ~1e-10 at this level; the run by
    ~2e-11 on the GB300)."""
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    path = tmp_path / "grid_4.txt"
    g.generate_grid_file(4, path)
    angvel, P, dt, n = O.derive_time(5.307e-5, 59.197)
    p = dict(radius=RADIUS, g=0.113, angvel=angvel, h=1e4, alpha=1e-5, ecc=0.0047, dt=dt, potential=O.ECC,
             sh_lmax=8, sh_factors=O.benchmark_sh_factors(0.113, RADIUS, 8, seed=1))
    orc = O.OracleSolver(O.OracleMesh(path, RADIUS), **p)
    po = orc.run(1500)
    _, vo, eo, _, _ = orc.get_state()
    sol = g.Solver(g.make_params(precision=g.FP64, **p), g.Mesh.generate(4, RADIUS, device=True))
    pg = sol.run(1500)
    _, vg, eg, _, _ = sol.get_state()
    errs = rel_err(eg, eo), rel_err(vg, vo), rel_err(pg, po)
    print(f"device mesh, level 4, 1500 steps: eta {errs[0]:.2e} v {errs[1]:.2e} power {errs[2]:.2e}")
    assert max(errs) < 1e-10
    sol.close()


def test_malformed_arrays_rejected(built):
    import geodesicodis_gb300 as g
    nd, fr, cd = g.generate_grid(2)
    ns, cs = np.deg2rad(nd), np.deg2rad(cd)
    bad = fr.copy()
    bad[7, 2] = len(nd) + 5                                  # a friend outside the mesh
    with pytest.raises(g.OdisError):
        g.Mesh.from_arrays(ns, bad, cs, RADIUS, device=True)
    bad = fr.copy()
    bad[7, 2] = bad[7, 3]                                    # a repeated friend: no consistent numbering
    with pytest.raises(g.OdisError):
        g.Mesh.from_arrays(ns, bad, cs, RADIUS, device=True)
    g.Mesh.from_arrays(ns, fr, cs, RADIUS, device=True)      # and the context still builds a good mesh
