"""friction type QUADRATIC on the GPU against the FP64 oracle.

In the reference the friction type changes only what updateEnergy reports
(src/energy.cpp:45-53: e_e = alpha / h |u| |u|^2 instead of alpha 1000 h |u|^2);
the momentum equation keeps the linear drag -alpha v in both.  So the state
after N steps is the LINEAR run's, and the power series is the quadratic one.

Tolerances are those of the LINEAR parity tests: 1e-14 / 1e-12 for the
per-operator call, 1e-10 for the FP64 and double-float time loops, 1e-4 for the
FP32-state method's power.
"""
import numpy as np
import pytest

from conftest import RADIUS, ecc_case_params, rel_err

pytestmark = pytest.mark.gpu


def _pair(path, precision=0, **over):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    p = ecc_case_params(**over)
    orc = O.OracleSolver(O.OracleMesh(path, RADIUS), **p)
    gp = g.make_params(precision=precision, **p)
    return orc, g.Solver(gp, g.Mesh.from_file(path, RADIUS))


def test_quadratic_update_energy(grid_dir):
    orc, gpu = _pair(grid_dir / "grid_3.txt", friction=1)
    uv = np.random.default_rng(21).standard_normal((orc.E, 2)) * 0.05
    a_o, e_o = orc.updateEnergy(uv)
    a_g, e_g = gpu.updateEnergy(uv)
    assert rel_err(e_g, e_o) < 1e-14
    assert abs(a_g - a_o) / abs(a_o) < 1e-12
    # the |u|^3 branch, not the |u|^2 one: alpha / h |u|^3 per face
    q = (uv ** 2).sum(axis=1)
    p = ecc_case_params()
    np.testing.assert_allclose(e_g, p["alpha"] / p["h"] * np.sqrt(q) * q, rtol=1e-14)


@pytest.mark.parametrize("precision", [0, 2])
def test_quadratic_fused_loop_parity(grid_dir, precision):
    orc, gpu = _pair(grid_dir / "grid_3.txt", precision=precision, friction=1)
    po, pg = orc.run(2500), gpu.run(2500)
    _, vo, eo, _, _ = orc.get_state()
    it, vg, eg, _, _ = gpu.get_state()
    assert it == 2500
    assert rel_err(eg, eo) < 1e-10 and rel_err(vg, vo) < 1e-10
    assert rel_err(pg, po) < 1e-10
    # same state as a LINEAR run, different reported power
    orc_l, _ = _pair(grid_dir / "grid_3.txt", precision=precision)
    pl = orc_l.run(2500)
    assert rel_err(orc_l.get_state()[1], vo) == 0.0
    assert rel_err(pl, po) > 0.5


@pytest.mark.parametrize("precision", [0, 2])
def test_quadratic_persistent_loop(grid_dir, precision):
    orc, a = _pair(grid_dir / "grid_4.txt", precision=precision, friction=1)
    assert a.set_persistent(True) is True
    pa = np.concatenate([a.run(37), a.run(300)])
    assert rel_err(pa, orc.run(337)) < 1e-10


def test_quadratic_fp32_power(grid_dir):
    orc, gpu = _pair(grid_dir / "grid_3.txt", precision=1, friction=1)
    po, pg = orc.run(4000), gpu.run(4000)
    assert rel_err(pg[-2000:], po[-2000:]) < 1e-4


@pytest.mark.parametrize("precision", [0, 2])
def test_quadratic_advective_loop(grid_dir, precision):
    orc, gpu = _pair(grid_dir / "grid_3.txt", precision=precision, advection=1, friction=1)
    po, pg = orc.run(400), gpu.run(400)
    assert rel_err(pg, po) < 1e-10
    _, vo, eo, _, _ = orc.get_state()
    _, vg, eg, _, _ = gpu.get_state()
    assert rel_err(eg, eo) < 1e-10 and rel_err(vg, vo) < 1e-10
