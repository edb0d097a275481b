"""Failure detection without a GPU fault: the bounded device waits run out and the host reads the status.

The persistent loop waits on its neighbour CTAs' step flags and the batch kernel on grid barriers; every
wait has a poll limit, after which the CTA records ODIS_ERR_TIMEOUT and leaves its kernel.  A test hook
(odis_set_wait_limit / odis_batch_set_wait_limit) shortens the limit and makes one CTA withhold its flag or
barrier arrival, so that the waits on it run out by construction: nothing faults, traps or hangs, and the
context must run clean steps afterwards.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ANGVEL_IN, GRAV, RADIUS, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 2])
def test_persistent_loop_wait_runs_out(grid_dir, precision):
    import geodesicodis_gb300 as g
    from conftest import ecc_case_params
    path = grid_dir / "grid_4.txt"
    mesh = g.Mesh.from_file(path, RADIUS)
    a = g.Solver(g.make_params(precision=precision, **ecc_case_params()), mesh)
    b = g.Solver(g.make_params(precision=precision, **ecc_case_params()), mesh)
    assert a.set_persistent(True) and b.set_persistent(True)
    a.run(50)
    state = a.get_state()
    a.set_wait_limit(4096, 3)                 # CTA 3 publishes nothing; waits give up after 4096 polls
    with pytest.raises(g.OdisError) as ei:
        a.run(100)
    assert ei.value.code == g.ERR_TIMEOUT
    # the context is still usable: restore the state, lift the hook, and it matches an undisturbed run
    a.set_wait_limit(0, -1)
    a.set_state(*state)
    pa = a.run(200)
    b.run(50)
    pb = b.run(200)
    # FP64 state round-trips exactly; the double-float pairs through FP64 to within their own rounding
    tol = 0.0 if precision == 0 else 1e-12
    assert rel_err(pa, pb) <= tol
    for x, y in zip(a.get_state()[1:], b.get_state()[1:]):
        assert rel_err(x, y) <= tol
    a.close()
    b.close()


def test_batch_barrier_wait_runs_out(grid_dir, monkeypatch):
    import geodesicodis_gb300 as g
    monkeypatch.setenv("ODIS_BATCH_ROWS", "2")      # both batches run the same kernel variant
    from oracle import pyoracle as O
    angvel, P, _, _ = O.derive_time(ANGVEL_IN, 59.197)
    meshes = [g.Mesh.from_file(grid_dir / f"grid_{lv}.txt", RADIUS) for lv in (2, 3)]
    rng = np.random.default_rng(4)
    members = [dict(mesh=i % 2, steps_per_orbit=2000, h=float(10 ** rng.uniform(3.0, 4.0)),
                    alpha=float(10 ** rng.uniform(-7, -4)), ecc=float(rng.uniform(0.001, 0.01)),
                    obliq=float(np.deg2rad(rng.uniform(0.0, 0.5)))) for i in range(6)]
    common = g.make_params(radius=RADIUS, g=GRAV, angvel=angvel, h=1.0, alpha=0.0, dt=1.0, potential=g.POT_FULL)
    a = g.Batch(common, meshes, members)
    b = g.Batch(common, meshes, members)
    a.set_wait_limit(4096, 1)                 # CTA 1 never arrives at a grid barrier
    with pytest.raises(g.OdisError) as ei:
        a.run(steps=100)
    assert ei.value.code == g.ERR_TIMEOUT
    a.set_wait_limit(0, -1)
    for i in range(len(members)):             # restart every member from rest, as the undisturbed batch
        a.set_member(i, None, None)
    _, pa = a.run(steps=300, step_power=True)
    _, pb = b.run(steps=300, step_power=True)
    np.testing.assert_array_equal(pa, pb)
    for i in range(len(members)):
        np.testing.assert_array_equal(a.get_member(i)[1], b.get_member(i)[1])
    a.close()
    b.close()
