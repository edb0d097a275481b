"""The reference's analytical LTE solution (src/analyticalLTE.cpp:22-181, case OBLIQ_WEST) and its
"initial conditions ANALYTICAL" (src/initialConditions.cpp:150-211).

* The product's closed form (odis_analytical_state, C++) against the oracle's numpy restatement.
* Physics pin of the discrete loop: without drag the closed form solves the continuous equations
  exactly, and the FP64 loop started from it stays on it with an error that falls at second order
  in the grid spacing (oracle on the CPU; the product's methods on the GPU, at finer grids) and at
  first order in the time step (the forcing term's treatment in the reference's loop).
"""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ANGVEL_IN, GRAV, RADIUS


def _params(**over):
    from oracle import pyoracle as O
    angvel, P, dt, n = O.derive_time(ANGVEL_IN, 59.197)
    p = dict(radius=RADIUS, g=GRAV, angvel=angvel, h=1e4, alpha=0.0, ecc=0.0, obliq=0.01, love_reduct=1.0,
             dt=dt, potential=O.OBLIQ_WEST, init_load=0)
    p.update(over)
    return p, n


def _oracle_state(om, p, t):
    from oracle import lte_analytic as A
    ap = {k: p[k] for k in ("radius", "g", "angvel", "h", "alpha")} | {"obliq": p["obliq"]}
    return A.state(om.field(4), om.field(5), om.field(8), om.field(9), om.field(12), om.field(13), t, p["dt"], **ap)


@pytest.mark.parametrize("level,alpha", [(2, 0.0), (3, 1e-5), (4, 1e-6)])
def test_closed_form_matches_oracle(grid_dir, level, alpha):
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    p, n = _params(alpha=alpha, h=3e3)
    path = grid_dir / f"grid_{level}.txt"
    om = O.OracleMesh(path, RADIUS)
    gm = g.Mesh.from_file(path, RADIUS)
    for t in (0.0, 0.3 * n * p["dt"]):
        got = g.analytical_state(g.make_params(**p), gm, t)
        ref = _oracle_state(om, p, t)
        for a, b in zip(got, ref):
            assert np.max(np.abs(a - b)) <= 1e-12 * max(np.max(np.abs(b)), 1e-300)


def test_closed_form_only_for_obliq_west(grid_dir):
    import geodesicodis_gb300 as g
    p, _ = _params(potential=g.POT_ECC)
    with pytest.raises(g.OdisError) as ei:
        g.analytical_state(g.make_params(**p), g.Mesh.from_file(grid_dir / "grid_2.txt", RADIUS))
    assert ei.value.code == g.ERR_ARG


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_oracle_converges_to_closed_form(grid_dir):
    """One orbit from the undamped closed-form state, levels 2-4: the velocity error falls by close to
    4x per level (second order), and is below 1 % at level 4."""
    from oracle import pyoracle as O
    p, n = _params()
    errs = []
    for level in (2, 3, 4):
        om = O.OracleMesh(grid_dir / f"grid_{level}.txt", RADIUS)
        orc = O.OracleSolver(om, **p)
        orc.set_state(0, *_oracle_state(om, p, 0.0))
        orc.run(n)
        _, v, _, _, _ = orc.get_state()
        errs.append(_rel(v, _oracle_state(om, p, n * p["dt"])[0]))
    assert errs[0] / errs[1] > 3.2 and errs[1] / errs[2] > 3.2, errs
    assert errs[2] < 0.01, errs


def _product_error(level, steps, precision):
    import geodesicodis_gb300 as g
    p, n = _params(h=1e3)
    p["dt"] = p["dt"] * n / steps
    mesh = g.Mesh.generate(level, RADIUS)
    gp = g.make_params(precision=getattr(g, precision), **p)
    sol = g.Solver(gp, mesh)
    sol.set_state(0, *g.analytical_state(gp, mesh, 0.0))
    sol.run(steps, power=False)
    _, v, _, _, _ = sol.get_state()
    return _rel(v, g.analytical_state(gp, mesh, steps * p["dt"])[0])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["FP64", "DF64"])
def test_product_converges_to_closed_form_in_space(precision):
    """The pin through the product at levels 4-6 (h = 1 km), one orbit of 32000 steps so that the
    time error stays below the space error: the velocity error falls 4x per level (measured on a
    GB300: 5.9e-3, 1.5e-3, 3.7e-4)."""
    errs = [_product_error(level, 32000, precision) for level in (4, 5, 6)]
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5, errs
    assert errs[2] < 5e-4, errs


@pytest.mark.gpu
def test_product_time_error_is_first_order():
    """At level 7 the error halves with dt (4000, 8000, 16000 steps per orbit; measured 7.3e-4,
    3.7e-4, 1.9e-4).  The loop adds dt (-alpha v + G U(t + dt)) outside the AB3 sum
    (src/timeIntegrator.cpp:219-224), a first-order treatment of the forcing."""
    errs = [_product_error(7, steps, "FP64") for steps in (4000, 8000, 16000)]
    for a, b in zip(errs, errs[1:]):
        assert 1.7 < a / b < 2.3, errs


@pytest.mark.gpu
def test_cli_analytical_initial_conditions(built, tmp_path):
    """odis_run with "initial conditions ANALYTICAL" and potential OBLIQ_WEST starts from the closed
    form: its final state equals the library's run from g.analytical_state."""
    import geodesicodis_gb300 as g
    from test_capi import INPUT_IN
    from test_cli import CLI
    d = tmp_path / "run"
    d.mkdir()
    text = INPUT_IN.replace("Geodesic Grid Level; \t \t \t5;", "Geodesic Grid Level; \t \t \t4;")
    text = text.replace("initial conditions; \t      NONE;", "initial conditions; \t      ANALYTICAL;")
    text = text.replace("potential; \t \t \t      ECC;", "potential; \t \t \t      OBLIQ_WEST;")
    (d / "input.in").write_text(text)
    r = subprocess.run([str(CLI), "--dir", str(d), "--orbits", "0.1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = g.read_input(d / "input.in")
    assert inp.init_kind == 2 and inp.params.potential == g.POT_OBLIQ_WEST
    mesh = g.Mesh.generate(inp.grid_level - 1, inp.params.radius)
    sol = g.Solver(inp.params, mesh)
    sol.set_state(0, *g.analytical_state(inp.params, mesh, 0.0))
    sol.run(200, power=False)
    _, v, eta, _, _ = sol.get_state()
    vf = np.loadtxt(d / "InitialConditions" / "vel_init.txt", delimiter=",")[:, 0]
    ef = np.loadtxt(d / "InitialConditions" / "pres_init.txt", delimiter=",")[:, 0]
    assert np.max(np.abs(vf - v)) <= 1e-6 * np.max(np.abs(v))
    assert np.max(np.abs(ef - eta)) <= 1e-6 * np.max(np.abs(eta))
