"""The run driver odis_run (C++ over the C ABI): input.in in, OUTPUT.txt / DATA / InitialConditions out."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_capi import INPUT_IN

CLI = ROOT / "geodesicodis_gb300" / "bin" / "odis_run"


def test_cli_is_built_and_rejects_bad_arguments(built):
    assert CLI.exists()
    r = subprocess.run([str(CLI), "--nope"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def _rundir(tmp_path, init="NONE"):
    d = tmp_path / "run"
    d.mkdir(exist_ok=True)
    text = INPUT_IN.replace("Geodesic Grid Level; \t \t \t5;", "Geodesic Grid Level; \t \t \t3;")
    text = text.replace("initial conditions; \t      NONE;", f"initial conditions; \t      {init};")
    (d / "input.in").write_text(text)
    return d


def _read(path):
    a = np.loadtxt(path, delimiter=",")
    return a[:, 0], a[:, 1:]


@pytest.mark.gpu
def test_cli_run_and_restart_match_the_library(built, tmp_path):
    import geodesicodis_gb300 as g
    d = _rundir(tmp_path)
    r = subprocess.run([str(CLI), "--dir", str(d), "--orbits", "0.1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = (d / "OUTPUT.txt").read_text().splitlines()
    assert lines[-1].startswith("DUMPING DATA AT 0.100000 AVG DISS:")
    inp = g.read_input(d / "input.in")
    mesh = g.Mesh.generate(inp.grid_level - 1, inp.params.radius)
    sol = g.Solver(inp.params, mesh)
    pw = sol.run(200)
    _, v, eta, dv, de = sol.get_state()
    vf, dvf = _read(d / "InitialConditions" / "vel_init.txt")
    ef, def_ = _read(d / "InitialConditions" / "pres_init.txt")
    assert np.max(np.abs(vf - v)) <= 1e-6 * np.max(np.abs(v))
    assert np.max(np.abs(ef - eta)) <= 1e-6 * np.max(np.abs(eta))
    data = np.loadtxt(d / "DATA" / "power.txt", ndmin=2)
    assert abs(data[-1, 1] / pw.mean() - 1) < 1e-12
    nodes = np.loadtxt(d / "DATA" / "final_nodes.txt")
    ux = sol.interpolateVelocityCart(v)
    assert np.max(np.abs(nodes[:, 1:] - ux)) <= 1e-8 * np.max(np.abs(ux))
    # restart from the written state (initial conditions LOAD) against the library run from the same numbers
    d2 = _rundir(tmp_path, "LOAD")
    r = subprocess.run([str(CLI), "--dir", str(d2), "--orbits", "0.1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp2 = g.read_input(d2 / "input.in")
    sol2 = g.Solver(inp2.params, mesh)
    sol2.set_state(0, vf, ef, dvf, def_)
    sol2.run(200)
    _, v2, eta2, _, _ = sol2.get_state()
    vf2, _ = _read(d2 / "InitialConditions" / "vel_init.txt")
    assert np.max(np.abs(vf2 - v2)) <= 1e-6 * np.max(np.abs(v2))
