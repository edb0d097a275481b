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


def test_quadratic_friction_reaches_params(built, tmp_path):
    """friction type QUADRATIC (src/globals.cpp:232-234) selects updateEnergy's |u|^3 branch
    (src/energy.cpp:45-53) through odis_params.friction; LINEAR is the other value."""
    import geodesicodis_gb300 as g
    f = tmp_path / "input.in"
    f.write_text(INPUT_IN.replace("friction type; \t \t     LINEAR;", "friction type; \t \t     QUADRATIC;"))
    assert "QUADRATIC" in f.read_text()
    inp = g.read_input(f)
    assert inp.fric_linear == 0 and inp.params.friction == 1
    f.write_text(INPUT_IN)
    assert g.read_input(f).params.friction == 0


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


OUTPUT_KEYS = """dissipation output; 	      true; 	 	 	 data out opt;
dissipation avg output;       true; 	 	 	 data out opt;
kinetic avg output; 	      true; 	 	 	 data out opt;
displacement output; 	 	  true; 	 	 	 data out opt;
velocity output; 	 	 	  true; 	 	 	 data out opt;
velocity cartesian output; 	 	  true; 	 	 	 data out opt;
dummy1 output;                true;                  div;
"""


@pytest.mark.gpu
def test_cli_device_mesh(built, tmp_path):
    """--device-mesh builds the grid and mesh on the GPU: the same run as the host-built mesh, power to the
    geometry's conditioning at this level (grid level 3 of input.in, 642 cells)."""
    outs = []
    for extra, name in (([], "host"), (["--device-mesh"], "device")):
        (tmp_path / name).mkdir()
        d = _rundir(tmp_path / name)
        r = subprocess.run([str(CLI), "--dir", str(d), "--orbits", "0.1", *extra], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        outs.append(np.loadtxt(d / "DATA" / "power.txt", ndmin=2))
    assert outs[0].shape == outs[1].shape
    assert np.max(np.abs(outs[1][:, 1] - outs[0][:, 1])) <= 1e-10 * np.max(np.abs(outs[0][:, 1]))


@pytest.mark.gpu
def test_cli_writes_data_h5(built, tmp_path):
    """DATA/data.h5 in the reference's layout (src/outFiles.cpp:138-823), read back with the
    specification reader: one row per dump (the initial state, then every output interval), each
    row the float32 of the library's own operators on the state at that dump."""
    import geodesicodis_gb300 as g
    import h5read
    d = _rundir(tmp_path)
    (d / "input.in").write_text((d / "input.in").read_text() + OUTPUT_KEYS)
    r = subprocess.run([str(CLI), "--dir", str(d), "--orbits", "0.2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = (d / "OUTPUT.txt").read_text().splitlines()
    assert lines[0].startswith("DUMPING DATA AT 0.000000 AVG DISS:") and lines[0].endswith("GW1")
    assert lines[-1].endswith("GW3")
    inp = g.read_input(d / "input.in")
    mesh = g.Mesh.generate(inp.grid_level - 1, inp.params.radius)
    N, E = mesh.n_cells, mesh.n_edges
    ds = h5read.H5File(d / "DATA" / "data.h5").datasets()
    T = 3                                      # 0.2 orbits at 10 dumps per orbit, plus the initial dump
    shapes = {"east velocity": (T, E), "north velocity": (T, E), "x velocity": (T, N), "y velocity": (T, N),
              "z velocity": (T, N), "displacement": (T, N), "dissipated energy": (T, E),
              "dissipation avg output": (T,), "kinetic avg output": (T,), "dummy1 output": (T, N),
              "face longitude": (E,), "face latitude": (E,)}
    assert {k: v.shape for k, v in ds.items()} == shapes
    a = {k: v.read() for k, v in ds.items()}
    sol = g.Solver(inp.params, mesh)
    for t in range(T):
        if t:
            sol.run(200)
        _, v, eta, _, _ = sol.get_state()
        uv = sol.interpolateVelocity(v)
        avg, e = sol.updateEnergy(uv)
        ux = sol.interpolateVelocityCart(v)
        for name, ref in (("east velocity", uv[:, 0]), ("north velocity", uv[:, 1]), ("displacement", eta),
                          ("x velocity", ux[:, 0]), ("y velocity", ux[:, 1]), ("z velocity", ux[:, 2]),
                          ("dissipated energy", e)):
            scale = max(np.max(np.abs(ref)), 1e-30)
            assert np.max(np.abs(a[name][t] - ref.astype(np.float32))) <= 1e-6 * scale, (name, t)
        assert a["dissipation avg output"][t] == pytest.approx(avg, rel=1e-6, abs=1e-30)
        assert a["kinetic avg output"][t] == np.float32(t * 200 * inp.params.dt)
    assert not a["dummy1 output"].any()
    np.testing.assert_array_equal(a["face latitude"], (mesh.field(4).astype(np.float32).astype(np.float64) * 180.0
                                                        / np.pi).astype(np.float32))
    np.testing.assert_array_equal(a["face longitude"], (mesh.field(5).astype(np.float32).astype(np.float64) * 180.0
                                                         / np.pi).astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_cli_nonlinear_run(built, tmp_path, precision):
    """The reference's default mode, advection true, through the driver in FP64 and in double-float:
    the final state equals the library's run of the same steps, and DATA/data.h5 holds the dumps."""
    import geodesicodis_gb300 as g
    import h5read
    d = _rundir(tmp_path)
    text = (d / "input.in").read_text().replace("advection;                     false;",
                                                "advection;                     true;")
    assert "advection;                     true;" in text
    (d / "input.in").write_text(text + OUTPUT_KEYS)
    r = subprocess.run([str(CLI), "--dir", str(d), "--orbits", "0.1", "--precision", precision],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = g.read_input(d / "input.in")
    assert inp.params.advection == 1
    mesh = g.Mesh.generate(inp.grid_level - 1, inp.params.radius)
    p = inp.params
    p.precision = g.DF64 if precision == "df64" else g.FP64
    sol = g.Solver(p, mesh)
    sol.run(200, power=False)
    _, v, eta, _, _ = sol.get_state()
    vf = np.loadtxt(d / "InitialConditions" / "vel_init.txt", delimiter=",")[:, 0]
    assert np.max(np.abs(vf - v)) <= 1e-6 * np.max(np.abs(v))
    ds = h5read.H5File(d / "DATA" / "data.h5").datasets()
    assert ds["displacement"].shape == (2, mesh.n_cells)
    last = ds["displacement"].read()[1]
    assert np.max(np.abs(last - eta.astype(np.float32))) <= 1e-6 * np.max(np.abs(eta))


@pytest.mark.gpu
def test_cli_sigint_checkpoint_and_exact_resume(built, tmp_path):
    """SIGINT (CatchExit, src/timeIntegrator.cpp:32-37, 307-316): the run stops within one step chunk, writes
    "Terminate signal caught..." to OUTPUT.txt, saves InitialConditions (the reference's text files and the
    exact FP64 state.bin) and exits with status 1.  --resume continues from state.bin and ends on the same
    state bits as an uninterrupted run of the same length."""
    import signal
    import struct
    orbits = "100"
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    a = _rundir(tmp_path / "a")
    r = subprocess.run([str(CLI), "--dir", str(a), "--orbits", orbits], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    b = _rundir(tmp_path / "b")
    p = subprocess.Popen([str(CLI), "--dir", str(b), "--orbits", orbits], stdout=subprocess.PIPE,
                         stderr=subprocess.PIPE, text=True)
    seen = 0
    for line in p.stdout:
        seen += line.startswith("DUMPING DATA AT")
        if seen == 4:                         # the initial dump and three orbits
            p.send_signal(signal.SIGINT)
            break
    out, err = p.communicate(timeout=600)
    assert p.returncode == 1, err
    assert "Caught Terminate Signal..." in out and "Terminate signal caught..." in out
    assert "Terminate signal caught..." in (b / "OUTPUT.txt").read_text()
    ckp = (b / "InitialConditions" / "state.bin").read_bytes()
    assert ckp[:8] == b"ODISCKP1"
    steps_done = struct.unpack("<q", ckp[8:16])[0]
    assert 0 < steps_done < 100 * 2000
    assert (b / "InitialConditions" / "vel_init.txt").exists()
    r = subprocess.run([str(CLI), "--dir", str(b), "--orbits", orbits, "--resume"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ca = (a / "InitialConditions" / "state.bin").read_bytes()
    cb = (b / "InitialConditions" / "state.bin").read_bytes()
    assert struct.unpack("<q", ca[8:16])[0] == struct.unpack("<q", cb[8:16])[0] == 100 * 2000
    assert ca == cb
