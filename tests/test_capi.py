"""C ABI surface (no GPU needed): exported symbols, input.in parsing, error codes."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ANGVEL_IN, ROOT

HEADER = ROOT / "include" / "odis_gpu.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(odis_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    import geodesicodis_gb300 as g
    L = C.CDLL(str(g.LIB_PATH))
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_header_is_plain_c(built, tmp_path):
    import subprocess
    src = tmp_path / "t.c"
    src.write_text('#include "odis_gpu.h"\nint main(void){ odis_params p; (void)p; return 0; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-c", str(src),
                    "-o", str(tmp_path / "t.o")], check=True)


INPUT_IN = """radius; 	 	 	         252.1e3;  	 	 top radius 	;
k2; 	 	 	                   0.0; 	 	 	 k2 Love number;
h2; 	 	 	                   0.0; 	 	 	 h2 Love number;
love reduction factor;          1.0;                U prefactor;
angular velocity;      	5.307e-5; 	 	 	 Spin rate/mean motion;
surface gravity;    	0.113; 	 	 	 gravity;
eccentricity; 	     	 	  0.0047; 	 	 	 e;
obliquity; 	 	 	          0.2; 	 	 	 theta;
orbital period;     	1.0; 	 	 	 P;
ocean thickness;    	     1e4; 	 	 	 h_o;
friction coefficient;      1e-5; 	 	 	 alpha;
friction type; 	 	     LINEAR; 	 	 	 friction;
potential; 	 	 	      ECC; 	 	 	 potential;
surface type; 	          FREE; 	 	 	 top boundary condition;
advection;                     false;             advection switch;
solver type; 	 	 	        AB3; 	 	 	 potential;
Geodesic Grid Level; 	 	 	5; 	 	 	 recursion level;
output time; 	 	 	      10; 	 	 	 data out opt;
unknown key;    42;     skipped;
initial conditions; 	      NONE; 	 	 	 use initial conditions;
simulation end time; 	 	  10;	 	 	 endTime;
time step; 	 	 	          59.197; 	 	 	 timeStep;
"""


def test_input_in_semantics(built, tmp_path):
    import geodesicodis_gb300 as g
    f = tmp_path / "input.in"
    f.write_text(INPUT_IN)
    inp = g.read_input(f)
    p = inp.params
    assert inp.period == 118394.0                                  # rounded, 'orbital period' ignored
    assert p.angvel == 2 * np.pi / 118394.0
    assert inp.steps_per_orbit == 2000 and p.dt == 118394.0 / 2000
    assert p.obliq == 0.2 * np.pi / 180.0                          # degrees -> radians
    assert p.love_reduct == 1.0 and p.potential == g.POT_ECC
    assert inp.grid_level == 5                                     # keys are case-insensitive
    assert inp.advection == 0 and inp.params.advection == 0 and inp.fric_linear == 1 and inp.init_kind == 0
    assert p.radius == 252.1e3 and p.h == 1e4 and p.alpha == 1e-5 and p.g == 0.113
    assert inp.end_time == 10 and inp.output_time == 10


def test_input_in_bad_enum_and_missing_file(built, tmp_path):
    import geodesicodis_gb300 as g
    f = tmp_path / "input.in"
    f.write_text(INPUT_IN.replace("ECC;", "NOT_A_TIDE;"))
    with pytest.raises(g.OdisError) as e:
        g.read_input(f)
    assert e.value.code == g.ERR_ARG
    with pytest.raises(g.OdisError) as e:
        g.read_input(tmp_path / "nope.in")
    assert e.value.code == g.ERR_IO


def test_reference_input_in_parses(built):
    """The reference's own input.in (OBLIQ_WEST, advection true) parses with its documented values."""
    import geodesicodis_gb300 as g
    from conftest import ref_file
    src = ref_file("input.in")
    inp = g.read_input(src)
    assert inp.params.potential == g.POT_OBLIQ_WEST
    assert inp.advection == 1 and inp.params.advection == 1 and inp.grid_level == 6
    assert inp.params.obliq == -2.0 * np.pi / 180.0
    assert inp.period == 2 * round(2 * np.pi / 7.292e-5 / 2)


def test_derive_time_rejects_bad_args(built):
    import geodesicodis_gb300 as g
    with pytest.raises(g.OdisError):
        g.derive_time(-1.0, 10.0)
    a, P, dt, n = g.derive_time(ANGVEL_IN, 29.5985)
    assert n == 4000 and dt == P / 4000


@pytest.mark.gpu
def test_forcing_takes_the_reference_enum(tmp_path, built):
    """odis_forcing bound with plain ctypes, called as the reference's time loop calls forcing(): the type is
    globals->tide_type, a value of enum Potential (include/globals.h:60-76: OBLIQ 0, OBLIQ_WEST 1, ECC 5,
    FULL 8, FULL2 9), and the eccentricity and obliquity are explicit arguments."""
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    L = C.CDLL(str(g.LIB_PATH))
    L.odis_forcing.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]
    path = tmp_path / "grid_3.txt"
    g.generate_grid_file(3, path)
    angvel, P, dt, n = g.derive_time(ANGVEL_IN, 59.197)
    sol = g.Solver(g.make_params(radius=252.1e3, g=0.113, angvel=angvel, h=1e4, alpha=1e-5, ecc=0.0,
                                 obliq=0.0, dt=dt, potential=5), g.Mesh.from_file(path, 252.1e3))
    orc = O.OracleSolver(O.OracleMesh(path, 252.1e3), radius=252.1e3, g=0.113, angvel=angvel, h=1e4,
                         alpha=1e-5, dt=dt)
    for tide_type in (5, 0, 1, 8, 9):                 # ECC, OBLIQ, OBLIQ_WEST, FULL, FULL2
        U = np.zeros(orc.N)
        st = L.odis_forcing(sol._h, U.ctypes.data, tide_type, 4321.0, 0.0047, 0.0087, g.MEM_HOST)
        assert st == 0
        ref = orc.forcing(tide_type, 4321.0, 0.0047, 0.0087)
        assert np.max(np.abs(ref)) > 0
        assert np.max(np.abs(U - ref)) <= 1e-12 * np.max(np.abs(ref)), tide_type
    assert L.odis_forcing(sol._h, U.ctypes.data, 17, 0.0, 0.0, 0.0, g.MEM_HOST) == g.ERR_ARG
    sol.close()
