"""ctypes view of the FP64 CPU oracle (odis_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU baseline / reference arm.  The product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libodis_oracle.so"

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p

# forcing types: the values of the reference's enum Potential (include/globals.h:60-76)
(OBLIQ, OBLIQ_WEST, OBLIQ_EAST, ECC_RAD, ECC_LIB, ECC, ECC_WEST, ECC_EAST, FULL, FULL2, TOTAL, ECC_W3, OBLIQ_W3,
 PLANET, PLANET_OBL, GENERAL, NONE) = range(17)


class OrcParams(C.Structure):
    _fields_ = [("radius", C.c_double), ("g", C.c_double), ("angvel", C.c_double), ("h", C.c_double),
                ("alpha", C.c_double), ("ecc", C.c_double), ("obliq", C.c_double), ("love_reduct", C.c_double),
                ("dt", C.c_double), ("potential", C.c_int), ("init_load", C.c_int), ("advection", C.c_int),
                ("friction", C.c_int), ("semimajor_axis", C.c_double), ("fourier_freq", C.c_int)]


_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        sig = {
            "orc_mesh_load": ([C.c_char_p, C.c_double, _I], _V),
            "orc_mesh_from_arrays": ([C.c_int, _D, _I, _D, C.c_double, _I], _V),
            "orc_mesh_free": ([_V], None),
            "orc_mesh_sizes": ([_V, _I, _I, _I], None),
            "orc_mesh_get_field": ([_V, C.c_int, _D], C.c_int),
            "orc_mesh_get_topology": ([_V, _I, _I, _I, _I, _D, _I], None),
            "orc_mesh_get_csr": ([_V, C.c_int, _I, _I, _D], C.c_int),
            "orc_derive_time": ([C.c_double, C.c_double, _D, _D, _D, _I], None),
            "orc_solver_create": ([_V, C.POINTER(OrcParams)], _V),
            "orc_solver_free": ([_V], None),
            "orc_solver_set_loading": ([_V, C.c_int, _D], C.c_int),
            "orc_update_momentum": ([_V, _D, _D, _D], None),
            "orc_update_eta": ([_V, _D, _D], None),
            "orc_forcing": ([_V, _D, C.c_int, C.c_double, C.c_double, C.c_double], None),
            "orc_generate_grid_file": ([C.c_int, C.c_char_p], C.c_int),
            "orc_loading_factors": ([C.c_double, C.c_double, C.c_int, _D], None),
            "orc_ab3": ([C.c_double, _D, _D, C.c_int, C.c_int, C.c_int], None),
            "orc_interpolate_velocity": ([_V, _D, _D], None),
            "orc_interpolate_cartesian": ([_V, _D, _D], None),
            "orc_momentum_advection": ([_V, C.c_double, _D, _D, _D, _D], None),
            "orc_lsq_flux": ([_V, C.c_double, _D, _D, _D], C.c_int),
            "orc_mesh_vertex_field": ([_V, C.c_int, _D], C.c_int),
            "orc_mesh_vertex_topology": ([_V, _I, _I, _I, _I], None),
            "orc_update_energy": ([_V, C.c_double, C.c_double, _D, _D], C.c_double),
            "orc_update_energy_fric": ([_V, C.c_double, C.c_double, C.c_int, _D, _D], C.c_double),
            "orc_plmbar": ([C.c_int, C.c_double, _D], None),
            "orc_sh_basis": ([_V, C.c_int, _D], None),
            "orc_sh_analysis": ([_V, _D, _D], None),
            "orc_sim_create": ([_V], _V),
            "orc_sim_free": ([_V], None),
            "orc_sim_set_state": ([_V, C.c_int, _D, _D, _D, _D], None),
            "orc_sim_get_state": ([_V, _I, _D, _D, _D, _D], None),
            "orc_sim_step": ([_V], C.c_double),
            "orc_sim_run": ([_V, C.c_int, _D], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def derive_time(angvel_in, dt_target):
    a, p, d, n = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    lib().orc_derive_time(angvel_in, dt_target, C.byref(a), C.byref(p), C.byref(d), C.byref(n))
    return a.value, p.value, d.value, n.value


class OracleMesh:
    def __init__(self, path: str | os.PathLike, radius: float):
        st = C.c_int()
        h = lib().orc_mesh_load(os.fsencode(str(path)), radius, C.byref(st))
        if not h:
            raise RuntimeError(f"oracle could not load {path}: status {st.value}")
        self._h = C.c_void_p(h)
        n, e, v = C.c_int(), C.c_int(), C.c_int()
        lib().orc_mesh_sizes(self._h, C.byref(n), C.byref(e), C.byref(v))
        self.n_cells, self.n_edges, self.n_vertices = n.value, e.value, v.value

    def field(self, which: int) -> np.ndarray:
        out = np.zeros(self.n_cells if which in (3, 12, 13) else self.n_edges)
        lib().orc_mesh_get_field(self._h, which, _dp(out))
        return out

    def topology(self):
        E, N = self.n_edges, self.n_cells
        fn = np.zeros((E, 2), np.int32)
        faces = np.zeros((N, 6), np.int32)
        nfd = np.zeros((N, 6), np.int32)
        ifr = np.zeros((E, 10), np.int32)
        iw = np.zeros((E, 10))
        inn = np.zeros(E, np.int32)
        lib().orc_mesh_get_topology(self._h, _ip(fn), _ip(faces), _ip(nfd), _ip(ifr), _dp(iw), _ip(inn))
        return dict(face_nodes=fn, faces=faces, node_face_dir=nfd, interp_friends=ifr, interp_w=iw, interp_n=inn)

    def vertex_field(self, which: int) -> np.ndarray:
        """0 vertex area, 1-3 kite fractions R(v, j) of the vertex's nodes, 4 sin(lat)."""
        out = np.zeros(self.n_vertices)
        lib().orc_mesh_vertex_field(self._h, which, _dp(out))
        return out

    def vertex_topology(self):
        V, E = self.n_vertices, self.n_edges
        vn = np.zeros((V, 3), np.int32)
        vf = np.zeros((V, 3), np.int32)
        vd = np.zeros((V, 3), np.int32)
        fv = np.zeros((E, 2), np.int32)
        lib().orc_mesh_vertex_topology(self._h, _ip(vn), _ip(vf), _ip(vd), _ip(fv))
        return dict(vert_nodes=vn, vert_faces=vf, vert_face_dir=vd, face_verts=fv)

    def csr(self, op: int):
        """op 0 gradient (E x N), 1 divergence (N x E), 2 Coriolis with Omega = 1 (E x E)."""
        rows = self.n_edges if op != 1 else self.n_cells
        nnz = lib().orc_mesh_get_csr(self._h, op, None, None, None)
        rp = np.zeros(rows + 1, np.int32)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        lib().orc_mesh_get_csr(self._h, op, _ip(rp), _ip(col), _dp(val))
        return rp, col, val

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.orc_mesh_free(self._h)
            self._h = C.c_void_p()


class OracleSolver:
    """FP64 restatement of the reference step (see odis_oracle.c)."""

    def __init__(self, mesh: OracleMesh, *, radius, g, angvel, h, alpha, ecc=0.0, obliq=0.0, love_reduct=1.0,
                 dt, potential=ECC, init_load=0, sh_lmax=0, sh_factors=None, advection=0, friction=0,
                 semimajor_axis=1221.87e6, fourier_freq=1):
        self.mesh = mesh
        self.p = OrcParams(radius, g, angvel, h, alpha, ecc, obliq, love_reduct, dt, potential, init_load, advection,
                           friction, semimajor_axis, fourier_freq)
        self._s = C.c_void_p(lib().orc_solver_create(mesh._h, C.byref(self.p)))
        if sh_lmax:
            f = np.ascontiguousarray(sh_factors, np.float64)
            st = lib().orc_solver_set_loading(self._s, int(sh_lmax), _dp(f))
            if st != 0:
                raise RuntimeError(f"oracle SH setup failed: {st}")
        self._x = C.c_void_p(lib().orc_sim_create(self._s))
        self.E, self.N = mesh.n_edges, mesh.n_cells
        self.sh_lmax = int(sh_lmax)

    def updateMomentum(self, v, eta):
        out = np.zeros(self.E)
        lib().orc_update_momentum(self._s, _dp(out), _dp(np.ascontiguousarray(v, np.float64)),
                                  _dp(np.ascontiguousarray(eta, np.float64)))
        return out

    def updateEta(self, v):
        out = np.zeros(self.N)
        lib().orc_update_eta(self._s, _dp(out), _dp(np.ascontiguousarray(v, np.float64)))
        return out

    def forcing(self, type_, t, ecc=None, obl=None, out=None):
        """forcing(..., type, time, ecc, obl) (src/tidalPotentials.cpp:29-334); ecc/obl default to the
        solver's.  Types without a case leave `out` (zeros if not given) untouched."""
        out = np.zeros(self.N) if out is None else np.ascontiguousarray(out, np.float64)
        lib().orc_forcing(self._s, _dp(out), int(type_), float(t), float(self.p.ecc if ecc is None else ecc),
                          float(self.p.obliq if obl is None else obl))
        return out

    def integrateAB3scalar(self, s, ds_dt, it):
        lib().orc_ab3(self.p.dt, _dp(s), _dp(ds_dt), int(it), int(s.shape[0]), int(self.p.init_load))

    def interpolateVelocity(self, v):
        out = np.zeros((self.E, 2))
        lib().orc_interpolate_velocity(self.mesh._h, _dp(out), _dp(np.ascontiguousarray(v, np.float64)))
        return out

    def interpolateVelocityCart(self, v):
        out = np.zeros((self.N, 3))
        lib().orc_interpolate_cartesian(self.mesh._h, _dp(out), _dp(np.ascontiguousarray(v, np.float64)))
        return out

    def calculateMomentumAdvection(self, dvdt, v, h_total):
        """dvdt + PV flux - grad KE (src/momAdvection.cpp:11-267); returns (dvdt, ekin)."""
        out = np.array(dvdt, np.float64, copy=True)
        ekin = np.zeros(self.N)
        lib().orc_momentum_advection(self.mesh._h, self.p.angvel, _dp(out), _dp(np.ascontiguousarray(v, np.float64)),
                                     _dp(np.ascontiguousarray(h_total, np.float64)), _dp(ekin))
        return out, ekin

    def interpolateLSQFlux(self, v, h_total, eps=0.25):
        """Third-order thickness flux across the faces (src/interpolation.cpp:311-356)."""
        out = np.zeros(self.E)
        st = lib().orc_lsq_flux(self.mesh._h, eps, _dp(out), _dp(np.ascontiguousarray(v, np.float64)),
                                _dp(np.ascontiguousarray(h_total, np.float64)))
        if st != 0:
            raise RuntimeError(f"oracle LSQ operator failed: {st}")
        return out

    def updateEnergy(self, uv):
        e = np.zeros(self.E)
        avg = lib().orc_update_energy_fric(self.mesh._h, self.p.alpha, self.p.h, self.p.friction, _dp(e),
                                           _dp(np.ascontiguousarray(uv, np.float64)))
        return avg, e

    def sh_analysis(self, eta):
        """Least-squares SH coefficients c[(L+1)^2] of a node field (needs sh_lmax)."""
        K = (self.sh_lmax + 1) ** 2
        out = np.zeros(K)
        lib().orc_sh_analysis(self._s, _dp(np.ascontiguousarray(eta, np.float64)), _dp(out))
        return out

    def run(self, nsteps):
        out = np.zeros(nsteps)
        lib().orc_sim_run(self._x, int(nsteps), _dp(out))
        return out

    def get_state(self):
        it = C.c_int()
        v, eta = np.zeros(self.E), np.zeros(self.N)
        dv, de = np.zeros((self.E, 3)), np.zeros((self.N, 3))
        lib().orc_sim_get_state(self._x, C.byref(it), _dp(v), _dp(eta), _dp(dv), _dp(de))
        return it.value, v, eta, dv, de

    def set_state(self, it, v, eta, dvdt, detadt):
        a = [np.ascontiguousarray(x, np.float64) for x in (v, eta, dvdt, detadt)]
        lib().orc_sim_set_state(self._x, int(it), *[_dp(x) for x in a])

    def __del__(self):
        if _lib is None:
            return
        if getattr(self, "_x", None) and self._x.value:
            _lib.orc_sim_free(self._x)
            self._x = C.c_void_p()
        if getattr(self, "_s", None) and self._s.value:
            _lib.orc_solver_free(self._s)
            self._s = C.c_void_p()


def generate_grid_file(level: int, path: str | os.PathLike) -> None:
    """Icosahedral grid of 10*4^level+2 cells in the reference's grid-file format, generated by the oracle
    (its own numbering; the same mesh as the product's generator)."""
    st = lib().orc_generate_grid_file(int(level), os.fsencode(str(path)))
    if st != 0:
        raise RuntimeError(f"oracle grid generation failed: {st}")


def loading_factors(g: float, radius: float, lmax: int) -> np.ndarray:
    """FREE_LOADING gamma_l, l = 0..lmax (src/boundaryConditions.cpp:29-76)."""
    out = np.zeros(lmax + 1)
    lib().orc_loading_factors(float(g), float(radius), int(lmax), _dp(out))
    return out


def benchmark_sh_factors(g: float, radius: float, lmax: int, seed: int = 1) -> np.ndarray:
    """f_l * gamma_l with f_l ~ U[0.5, 1.5] (numpy default_rng(seed), degrees 2..lmax in order); entries 0, 1 zero."""
    f = np.zeros(lmax + 1)
    f[2:] = np.random.default_rng(seed).uniform(0.5, 1.5, lmax - 1)
    return f * np.where(np.arange(lmax + 1) >= 2, loading_factors(g, radius, lmax), 0.0)


def plmbar(L: int, z: float) -> np.ndarray:
    out = np.zeros((L + 1) * (L + 2) // 2)
    lib().orc_plmbar(int(L), float(z), _dp(out))
    return out
