"""GB300-native GeodesicODIS LTE timestep.

Python view of libodis_gpu.so (C ABI in include/odis_gpu.h).  The names
mirror the reference's free functions (updateMomentum, updateEta, forcing,
integrateAB3scalar, interpolateVelocity, updateEnergy) and its time loop
(ab3Explicit), with the same argument meaning; errors raise OdisError with
the library's status code instead of the reference's exit(0).

The CUDA library is required: importing works without a GPU (the mesh and
input.in code is host C++), but every call that computes on the device fails
loudly when no GPU or no built library is present.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

__all__ = [
    "OdisError", "lib", "Params", "Input", "Mesh", "Solver", "generate_grid_file", "derive_time",
    "read_input", "Batch", "BatchMember", "MLP", "POT_NONE", "POT_ECC", "POT_OBLIQ", "POT_OBLIQ_WEST", "POT_FULL",
    "POT_FULL2", "POT_PLANET", "POT_GENERAL", "FP64", "FP32", "DF64",
]

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libodis_gpu.so"

OK, ERR_ARG, ERR_CUDA, ERR_OOB, ERR_NONFINITE, ERR_TIMEOUT, ERR_IO, ERR_MESH, ERR_NOMEM = range(9)
_NAMES = {1: "ODIS_ERR_ARG", 2: "ODIS_ERR_CUDA", 3: "ODIS_ERR_OOB", 4: "ODIS_ERR_NONFINITE",
          5: "ODIS_ERR_TIMEOUT", 6: "ODIS_ERR_IO", 7: "ODIS_ERR_MESH", 8: "ODIS_ERR_NOMEM"}
# forcing types: the values of the reference's enum Potential (include/globals.h:60-76)
(POT_OBLIQ, POT_OBLIQ_WEST, POT_OBLIQ_EAST, POT_ECC_RAD, POT_ECC_LIB, POT_ECC, POT_ECC_WEST, POT_ECC_EAST, POT_FULL,
 POT_FULL2, POT_TOTAL, POT_ECC_W3, POT_OBLIQ_W3, POT_PLANET, POT_PLANET_OBL, POT_GENERAL, POT_NONE) = range(17)
FP64, FP32, DF64 = 0, 1, 2
MEM_HOST, MEM_DEVICE = 0, 1


class OdisError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where}: {_NAMES.get(code, code)}")
        self.code = code


FRIC_LINEAR, FRIC_QUADRATIC = 0, 1      # odis_params.friction (input.in "friction type")


class Params(C.Structure):
    _fields_ = [("radius", C.c_double), ("g", C.c_double), ("angvel", C.c_double), ("h", C.c_double),
                ("alpha", C.c_double), ("ecc", C.c_double), ("obliq", C.c_double), ("love_reduct", C.c_double),
                ("dt", C.c_double), ("potential", C.c_int), ("init_load", C.c_int), ("precision", C.c_int),
                ("sh_lmax", C.c_int), ("sh_factors", C.POINTER(C.c_double)), ("advection", C.c_int),
                ("friction", C.c_int), ("semimajor_axis", C.c_double), ("fourier_freq", C.c_int)]


class BatchMember(C.Structure):
    _fields_ = [("mesh", C.c_int), ("steps_per_orbit", C.c_int), ("h", C.c_double), ("alpha", C.c_double),
                ("ecc", C.c_double), ("obliq", C.c_double)]


class Input(C.Structure):
    _fields_ = [("params", Params), ("period", C.c_double), ("end_time", C.c_double),
                ("steps_per_orbit", C.c_int), ("grid_level", C.c_int), ("output_time", C.c_int),
                ("sh_degree", C.c_int), ("advection", C.c_int), ("fric_linear", C.c_int),
                ("surface_free", C.c_int), ("init_kind", C.c_int), ("out_flags", C.c_int),
                ("potential_name", C.c_char * 32), ("friction_name", C.c_char * 32),
                ("surface_name", C.c_char * 32), ("solver_name", C.c_char * 32), ("init_name", C.c_char * 32)]


_lib = None

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p

_SIGS = {
    "odis_grid_generate_file": ([C.c_int, C.c_char_p], C.c_int),
    "odis_mesh_from_file": ([C.c_char_p, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_generate": ([C.c_int, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_generate_device": ([C.c_int, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_from_file_device": ([C.c_char_p, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_from_arrays_device": ([C.c_int, _D, _I, _D, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_from_arrays": ([C.c_int, _D, _I, _D, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_grid_generate_arrays": ([C.c_int, C.c_int, _D, _I, _D], C.c_int),
    "odis_mesh_compare": ([_V, _V, _D, C.POINTER(C.c_longlong)], C.c_int),
    "odis_text_round16": ([_D, _D, C.c_longlong], C.c_int),
    "odis_mesh_from_arrays": ([C.c_int, _D, _I, _D, C.c_double, C.POINTER(_V)], C.c_int),
    "odis_mesh_sizes": ([_V, _I, _I, _I], C.c_int),
    "odis_mesh_field": ([_V, C.c_int, _D], C.c_int),
    "odis_mesh_topology": ([_V, _I, _I, _I, _I, _D, _I], C.c_int),
    "odis_mesh_vertex_field": ([_V, C.c_int, _D], C.c_int),
    "odis_mesh_vertex_topology": ([_V, _I, _I, _I, _I], C.c_int),
    "odis_mesh_destroy": ([_V], None),
    "odis_mesh_gravity_wave_omega": ([_V, C.c_double, C.c_double, C.c_int, _D], C.c_int),
    "odis_stable_steps_per_orbit": ([C.c_double, C.c_double, C.c_double, _I], C.c_int),
    "odis_loading_factors": ([C.c_double, C.c_double, C.c_int, _D], C.c_int),
    "odis_derive_time": ([C.c_double, C.c_double, _D, _D, _D, _I], C.c_int),
    "odis_params_from_input": ([C.c_char_p, C.POINTER(Input)], C.c_int),
    "odis_create": ([C.POINTER(Params), _V, C.POINTER(_V)], C.c_int),
    "odis_destroy": ([_V], None),
    "odis_set_stream": ([_V, _V], C.c_int),
    "odis_synchronize": ([_V], C.c_int),
    "odis_device_status": ([_V], C.c_int),
    "odis_update_momentum": ([_V, _V, _V, _V, C.c_int], C.c_int),
    "odis_update_eta": ([_V, _V, _V, C.c_int], C.c_int),
    "odis_forcing": ([_V, _V, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int], C.c_int),
    "odis_ab3": ([_V, _V, _V, C.c_int, C.c_int, C.c_int], C.c_int),
    "odis_interpolate_velocity": ([_V, _V, _V, C.c_int], C.c_int),
    "odis_interpolate_cartesian": ([_V, _V, _V, C.c_int], C.c_int),
    "odis_momentum_advection": ([_V, _V, _V, _V, _V, _V, C.c_int], C.c_int),
    "odis_lsq_flux": ([_V, _V, _V, _V, _V, C.c_int], C.c_int),
    "odis_update_energy": ([_V, _V, _V, _V, C.c_int], C.c_int),
    "odis_run_steps": ([_V, C.c_int, _V, C.c_int], C.c_int),
    "odis_get_state": ([_V, _I, _D, _D, _D, _D], C.c_int),
    "odis_set_state": ([_V, C.c_int, _D, _D, _D, _D], C.c_int),
    "odis_launch_count": ([_V, C.POINTER(C.c_longlong)], C.c_int),
    "odis_set_wait_limit": ([_V, C.c_uint, C.c_int], C.c_int),
    "odis_measure_fp64_rate": ([_D], C.c_int),
    "odis_batch_set_wait_limit": ([_V, C.c_uint, C.c_int], C.c_int),
    "odis_batch_graph_runs": ([_V, C.POINTER(C.c_longlong)], C.c_int),
    "odis_profile_kernels": ([_V, C.c_int, _D], C.c_int),
    "odis_set_persistent": ([_V, C.c_int, _I], C.c_int),
    "odis_sh_tiles": ([_V, _I, _I, _I, _I, _I], C.c_int),
    "odis_sh_layout": ([_V, _I, _I, C.POINTER(C.c_longlong)], C.c_int),
    "odis_batch_create": ([C.POINTER(Params), C.POINTER(_V), C.c_int, _V, C.c_int, C.POINTER(_V)], C.c_int),
    "odis_batch_destroy": ([_V], None),
    "odis_batch_run": ([_V, C.c_double, C.c_int, _D, C.c_int, _D, C.c_int, C.c_int], C.c_int),
    "odis_batch_get_member": ([_V, C.c_int, _I, _D, _D], C.c_int),
    "odis_batch_set_member": ([_V, C.c_int, _D, _D], C.c_int),
    "odis_batch_info": ([_V, _I, _I, _I, C.POINTER(C.c_longlong), _I], C.c_int),
    "odis_batch_get_mesh_members": ([_V, C.c_int, _D, _D], C.c_int),
    "odis_batch_set_mesh_members": ([_V, C.c_int, _D, _D], C.c_int),
    "odis_batch_project": ([_V, C.c_int, _V, C.c_int, _V, C.c_int, _D, C.c_int], C.c_int),
    "odis_analytical_state": ([C.POINTER(Params), _V, C.c_double, _D, _D, _D, _D], C.c_int),
    "odis_h5_create": ([C.c_char_p, C.c_int, C.POINTER(C.c_char_p), _I, C.POINTER(C.c_longlong), C.POINTER(_V)], C.c_int),
    "odis_h5_write_rows": ([_V, C.c_int, C.c_longlong, C.c_longlong, _V], C.c_int),
    "odis_h5_close": ([_V], C.c_int),
    "odis_mlp_create": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(_V)], C.c_int),
    "odis_mlp_destroy": ([_V], None),
    "odis_mlp_num_params": ([_V, C.POINTER(C.c_longlong)], C.c_int),
    "odis_mlp_get_params": ([_V, _V], C.c_int),
    "odis_mlp_set_params": ([_V, _V], C.c_int),
    "odis_mlp_predict": ([_V, _V, _V, C.c_int, _V], C.c_int),
    "odis_mlp_gradient": ([_V, _V, _V, _V, _V, C.c_int, _D, _V], C.c_int),
    "odis_mlp_train": ([_V, _V, _V, _V, _V, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong, _D], C.c_int),
}


def lib() -> C.CDLL:
    """Load libodis_gpu.so (built in-tree by build_ext.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise OdisError(ERR_CUDA, f"{LIB_PATH} is missing; build it with geodesicodis_gb300.build_ext.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _ck(code: int, where: str) -> None:
    if code != OK:
        raise OdisError(code, where)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _vp(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def generate_grid_file(level: int, path: str | os.PathLike) -> None:
    """Icosahedral grid at `level` (10*4^level+2 cells) in the reference grid-file format."""
    _ck(lib().odis_grid_generate_file(int(level), os.fsencode(str(path))), "odis_grid_generate_file")


def generate_grid(level: int, device: bool = False):
    """The level-n icosahedral grid as arrays (node_deg [N,2], friends [N,6], cent_deg [N,6,2], degrees), the
    contents of generate_grid_file; device=True generates it with kernels on the current GPU."""
    n = 10 * 4 ** int(level) + 2
    nd, fr, cd = np.zeros((n, 2)), np.zeros((n, 6), np.int32), np.zeros((n, 6, 2))
    _ck(lib().odis_grid_generate_arrays(int(level), int(bool(device)), _dp(nd), fr.ctypes.data_as(_I), _dp(cd)),
        "odis_grid_generate_arrays")
    return nd, fr, cd


def text_round16(values) -> np.ndarray:
    """Each value through the grid file's text form: float("%.16f" % v), as the generators store coordinates."""
    x = np.ascontiguousarray(values, np.float64).ravel().copy()
    _ck(lib().odis_text_round16(_dp(x), _dp(x), x.size), "odis_text_round16")
    return x.reshape(np.shape(values))


def analytical_state(params: Params, mesh: "Mesh", t: float = 0.0):
    """(v[E], eta[N], dvdt[E,3], detadt[N,3]) of "initial conditions ANALYTICAL": the reference's
    closed-form westward obliquity-tide solution at time t (potential POT_OBLIQ_WEST)."""
    E, N = mesh.n_edges, mesh.n_cells
    v, eta, dv, de = np.zeros(E), np.zeros(N), np.zeros((E, 3)), np.zeros((N, 3))
    _ck(lib().odis_analytical_state(C.byref(params), mesh._h, float(t), _dp(v), _dp(eta), _dp(dv), _dp(de)),
        "odis_analytical_state")
    return v, eta, dv, de


class H5Writer:
    """DATA/data.h5-style output (src/outFiles.cpp:138-823): float32 datasets of
    rank 1 or 2 in the root group of an HDF5 file, written by the library's own
    writer (odis_h5_*).  `datasets` is a list of (name, shape); storage is
    zero-filled at creation and rows are written in place."""

    def __init__(self, path: str | os.PathLike, datasets):
        names = [str(n).encode() for n, _ in datasets]
        shapes = [tuple(int(x) for x in sh) for _, sh in datasets]
        arr = (C.c_char_p * len(names))(*names)
        ranks = np.array([len(sh) for sh in shapes], np.int32)
        dims = np.array([[sh[0], sh[1] if len(sh) > 1 else 0] for sh in shapes], np.int64).ravel()
        self.shapes = shapes
        self.index = {n: k for k, (n, _) in enumerate(datasets)}
        h = _V()
        _ck(lib().odis_h5_create(os.fsencode(str(path)), len(names), arr, ranks.ctypes.data_as(_I),
                                 dims.ctypes.data_as(C.POINTER(C.c_longlong)), C.byref(h)), "odis_h5_create")
        self._h = h

    def write_rows(self, name: str, row0: int, rows) -> None:
        k = self.index[name]
        a = np.ascontiguousarray(rows, dtype=np.float32)
        per_row = self.shapes[k][1] if len(self.shapes[k]) == 2 else 1
        n = a.size // per_row
        if a.size != n * per_row:
            raise OdisError(ERR_ARG, f"{name}: {a.size} values are not whole rows of {per_row}")
        _ck(lib().odis_h5_write_rows(self._h, k, int(row0), int(n), _vp(a)), "odis_h5_write_rows")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            h, self._h = self._h, None
            _ck(lib().odis_h5_close(h), "odis_h5_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.odis_h5_close(self._h)


def derive_time(angvel_in: float, dt_target: float):
    """(angvel, period, dt, steps_per_orbit) after period rounding and dt snapping."""
    a, p, d, n = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    _ck(lib().odis_derive_time(angvel_in, dt_target, C.byref(a), C.byref(p), C.byref(d), C.byref(n)),
        "odis_derive_time")
    return a.value, p.value, d.value, n.value


STABILITY_LIMIT = 6.0 / 11.0   # omega_max * dt bound of the reference's forward-backward AB3 loop


def stable_steps_per_orbit(period: float, omega_max: float, margin: float = 0.95) -> int:
    """Smallest multiple of 100 steps per orbit with omega_max * dt <= margin * 6/11."""
    n = C.c_int()
    _ck(lib().odis_stable_steps_per_orbit(period, omega_max, margin, C.byref(n)), "odis_stable_steps_per_orbit")
    return n.value


def loading_factors(g: float, radius: float, lmax: int) -> np.ndarray:
    """gamma_l of the reference's FREE_LOADING surface, l = 0..lmax."""
    out = np.zeros(lmax + 1)
    _ck(lib().odis_loading_factors(g, radius, int(lmax), _dp(out)), "odis_loading_factors")
    return out


def benchmark_sh_factors(g: float, radius: float, lmax: int, seed: int = 1) -> np.ndarray:
    """Per-degree self-gravity factors of the level-6 benchmark: f_l * gamma_l with
    f_l ~ U[0.5, 1.5] (numpy default_rng(seed), degrees 2..lmax in order)."""
    f = np.zeros(lmax + 1)
    f[2:] = np.random.default_rng(seed).uniform(0.5, 1.5, lmax - 1)
    return f * loading_factors(g, radius, lmax)


def measure_fp64_rate() -> float:
    """FP64 FMA rate of this GPU in TFLOP/s (odis_measure_fp64_rate)."""
    t = C.c_double()
    _ck(lib().odis_measure_fp64_rate(C.byref(t)), "odis_measure_fp64_rate")
    return t.value


def read_input(path: str | os.PathLike) -> Input:
    inp = Input()
    _ck(lib().odis_params_from_input(os.fsencode(str(path)), C.byref(inp)), "odis_params_from_input")
    return inp


class Mesh:
    """Geometry and operators of an icosahedral-geodesic mesh (the reference's Mesh)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        n, e, v = C.c_int(), C.c_int(), C.c_int()
        _ck(lib().odis_mesh_sizes(self._h, C.byref(n), C.byref(e), C.byref(v)), "odis_mesh_sizes")
        self.n_cells, self.n_edges, self.n_vertices = n.value, e.value, v.value

    # device=True: geometry and TRiSK weights built by kernels on the current GPU (and the grid generated
    # there); integer arrays identical to the host build, geometry to the device's transcendental rounding

    @classmethod
    def from_file(cls, path: str | os.PathLike, radius: float, device: bool = False) -> "Mesh":
        h = C.c_void_p()
        fn = "odis_mesh_from_file_device" if device else "odis_mesh_from_file"
        _ck(getattr(lib(), fn)(os.fsencode(str(path)), radius, C.byref(h)), fn)
        return cls(h.value)

    @classmethod
    def generate(cls, level: int, radius: float, device: bool = False) -> "Mesh":
        h = C.c_void_p()
        fn = "odis_mesh_generate_device" if device else "odis_mesh_generate"
        _ck(getattr(lib(), fn)(int(level), radius, C.byref(h)), fn)
        return cls(h.value)

    @classmethod
    def from_arrays(cls, node_sph: np.ndarray, friends: np.ndarray, cent_sph: np.ndarray, radius: float,
                    device: bool = False) -> "Mesh":
        """node_sph [N,2] and cent_sph [N,6,2] in radians, friends [N,6] (-1 in slot 5 for pentagons)."""
        ns = np.ascontiguousarray(node_sph, np.float64)
        fr = np.ascontiguousarray(friends, np.int32)
        cs = np.ascontiguousarray(cent_sph, np.float64)
        h = C.c_void_p()
        fn = "odis_mesh_from_arrays_device" if device else "odis_mesh_from_arrays"
        _ck(getattr(lib(), fn)(len(ns), _dp(ns), fr.ctypes.data_as(_I), _dp(cs), radius, C.byref(h)), fn)
        return cls(h.value)

    def compare(self, other: "Mesh"):
        """(largest max|a-b|/max|b| over the floating-point arrays, differing integer entries) against other."""
        rel, bad = C.c_double(), C.c_longlong()
        _ck(lib().odis_mesh_compare(self._h, other._h, C.byref(rel), C.byref(bad)), "odis_mesh_compare")
        return rel.value, bad.value

    def field(self, which: int) -> np.ndarray:
        n = self.n_cells if which in (3, 12, 13) else self.n_edges
        out = np.zeros(n)
        _ck(lib().odis_mesh_field(self._h, which, _dp(out)), "odis_mesh_field")
        return out

    def gravity_wave_omega(self, g: float, h: float, iters: int = 300) -> float:
        """sqrt of the largest eigenvalue of -g h D G (rad/s)."""
        w = C.c_double()
        _ck(lib().odis_mesh_gravity_wave_omega(self._h, g, h, int(iters), C.byref(w)), "odis_mesh_gravity_wave_omega")
        return w.value

    def topology(self):
        E, N = self.n_edges, self.n_cells
        fn = np.zeros((E, 2), np.int32)
        faces = np.zeros((N, 6), np.int32)
        nfd = np.zeros((N, 6), np.int32)
        ifr = np.zeros((E, 10), np.int32)
        iw = np.zeros((E, 10))
        inn = np.zeros(E, np.int32)
        ip = lambda a: a.ctypes.data_as(_I)  # noqa: E731
        _ck(lib().odis_mesh_topology(self._h, ip(fn), ip(faces), ip(nfd), ip(ifr), _dp(iw), ip(inn)),
            "odis_mesh_topology")
        return dict(face_nodes=fn, faces=faces, node_face_dir=nfd, interp_friends=ifr, interp_w=iw, interp_n=inn)

    def vertex_field(self, which: int) -> np.ndarray:
        """0 area of the vertex's node triangle, 1-3 kite fractions R(v, j), 4 sin(lat)."""
        out = np.zeros(self.n_vertices)
        _ck(lib().odis_mesh_vertex_field(self._h, which, _dp(out)), "odis_mesh_vertex_field")
        return out

    def vertex_topology(self):
        V, E = self.n_vertices, self.n_edges
        vn = np.zeros((V, 3), np.int32)
        vf = np.zeros((V, 3), np.int32)
        vd = np.zeros((V, 3), np.int32)
        fv = np.zeros((E, 2), np.int32)
        ip = lambda a: a.ctypes.data_as(_I)  # noqa: E731
        _ck(lib().odis_mesh_vertex_topology(self._h, ip(vn), ip(vf), ip(vd), ip(fv)), "odis_mesh_vertex_topology")
        return dict(vert_nodes=vn, vert_faces=vf, vert_face_dir=vd, face_verts=fv)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.odis_mesh_destroy(h)
            self._h = C.c_void_p()


def make_params(*, radius, g, angvel, h, alpha, ecc=0.0, obliq=0.0, love_reduct=1.0, dt, potential=POT_ECC,
                init_load=0, precision=FP64, sh_lmax=0, sh_factors=None, advection=0, friction=FRIC_LINEAR,
                semimajor_axis=1221.87e6, fourier_freq=1) -> Params:
    p = Params(radius, g, angvel, h, alpha, ecc, obliq, love_reduct, dt, potential, init_load, precision, sh_lmax, None,
               advection, friction, semimajor_axis, fourier_freq)
    if sh_lmax:
        arr = np.ascontiguousarray(sh_factors, dtype=np.float64)
        p._factors = arr  # keep alive
        p.sh_factors = arr.ctypes.data_as(_D)
    return p


class Solver:
    """One ocean instance on the GPU: the reference's per-operator functions and its AB3 time loop."""

    def __init__(self, params: Params, mesh: Mesh):
        self.params = params
        self.mesh = mesh
        h = C.c_void_p()
        _ck(lib().odis_create(C.byref(params), mesh._h, C.byref(h)), "odis_create")
        self._h = h
        self.E, self.N = mesh.n_edges, mesh.n_cells

    # -- the reference's free functions (host arrays) --------------------------------
    def updateMomentum(self, v: np.ndarray, eta: np.ndarray) -> np.ndarray:
        out = np.zeros(self.E)
        v, eta = np.ascontiguousarray(v, np.float64), np.ascontiguousarray(eta, np.float64)
        _ck(lib().odis_update_momentum(self._h, _vp(out), _vp(v), _vp(eta), MEM_HOST), "odis_update_momentum")
        return out

    def updateEta(self, v: np.ndarray) -> np.ndarray:
        out = np.zeros(self.N)
        v = np.ascontiguousarray(v, np.float64)
        _ck(lib().odis_update_eta(self._h, _vp(out), _vp(v), MEM_HOST), "odis_update_eta")
        return out

    def forcing(self, type_: int, t: float, ecc: float | None = None, obl: float | None = None,
                out: np.ndarray | None = None) -> np.ndarray:
        """forcing(..., type, time, ecc, obl): ecc/obl default to the context's; types without a case in
        the reference's switch leave `out` (zeros if not given) untouched."""
        out = np.zeros(self.N) if out is None else np.ascontiguousarray(out, np.float64)
        _ck(lib().odis_forcing(self._h, _vp(out), int(type_), float(t),
                               float(self.params.ecc if ecc is None else ecc),
                               float(self.params.obliq if obl is None else obl), MEM_HOST), "odis_forcing")
        return out

    def integrateAB3scalar(self, s: np.ndarray, ds_dt: np.ndarray, it: int) -> None:
        """In place on s[num] and ds_dt[num][3], as the reference."""
        assert s.dtype == np.float64 and ds_dt.dtype == np.float64 and s.flags.c_contiguous and ds_dt.flags.c_contiguous
        _ck(lib().odis_ab3(self._h, _vp(s), _vp(ds_dt), int(it), int(s.shape[0]), MEM_HOST), "odis_ab3")

    def interpolateVelocity(self, v: np.ndarray) -> np.ndarray:
        out = np.zeros((self.E, 2))
        v = np.ascontiguousarray(v, np.float64)
        _ck(lib().odis_interpolate_velocity(self._h, _vp(out), _vp(v), MEM_HOST), "odis_interpolate_velocity")
        return out

    def interpolateVelocityCart(self, v: np.ndarray) -> np.ndarray:
        """Cartesian velocity [N, 3] at the nodes (the reference's RBF reconstruction)."""
        out = np.zeros((self.N, 3))
        v = np.ascontiguousarray(v, np.float64)
        _ck(lib().odis_interpolate_cartesian(self._h, _vp(out), _vp(v), MEM_HOST), "odis_interpolate_cartesian")
        return out

    def calculateMomentumAdvection(self, dvdt: np.ndarray, v: np.ndarray, h_total: np.ndarray):
        """(dvdt + PV flux - grad KE, KE at the nodes): the reference's calculateMomentumAdvection."""
        out = np.array(dvdt, np.float64, copy=True)
        ekin = np.zeros(self.N)
        v = np.ascontiguousarray(v, np.float64)
        h = np.ascontiguousarray(h_total, np.float64)
        _ck(lib().odis_momentum_advection(self._h, self.mesh._h, _vp(out), _vp(v), _vp(h), _vp(ekin), MEM_HOST),
            "odis_momentum_advection")
        return out, ekin

    def interpolateLSQFlux(self, v: np.ndarray, h_total: np.ndarray) -> np.ndarray:
        """Third-order thickness flux across the faces: the reference's interpolateLSQFlux."""
        out = np.zeros(self.E)
        v = np.ascontiguousarray(v, np.float64)
        h = np.ascontiguousarray(h_total, np.float64)
        _ck(lib().odis_lsq_flux(self._h, self.mesh._h, _vp(out), _vp(v), _vp(h), MEM_HOST), "odis_lsq_flux")
        return out

    def updateEnergy(self, uv: np.ndarray):
        """(area-mean dissipation W/m^2, per-face dissipation)."""
        e = np.zeros(self.E)
        avg = np.zeros(1)
        uv = np.ascontiguousarray(uv, np.float64)
        _ck(lib().odis_update_energy(self._h, _vp(avg), _vp(e), _vp(uv), MEM_HOST), "odis_update_energy")
        return float(avg[0]), e

    # -- the time loop -------------------------------------------------------------
    def run(self, nsteps: int, power: bool = True) -> np.ndarray | None:
        out = np.zeros(nsteps) if power else None
        ptr = _vp(out) if power else None
        _ck(lib().odis_run_steps(self._h, int(nsteps), ptr, MEM_HOST), "odis_run_steps")
        return out

    def run_device(self, nsteps: int, power_dev_ptr: int | None) -> None:
        _ck(lib().odis_run_steps(self._h, int(nsteps), C.c_void_p(power_dev_ptr) if power_dev_ptr else None,
                                 MEM_DEVICE), "odis_run_steps")

    def get_state(self):
        it = C.c_int()
        v, eta = np.zeros(self.E), np.zeros(self.N)
        dv, de = np.zeros((self.E, 3)), np.zeros((self.N, 3))
        _ck(lib().odis_get_state(self._h, C.byref(it), _dp(v), _dp(eta), _dp(dv), _dp(de)), "odis_get_state")
        return it.value, v, eta, dv, de

    def set_state(self, it: int, v, eta, dvdt, detadt) -> None:
        a = [np.ascontiguousarray(x, np.float64) for x in (v, eta, dvdt, detadt)]
        _ck(lib().odis_set_state(self._h, int(it), *[_dp(x) for x in a]), "odis_set_state")

    def set_stream(self, stream_ptr: int) -> None:
        _ck(lib().odis_set_stream(self._h, C.c_void_p(stream_ptr)), "odis_set_stream")

    def set_persistent(self, enable) -> bool:
        """Use (True) or forbid (False) the persistent single-launch loop, or None for
        the faster of the two paths as timed at creation; returns whether runs will use it."""
        a = C.c_int()
        flag = -1 if enable is None else int(bool(enable))
        _ck(lib().odis_set_persistent(self._h, flag, C.byref(a)), "odis_set_persistent")
        return bool(a.value)

    def sh_tiles(self) -> tuple:
        """(tile_l, chunks, lanes) of the self-gravity transforms chosen at creation."""
        return self.sh_tuning()[:3]

    def sh_tuning(self) -> tuple:
        """(tile_l, chunks, lanes, cells, pre) of the self-gravity transforms chosen at creation."""
        a, b, c, d, e = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _ck(lib().odis_sh_tiles(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(e)), "odis_sh_tiles")
        return a.value, b.value, c.value, d.value, e.value

    def sh_layout(self) -> dict:
        """Self-gravity basis storage: antipodal half basis or full, cells covered, bytes per transform."""
        a, b, c = C.c_int(), C.c_int(), C.c_longlong()
        _ck(lib().odis_sh_layout(self._h, C.byref(a), C.byref(b), C.byref(c)), "odis_sh_layout")
        return {"half": bool(a.value), "cells": b.value, "basis_bytes": c.value}

    def launch_count(self) -> int:
        n = C.c_longlong()
        _ck(lib().odis_launch_count(self._h, C.byref(n)), "odis_launch_count")
        return n.value

    def set_wait_limit(self, polls: int = 0, withhold: int = -1) -> None:
        """Bound the persistent loop's neighbour waits to `polls` polls (0: default); withhold >= 0 makes that
        CTA publish no step flags (failure-detection test hook)."""
        _ck(lib().odis_set_wait_limit(self._h, int(polls), int(withhold)), "odis_set_wait_limit")

    def profile_kernels(self, reps: int = 200):
        ms = np.zeros(3)
        _ck(lib().odis_profile_kernels(self._h, int(reps), _dp(ms)), "odis_profile_kernels")
        return ms

    def set_state_ptrs(self, it: int, v: int, eta: int, dvdt: int, detadt: int) -> None:
        """set_state from raw host addresses (e.g. pinned buffers)."""
        _ck(lib().odis_set_state(self._h, int(it), C.cast(v, _D), C.cast(eta, _D), C.cast(dvdt, _D),
                                 C.cast(detadt, _D)), "odis_set_state")

    def get_state_ptrs(self, v: int, eta: int, dvdt: int, detadt: int) -> int:
        it = C.c_int()
        _ck(lib().odis_get_state(self._h, C.byref(it), C.cast(v, _D), C.cast(eta, _D), C.cast(dvdt, _D),
                                 C.cast(detadt, _D)), "odis_get_state")
        return it.value

    def run_host_ptr(self, nsteps: int, power_ptr: int) -> None:
        _ck(lib().odis_run_steps(self._h, int(nsteps), C.c_void_p(power_ptr), MEM_HOST), "odis_run_steps")

    def synchronize(self) -> None:
        _ck(lib().odis_synchronize(self._h), "odis_synchronize")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().odis_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many configurations of the time loop advanced by one persistent launch per chunk of steps.

    `meshes` is a list of Mesh; `members` a list of dicts (or BatchMember) with keys
    mesh (index into `meshes`), steps_per_orbit (even), h, alpha, ecc, obliq.  The
    common parameters (radius, g, angvel, potential, love_reduct, init_load) come
    from `params`.
    """

    def __init__(self, params: Params, meshes, members):
        self.params = params
        self.meshes = list(meshes)
        arr = (BatchMember * len(members))()
        for i, m in enumerate(members):
            if isinstance(m, BatchMember):
                arr[i] = m
            else:
                arr[i] = BatchMember(int(m["mesh"]), int(m["steps_per_orbit"]), float(m["h"]), float(m["alpha"]),
                                     float(m.get("ecc", 0.0)), float(m.get("obliq", 0.0)))
        self.members = arr
        self.count = len(members)
        handles = (C.c_void_p * len(self.meshes))(*[mm._h.value for mm in self.meshes])
        h = C.c_void_p()
        _ck(lib().odis_batch_create(C.byref(params), handles, len(self.meshes), C.cast(arr, C.c_void_p), self.count,
                                    C.byref(h)), "odis_batch_create")
        self._h = h

    def run(self, orbits: float = 0, steps: int = 0, step_power: bool = False, chunk: int = 0):
        """Advance every member; returns (orbit_power [count, n_orbits], step_power [count, n_steps] or None)."""
        spo = np.array([m.steps_per_orbit for m in self.members])
        runs = np.rint(orbits * spo).astype(np.int64) if orbits > 0 else np.full(self.count, steps)
        n_orb = int(np.max((runs + spo - 1) // spo))
        op = np.zeros((self.count, n_orb))
        sp = np.zeros((self.count, int(np.max(runs)))) if step_power else None
        _ck(lib().odis_batch_run(self._h, float(orbits), int(steps), _dp(op), n_orb,
                                 _dp(sp) if sp is not None else None, sp.shape[1] if sp is not None else 0, int(chunk)),
            "odis_batch_run")
        return op, sp

    def get_member(self, i: int):
        m = self.members[i]
        mesh = self.meshes[m.mesh]
        v, eta, it = np.zeros(mesh.n_edges), np.zeros(mesh.n_cells), C.c_int()
        _ck(lib().odis_batch_get_member(self._h, int(i), C.byref(it), _dp(v), _dp(eta)), "odis_batch_get_member")
        return it.value, v, eta

    def set_member(self, i: int, v=None, eta=None) -> None:
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        ee = None if eta is None else np.ascontiguousarray(eta, dtype=np.float64)
        _ck(lib().odis_batch_set_member(self._h, int(i), _dp(vv) if vv is not None else None,
                                        _dp(ee) if ee is not None else None), "odis_batch_set_member")

    def mesh_members(self, mesh: int) -> np.ndarray:
        return np.array([i for i in range(self.count) if self.members[i].mesh == mesh], dtype=np.int64)

    def get_mesh_members(self, mesh: int):
        """(v [m, E], eta [m, N]) of the members on `mesh`, in member order."""
        m = len(self.mesh_members(mesh))
        ms = self.meshes[mesh]
        v, eta = np.zeros((m, ms.n_edges)), np.zeros((m, ms.n_cells))
        _ck(lib().odis_batch_get_mesh_members(self._h, int(mesh), _dp(v), _dp(eta)), "odis_batch_get_mesh_members")
        return v, eta

    def set_mesh_members(self, mesh: int, v=None, eta=None) -> None:
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        ee = None if eta is None else np.ascontiguousarray(eta, dtype=np.float64)
        _ck(lib().odis_batch_set_mesh_members(self._h, int(mesh), _dp(vv) if vv is not None else None,
                                              _dp(ee) if ee is not None else None), "odis_batch_set_mesh_members")

    def project(self, mesh: int, basis_v: np.ndarray, basis_eta: np.ndarray) -> np.ndarray:
        """[m, kv + ke] projections of the members on `mesh` (member order) onto the row bases."""
        bv = np.ascontiguousarray(basis_v, dtype=np.float32)
        be = np.ascontiguousarray(basis_eta, dtype=np.float32)
        kv, ke = bv.shape[0], be.shape[0]
        out = np.zeros((self.count, kv + ke))
        _ck(lib().odis_batch_project(self._h, int(mesh), C.c_void_p(bv.ctypes.data), kv, C.c_void_p(be.ctypes.data), ke,
                                     _dp(out), kv + ke), "odis_batch_project")
        return out[self.mesh_members(mesh)]

    def set_wait_limit(self, polls: int = 0, withhold: int = -1) -> None:
        """Bound each grid-barrier wait to `polls` polls (0: default); withhold >= 0 makes that CTA never
        arrive (failure-detection test hook)."""
        _ck(lib().odis_batch_set_wait_limit(self._h, int(polls), int(withhold)), "odis_batch_set_wait_limit")

    def info(self) -> dict:
        g, p, gr, n, r = C.c_int(), C.c_int(), C.c_int(), C.c_longlong(), C.c_int()
        _ck(lib().odis_batch_info(self._h, C.byref(g), C.byref(p), C.byref(gr), C.byref(n), C.byref(r)),
            "odis_batch_info")
        gr_runs = C.c_longlong()
        _ck(lib().odis_batch_graph_runs(self._h, C.byref(gr_runs)), "odis_batch_graph_runs")
        return {"groups": g.value, "padded_members": p.value, "grid": gr.value, "launches": n.value,
                "rows_per_thread": r.value, "graph_runs": gr_runs.value}

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.odis_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()


def _fp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class MLP:
    """The warm-start network (odis_mlp_*): n_in -> width x depth (GELU) -> n_mix * n_out, mixed per sample."""

    def __init__(self, n_in: int, width: int, depth: int, n_out: int, n_mix: int = 0, seed: int = 0):
        self.n_in, self.width, self.depth, self.n_out, self.n_mix = n_in, width, depth, n_out, n_mix
        h = C.c_void_p()
        _ck(lib().odis_mlp_create(n_in, width, depth, n_out, n_mix, seed, C.byref(h)), "odis_mlp_create")
        self._h = h
        n = C.c_longlong()
        _ck(lib().odis_mlp_num_params(self._h, C.byref(n)), "odis_mlp_num_params")
        self.n_params = n.value

    def _rows(self, x, mix, t=None, w=None):
        x = np.ascontiguousarray(x, np.float32)
        mix = None if mix is None else np.ascontiguousarray(mix, np.float32)
        t = None if t is None else np.ascontiguousarray(t, np.float32)
        w = None if w is None else np.ascontiguousarray(w, np.float32)
        return x, mix, t, w

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        _ck(lib().odis_mlp_get_params(self._h, _fp(p)), "odis_mlp_get_params")
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        _ck(lib().odis_mlp_set_params(self._h, _fp(p)), "odis_mlp_set_params")

    def predict(self, x, mix=None) -> np.ndarray:
        x, mix, _, _ = self._rows(x, mix)
        y = np.zeros((x.shape[0], self.n_out), np.float32)
        _ck(lib().odis_mlp_predict(self._h, _fp(x), _fp(mix), x.shape[0], _fp(y)), "odis_mlp_predict")
        return y

    def gradient(self, x, t, mix=None, w=None):
        x, mix, t, w = self._rows(x, mix, t, w)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        _ck(lib().odis_mlp_gradient(self._h, _fp(x), _fp(mix), _fp(t), _fp(w), x.shape[0], C.byref(loss), _fp(g)),
            "odis_mlp_gradient")
        return loss.value, g

    def train(self, x, t, mix=None, w=None, epochs=100, batch=256, lr=1e-3, seed=0) -> np.ndarray:
        x, mix, t, w = self._rows(x, mix, t, w)
        losses = np.zeros(epochs)
        _ck(lib().odis_mlp_train(self._h, _fp(x), _fp(mix), _fp(t), _fp(w), x.shape[0], int(epochs), int(batch),
                                 float(lr), int(seed), _dp(losses)), "odis_mlp_train")
        return losses

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.odis_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()
