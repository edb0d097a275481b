"""odis_update_energy_noalloc: the area-mean dissipation for callers that cannot allocate.

Such callers (host callbacks, graph host nodes, fixed-budget real-time loops,
plugins handed only device buffers) cannot create an odis_ctx, because that
allocates.  The entry point takes device buffers only and keeps its reduction
scratch in a fixed __device__ array; here it is called twice in a row through
the C ABI and must give what the context path (odis_update_energy) gives.
Collected last so that a failure here never hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import RADIUS, ecc_case_params

pytestmark = pytest.mark.gpu


def _entry():
    import geodesicodis_gb300 as g
    f = g.lib().odis_update_energy_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_energy_matches_context_path(grid_dir):
    import torch
    import geodesicodis_gb300 as g
    f = _entry()
    dev = torch.device("cuda:0")
    mesh = g.Mesh.from_file(grid_dir / "grid_4.txt", RADIUS)
    p = ecc_case_params()
    sol = g.Solver(g.make_params(**p), mesh)
    E = mesh.n_edges
    area = torch.tensor(mesh.field(2), dtype=torch.float64, device=dev)
    rng = np.random.default_rng(7)
    for call in range(2):                       # two calls in a row share the scratch array
        uv_h = rng.standard_normal((E, 2)) * 0.01 * (call + 1)
        uv = torch.tensor(uv_h, dtype=torch.float64, device=dev)
        e_out = torch.full((E,), float("nan"), dtype=torch.float64, device=dev)
        avg = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = f(uv.data_ptr(), area.data_ptr(), E, p["alpha"], p["h"], RADIUS, e_out.data_ptr(), avg.data_ptr(), None)
        torch.cuda.synchronize()
        assert st == 0
        avg_ref, e_ref = sol.updateEnergy(uv_h)
        assert abs(avg.item() - avg_ref) <= 1e-12 * abs(avg_ref)
        np.testing.assert_allclose(e_out.cpu().numpy(), e_ref, rtol=1e-12, atol=0)


def test_noalloc_energy_rejects_oversize(grid_dir):
    import torch
    f = _entry()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    st = f(buf.data_ptr(), buf.data_ptr(), 8192 * 256 + 1, 1e-5, 1e4, RADIUS, None, buf.data_ptr(), None)
    assert st == 1                              # ODIS_ERR_ARG, nothing launched
