"""Time-step stability of the reference's time loop.

The loop advances v with AB3 using the old eta and then eta with AB3 using the
new v (src/timeIntegrator.cpp:213-253): a forward-backward AB3 whose
stability limit for a gravity-wave mode of frequency omega is omega*dt <= 6/11,
not the 0.72 of plain AB3.  The reference never checks it
(src/mesh.cpp:1566-1621 only snaps dt), so the library reports omega_max and
the smallest stable step count."""
import numpy as np
import pytest

from conftest import RADIUS, ecc_case_params

A, B, Cc = 23 / 12, -16 / 12, 5 / 12


def amplification(x):
    """Spectral radius of one loop step for the oscillator v' = -w eta, eta' = w v (x = w dt)."""
    M = np.zeros((6, 6))              # state: v, eta, fv(n-1), fv(n-2), fe(n-1), fe(n-2)
    M[0, 0], M[0, 1], M[0, 2], M[0, 3] = 1, -A * x, B, Cc
    M[1, :] = A * x * M[0, :]
    M[1, 1] += 1; M[1, 4] += B; M[1, 5] += Cc
    M[2, 1] = -x; M[3, 2] = 1
    M[4, :] = x * M[0, :]; M[5, 4] = 1
    return max(abs(np.linalg.eigvals(M)))


def test_forward_backward_ab3_limit_is_six_elevenths():
    assert amplification(6 / 11 - 1e-6) <= 1 + 1e-9
    assert amplification(6 / 11 + 1e-3) > 1 + 1e-6
    assert all(amplification(x) < 1 for x in np.linspace(0.05, 0.54, 20))


def test_gravity_wave_omega_matches_eigs(grid_dir):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    path = grid_dir / "grid_3.txt"
    om = O.OracleMesh(path, RADIUS)
    rp, c, v = om.csr(0)
    G = sp.csr_matrix((v, c, rp), shape=(om.n_edges, om.n_cells))
    rp, c, v = om.csr(1)
    D = sp.csr_matrix((v, c, rp), shape=(om.n_cells, om.n_edges))
    ev = sla.eigs(-(D @ G) * 0.113 * 1e4, k=1, which="LM", return_eigenvectors=False)
    w_ref = np.sqrt(abs(ev[0]))
    w = g.Mesh.from_file(path, RADIUS).gravity_wave_omega(0.113, 1e4, 2000)
    assert abs(w / w_ref - 1) < 1e-3


@pytest.mark.parametrize("ratio,grows", [(0.9, False), (1.15, True)])
def test_oracle_run_follows_the_limit(grid_dir, ratio, grows):
    """A level-3 run with omega_max*dt just below / above 6/11 decays / blows up."""
    import geodesicodis_gb300 as g
    from oracle import pyoracle as O
    path = grid_dir / "grid_3.txt"
    p = ecc_case_params()
    w = g.Mesh.from_file(path, RADIUS).gravity_wave_omega(p["g"], p["h"], 2000)
    p["dt"] = ratio * (6 / 11) / w
    s = O.OracleSolver(O.OracleMesh(path, RADIUS), **p)
    pw = s.run(3000)
    blew = not np.isfinite(pw[-1]) or pw[-1] > 1e6 * np.nanmax(pw[:500])
    assert blew == grows


def test_stable_steps_per_orbit(built):
    import geodesicodis_gb300 as g
    P = 118394.0
    n = g.stable_steps_per_orbit(P, 1.9111e-2, 1.0)
    assert n % 100 == 0 and P / n * 1.9111e-2 <= 6 / 11 and P / (n - 100) * 1.9111e-2 > 6 / 11


def test_loading_factors_follow_reference_formula(built):
    """gamma_l of src/boundaryConditions.cpp:29-76 (rigidity 40 GPa, rho_b 1609.22, rho_o 1000)."""
    import geodesicodis_gb300 as g
    gam = g.loading_factors(0.113, RADIUS, 16)
    for l in (2, 5, 16):
        eff = (2 * l * l + 4 * l + 3) / l * 40e9 / (1609.22 * 0.113 * RADIUS)
        k, h = -1 / (1 + eff), -(2 * l + 1) / 3 / (1 + eff)
        assert abs(gam[l] - (1 + k - h) * 3 * 1000 / ((2 * l + 1) * 1609.22)) < 1e-15
    f = g.benchmark_sh_factors(0.113, RADIUS, 16)
    assert np.all(f[2:] / gam[2:] >= 0.5) and np.all(f[2:] / gam[2:] <= 1.5) and f[0] == f[1] == 0
    assert np.all(f < 1)          # every degree keeps a restoring (positive) effective gravity
