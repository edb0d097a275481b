"""Host side of the warm start (CPU): harmonic bases, their inverses, the convergence rule."""
from __future__ import annotations

import numpy as np

from conftest import RADIUS


def test_real_harmonics_are_orthonormal_on_the_mesh(built):
    import geodesicodis_gb300 as g
    from geodesicodis_gb300 import surrogate as SU
    m = g.Mesh.generate(5, RADIUS)
    Y = SU.real_sh(8, m.field(12), m.field(13))
    A = m.field(3)
    Gm = (Y * A[:, None]).T @ Y / A.sum()          # int Y_k Y_k' dOmega / 4pi
    assert np.max(np.abs(Gm - np.eye(Y.shape[1]))) < 2e-2


def test_basis_round_trip_and_gradient_convention(built):
    import geodesicodis_gb300 as g
    from geodesicodis_gb300 import surrogate as SU
    m = g.Mesh.generate(4, RADIUS)
    B = SU.MeshBasis(m, RADIUS)
    rng = np.random.default_rng(0)
    c = rng.standard_normal((3, B.n_coef))
    v, eta = B.state(c)
    back = np.concatenate([v @ B.Pv.T, eta @ B.Pe.T], axis=1)
    assert np.max(np.abs(back - c)) < 1e-8 * np.max(np.abs(c))
    # the discrete gradient (G s)_e = (-m_e0 s_n0 + m_e1 s_n1) / d_e of a harmonic
    # projects onto the potential part of the same harmonic
    fn = m.topology()["face_nodes"]
    m0, m1, d = m.field(6), m.field(7), m.field(1)
    k = SU.harmonics(8).index((3, 2))
    s = B.Y[:, k]
    Gs = (-m0 * s[fn[:, 0]] + m1 * s[fn[:, 1]]) / d
    a = B.Pv @ Gs
    assert abs(a[k - 1] - 1.0) < 2e-2
    others = np.delete(a, k - 1)
    assert np.max(np.abs(others)) < 2e-2


def test_convergence_rule():
    from geodesicodis_gb300 import surrogate as SU
    assert SU.converged_at([1.0, 1.5, 1.6, 1.60001]) == 4
    assert SU.converged_at([1.0, 1.00001]) == 2
    assert SU.converged_at([1.0, 2.0, 3.0]) == -1
