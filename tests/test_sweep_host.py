"""Host side of the batched sweep (CPU): seeded parameter draws and the stable step counts."""
from __future__ import annotations

import math

import numpy as np


def test_draws_are_seeded_and_in_range(built):
    from geodesicodis_gb300 import sweep as S
    a = S.draw_parameters(300, 2)
    b = S.draw_parameters(300, 2)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    assert set(np.unique(a["level"])) <= {4, 5, 6}
    assert a["h"].min() >= 1e2 and a["h"].max() <= 1e5
    assert a["alpha"].min() >= 1e-7 and a["alpha"].max() <= 1e-4
    assert a["ecc"].min() >= 0.001 and a["ecc"].max() <= 0.01
    assert a["obliq"].min() >= 0 and a["obliq"].max() <= math.radians(0.5)


def test_steps_per_orbit_respect_the_stability_limit(built):
    import geodesicodis_gb300 as g
    from geodesicodis_gb300 import sweep as S
    _, period = S.common_params()
    M = S.SweepMeshes((3, 4))
    for lv in (3, 4):
        for h in (1e2, 1e3, 1e4, 1e5):
            n = M.steps_per_orbit(lv, h, period)
            assert n % 400 == 0 and n >= 2000
            w = M.meshes[lv].gravity_wave_omega(S.GRAV, h)
            assert w * period / n <= 0.95 * g.STABILITY_LIMIT + 1e-12
    # thicker oceans on finer meshes need more steps
    assert M.steps_per_orbit(4, 1e5, period) >= M.steps_per_orbit(3, 1e5, period)


def test_orbits_to_converge():
    from geodesicodis_gb300 import sweep as S
    P = np.array([[1.0, 1.2, 1.21, 1.210001], [1.0, 2.0, 3.0, 4.0]])
    np.testing.assert_array_equal(S.orbits_to_converge(P), [4, -1])
