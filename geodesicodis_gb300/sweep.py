"""Parameter sweeps over the batched engine (odis_batch_*).

The sweep distribution: mesh level uniform over a set of levels, ocean
thickness log-uniform in 0.1-100 km, linear drag log-uniform in 1e-7-1e-4 1/s,
eccentricity uniform in 0.001-0.01, obliquity uniform in 0-0.5 degrees, with
the eccentricity + obliquity (FULL) tide, src/tidalPotentials.cpp:158-174.

Each member runs at max(2000, stable) steps per orbit, where `stable` is the
smallest multiple of `quantum` steps with omega_max * dt <= 0.95 * 6/11 for
its mesh and thickness (omega_max from the discrete gravity-wave operator,
omega_max ~ sqrt(h)).  The nominal 2000 steps per orbit would put thick
oceans on fine meshes beyond the stability limit of the reference's
forward-backward AB3 loop.
"""
from __future__ import annotations

import math

import numpy as np

from . import Batch, Mesh, POT_FULL, derive_time, make_params, stable_steps_per_orbit

RADIUS, GRAV, ANGVEL_IN = 252.1e3, 0.113, 5.307e-5
NOMINAL_STEPS = 2000


def draw_parameters(count: int, seed: int, levels=(4, 5, 6)) -> dict:
    """Seeded draws, in this order: level, log10 h, log10 alpha, ecc, obliquity (degrees)."""
    rng = np.random.default_rng(seed)
    level = rng.choice(np.asarray(levels), count)
    h = 10.0 ** rng.uniform(2.0, 5.0, count)
    alpha = 10.0 ** rng.uniform(-7.0, -4.0, count)
    ecc = rng.uniform(0.001, 0.01, count)
    obl_deg = rng.uniform(0.0, 0.5, count)
    return {"level": level, "h": h, "alpha": alpha, "ecc": ecc, "obliq": np.deg2rad(obl_deg)}


class SweepMeshes:
    """Meshes by level, with the unit-thickness gravity-wave frequency of each."""

    def __init__(self, levels, radius=RADIUS, g=GRAV):
        self.levels = sorted(set(int(x) for x in levels))
        self.meshes = {lv: Mesh.generate(lv, radius) for lv in self.levels}
        self.omega1 = {lv: self.meshes[lv].gravity_wave_omega(g, 1.0) for lv in self.levels}

    def index(self, level: int) -> int:
        return self.levels.index(int(level))

    def steps_per_orbit(self, level: int, h: float, period: float, quantum: int = 400) -> int:
        stable = stable_steps_per_orbit(period, self.omega1[int(level)] * math.sqrt(h), 0.95)
        n = max(NOMINAL_STEPS, stable)
        return int(math.ceil(n / quantum) * quantum)


def sweep_members(params: dict, meshes: SweepMeshes, period: float, quantum: int = 400) -> list[dict]:
    out = []
    for i in range(len(params["h"])):
        lv = int(params["level"][i])
        out.append(dict(mesh=meshes.index(lv), steps_per_orbit=meshes.steps_per_orbit(lv, params["h"][i], period, quantum),
                        h=float(params["h"][i]), alpha=float(params["alpha"][i]), ecc=float(params["ecc"][i]),
                        obliq=float(params["obliq"][i])))
    return out


def common_params():
    angvel, period, _, _ = derive_time(ANGVEL_IN, 59.197)
    return make_params(radius=RADIUS, g=GRAV, angvel=angvel, h=1.0, alpha=0.0, dt=1.0, potential=POT_FULL), period


def make_sweep(count=256, seed=2, levels=(4, 5, 6), quantum: int = 400):
    """(Batch, members, meshes, period) for `count` seeded draws."""
    common, period = common_params()
    prm = draw_parameters(count, seed, levels)
    meshes = SweepMeshes(levels)
    members = sweep_members(prm, meshes, period, quantum)
    batch = Batch(common, [meshes.meshes[lv] for lv in meshes.levels], members)
    return batch, members, meshes, period


def cell_steps(members, meshes: SweepMeshes, orbits: float) -> int:
    """Total cell-steps of running every member `orbits` orbits."""
    tot = 0
    for m in members:
        n_cells = meshes.meshes[meshes.levels[m["mesh"]]].n_cells
        tot += n_cells * int(round(orbits * m["steps_per_orbit"]))
    return tot


def orbits_to_converge(orbit_power: np.ndarray, tol: float = 1e-4) -> np.ndarray:
    """First orbit k (1-based count of orbits run) with |P_k - P_{k-1}| / P_k < tol, or -1."""
    P = np.asarray(orbit_power, np.float64)
    out = np.full(P.shape[0], -1, np.int64)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.abs(np.diff(P, axis=1)) / np.abs(P[:, 1:])
    for i in range(P.shape[0]):
        hit = np.flatnonzero(rel[i] < tol)
        if hit.size:
            out[i] = int(hit[0]) + 2
    return out
