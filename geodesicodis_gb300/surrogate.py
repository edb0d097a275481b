"""Learned warm start of the tidal time loop.

A network maps the ocean parameters to the spherical-harmonic coefficients, to
degree 8, of the converged tidal state at the start of an orbit and a quarter
orbit later: eta, and the velocity potential chi and stream function psi of the
edge-normal velocity (v_e = n_e . grad chi + n_e . (k x grad psi)).  The LTE is
linear and the FULL tide is linear in eccentricity and obliquity, so the
network's input is (log thickness, log drag) only and its output is two
response heads, per unit eccentricity and per unit obliquity, mixed by the
member's amplitudes.  The predicted phase-0 state is loaded into the batched
integrator, which runs on from it until the orbit-mean dissipated power
converges: the plain integrator decides convergence, and a zero start is the
fallback and the reference for the number of orbits.

Everything that computes runs in this library's kernels: the integrator
(odis_batch_*), the projections of the states onto the harmonic bases
(odis_batch_project) and the network's training and inference (odis_mlp_*).
The harmonic bases and their least-squares inverses are set up once per mesh
on the host.

Convergence (the reference's `converge` key is unused): P_k = mean power over
orbit k; converged at the first k >= 2 with |P_k - P_{k-1}| / P_k < 1e-4.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import MLP, Batch
from . import sweep as S

LMAX = 8
PHASES = 8                 # parts of the last orbit of a round at which the state is projected
MODEL_PHASES = (0, 2)      # the phases the network predicts: the orbit start and a quarter orbit later
TOL = 1e-4


# ---------------------------------------------------------------------------
# real spherical harmonics on the mesh
# ---------------------------------------------------------------------------
def legendre(lmax: int, x: np.ndarray) -> dict:
    """4pi-normalised associated Legendre functions P[l, m](x), no Condon-Shortley phase."""
    x = np.asarray(x, np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {(0, 0): np.ones_like(x)}
    for m in range(1, lmax + 1):
        f = math.sqrt(3.0) if m == 1 else math.sqrt((2 * m + 1) / (2.0 * m))
        P[(m, m)] = f * s * P[(m - 1, m - 1)]
    for m in range(0, lmax):
        P[(m + 1, m)] = math.sqrt(2 * m + 3) * x * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((2 * l - 1) * (2 * l + 1) / ((l - m) * (l + m)))
            b = math.sqrt((2 * l + 1) * (l + m - 1) * (l - m - 1) / ((l - m) * (l + m) * (2 * l - 3)))
            P[(l, m)] = a * x * P[(l - 1, m)] - b * P[(l - 2, m)]
    return P


def harmonics(lmax: int):
    """(l, m) list of the real harmonics: m >= 0 -> P_lm cos(m lon), m < 0 -> P_l|m| sin(|m| lon)."""
    return [(l, m) for l in range(lmax + 1) for m in range(-l, l + 1)]


def real_sh(lmax: int, lat: np.ndarray, lon: np.ndarray) -> np.ndarray:
    P = legendre(lmax, np.sin(lat))
    cols = []
    for l, m in harmonics(lmax):
        cols.append(P[(l, abs(m))] * (np.cos(m * lon) if m >= 0 else np.sin(-m * lon)))
    return np.stack(cols, axis=1)


class MeshBasis:
    """Harmonic bases of one mesh and their least-squares inverses.

    eta:  Y [N, K] at the nodes, K = (lmax+1)^2.
    velocity: [n.grad Y_lm | n.(k x grad Y_lm)] [E, 2(K-1)] at the face centres
    (l >= 1; the face normal n is (east, north), from node 0 to node 1).
    """

    def __init__(self, mesh, radius: float, lmax: int = LMAX):
        self.lmax = lmax
        lat, lon = mesh.field(12), mesh.field(13)
        flat, flon = mesh.field(4), mesh.field(5)
        nx, ny = mesh.field(8), mesh.field(9)
        self.Y = real_sh(lmax, lat, lon)
        h = 1e-6
        dlon = (real_sh(lmax, flat, flon + h) - real_sh(lmax, flat, flon - h)) / (2 * h)
        dlat = (real_sh(lmax, flat + h, flon) - real_sh(lmax, flat - h, flon)) / (2 * h)
        ge = dlon / (radius * np.cos(flat))[:, None]          # east component of grad Y
        gn = dlat / radius                                    # north component
        grad_n = nx[:, None] * ge + ny[:, None] * gn          # n . grad Y
        curl_n = -nx[:, None] * gn + ny[:, None] * ge         # n . (k x grad Y)
        self.V = np.concatenate([grad_n[:, 1:], curl_n[:, 1:]], axis=1)
        self.K = self.Y.shape[1]
        self.KV = self.V.shape[1]
        self.Pe = np.linalg.pinv(self.Y)                      # [K, N]
        self.Pv = np.linalg.pinv(self.V)                      # [KV, E]
        self.Pe32 = self.Pe.astype(np.float32)
        self.Pv32 = self.Pv.astype(np.float32)

    @property
    def n_coef(self) -> int:
        return self.KV + self.K

    def state(self, coef: np.ndarray):
        """(v [.., E], eta [.., N]) from coefficient rows [.., KV + K] (velocity first)."""
        return coef[..., :self.KV] @ self.V.T, coef[..., self.KV:] @ self.Y.T


# ---------------------------------------------------------------------------
# running members to convergence
# ---------------------------------------------------------------------------
def converged_at(history: list[float], tol: float = TOL) -> int:
    """Orbit count (1-based) at which the orbit-mean power first changed by < tol, or -1."""
    for k in range(1, len(history)):
        if history[k] != 0 and abs(history[k] - history[k - 1]) / abs(history[k]) < tol:
            return k + 1
    return -1


def run_to_convergence(common, mesh, members, basis: MeshBasis | None, v0=None, eta0=None, round_orbits: int = 10,
                       max_orbits: int = 400, log=None, tol: float = TOL):
    """Run every member (all on `mesh`) from (v0, eta0) (None: rest) until its orbit-mean power converges.

    Members still running are re-batched after every round of `round_orbits`
    orbits (state carried over at orbital phase 0; the integrator restarts with
    a forward-Euler step).  The last orbit of each round is run in PHASES equal
    parts and, with `basis`, the state is projected after each part.  Returns
    dict(orbits [m], power [m] (last orbit mean), history [m] lists,
    coef [m, PHASES, n_coef] (phase p = p/PHASES orbits after the last
    completed orbit; p = 0 last), v [m, E], eta [m, N]).
    """
    m = len(members)
    E, N = mesh.n_edges, mesh.n_cells
    hist = [[] for _ in range(m)]
    orbits = np.full(m, -1, np.int64)
    coef = np.zeros((m, PHASES, basis.n_coef)) if basis is not None else None
    v_fin, e_fin = np.zeros((m, E)), np.zeros((m, N))
    active = np.arange(m)
    v_cur = np.zeros((m, E)) if v0 is None else np.asarray(v0, np.float64).copy()
    e_cur = np.zeros((m, N)) if eta0 is None else np.asarray(eta0, np.float64).copy()
    done_orbits = 0
    steps = 0
    while active.size and done_orbits < max_orbits:
        mem = [dict(members[i], mesh=0) for i in active]
        b = Batch(common, [mesh], mem)
        if done_orbits > 0 or v0 is not None:
            b.set_mesh_members(0, v_cur[active], e_cur[active])
        r = min(round_orbits, max_orbits - done_orbits)
        op_parts = []
        if r > 1:
            op, _ = b.run(orbits=r - 1)
            op_parts.append(op)
        eighth = np.zeros((active.size, PHASES))
        for p in range(PHASES):
            op8, _ = b.run(orbits=1.0 / PHASES)
            eighth[:, p] = op8[:, 0]
            if basis is not None:
                c = b.project(0, basis.Pv32, basis.Pe32)
                coef[active, (p + 1) % PHASES] = c
        last = eighth.sum(axis=1, keepdims=True)          # each part holds its steps' power / steps per orbit
        op_all = np.concatenate(op_parts + [last], axis=1) if op_parts else last
        v, e = b.get_mesh_members(0)
        steps += sum(int(round(r * mm["steps_per_orbit"])) for mm in mem) * N
        b.close()
        done_orbits += r
        keep = []
        for k, i in enumerate(active):
            hist[i].extend(op_all[k].tolist())
            v_cur[i], e_cur[i] = v[k], e[k]
            c = converged_at(hist[i], tol)
            if c > 0:
                orbits[i] = c
                v_fin[i], e_fin[i] = v[k], e[k]
            else:
                keep.append(i)
        if log:
            log(f"  {done_orbits} orbits: {m - len(keep)}/{m} converged")
        active = np.array(keep, np.int64)
    for i in active:                                   # not converged within max_orbits
        v_fin[i], e_fin[i] = v_cur[i], e_cur[i]
    power = np.array([h[-1] if h else 0.0 for h in hist])
    return dict(orbits=orbits, power=power, history=hist, coef=coef, v=v_fin, eta=e_fin, cell_steps=steps,
                max_orbits=max_orbits)


# ---------------------------------------------------------------------------
# features, targets and the network
# ---------------------------------------------------------------------------
def features(prm: dict) -> np.ndarray:
    """Network input: the response per unit forcing depends on thickness and drag only."""
    return np.stack([np.log10(prm["h"]), np.log10(prm["alpha"])], axis=1)


def mixing(prm: dict) -> np.ndarray:
    """Forcing amplitudes the response is linear in (eccentricity, obliquity), scaled to O(1)."""
    return np.stack([prm["ecc"] / 0.01, np.rad2deg(prm["obliq"]) / 0.5], axis=1)


class Surrogate:
    """Network(s) + the scalings between their units and the harmonic coefficients.

    ensemble > 1 trains that many networks of the same shape on the same data, each from its own
    initialisation and minibatch order (seeds seed, seed + 1, ...), and predicts their mean.  The
    prediction error of one network is dominated by its variance between fits (it grows with more
    epochs), which the mean reduces."""

    def __init__(self, basis: MeshBasis, width=512, depth=3, seed=0, ensemble: int = 1):
        self.basis = basis
        self.n_out = len(MODEL_PHASES) * basis.n_coef
        self.seed = seed
        self.nets = [MLP(2, width, depth, self.n_out, 2, seed=seed + k) for k in range(max(1, int(ensemble)))]
        self.net = self.nets[0]
        self.mu = self.sd = self.scale = None

    def _targets(self, coef: np.ndarray, prm: dict) -> np.ndarray:
        """coef [n, PHASES, KV+K] -> network units (the MODEL_PHASES rows): velocity coefficients times h
        (transport), per-output scale."""
        t = coef[:, list(MODEL_PHASES)].copy()
        t[:, :, :self.basis.KV] *= prm["h"][:, None, None]
        return t.reshape(t.shape[0], -1)

    def _coef(self, t: np.ndarray, prm: dict) -> np.ndarray:
        """Network units -> coef [n, len(MODEL_PHASES), KV+K]."""
        c = t.reshape(t.shape[0], len(MODEL_PHASES), self.basis.n_coef).copy()
        c[:, :, :self.basis.KV] /= prm["h"][:, None, None]
        return c

    def fit(self, prm: dict, coef: np.ndarray, epochs=800, batch=128, lr=1e-3, seed=0, orbits=None):
        """Train on converged coefficients.  Each sample's loss is its relative squared error, weighted by
        sqrt(orbits) when the zero-start orbit counts are given: the slowly converging (low-drag) members
        are where a warm start saves orbits.  Returns the first network's loss per epoch."""
        x = features(prm)
        self.mu, self.sd = x.mean(axis=0), x.std(axis=0) + 1e-12
        t = self._targets(coef, prm)
        mix = mixing(prm)
        # robust per-output scale (the median case is O(1); resonant cases stay large)
        self.scale = np.median(np.abs(t), axis=0) / np.median(np.abs(mix).sum(axis=1)) + 1e-30
        tn = t / self.scale
        w = 1.0 / np.maximum(np.sum(tn ** 2, axis=1), 1e-30) * tn.shape[1]
        if orbits is not None:
            cost = np.sqrt(np.maximum(np.asarray(orbits, np.float64), 1.0))
            w = w * cost / cost.mean()
        xn = (x - self.mu) / self.sd
        losses = None
        for k, net in enumerate(self.nets):
            lk = net.train(xn, tn, mix, w, epochs=epochs, batch=batch, lr=lr, seed=seed + k)
            losses = lk if losses is None else losses
        return losses

    def predict_coef(self, prm: dict, members: int | None = None) -> np.ndarray:
        """Predicted coefficients: the mean of the first `members` networks (all by default)."""
        x = (features(prm) - self.mu) / self.sd
        mix = mixing(prm)
        nets = self.nets[:members] if members else self.nets
        tn = np.mean([net.predict(x, mix).astype(np.float64) for net in nets], axis=0)
        return self._coef(tn * self.scale, prm)

    def warm_state(self, prm: dict, members: int | None = None):
        """Predicted phase-0 (v, eta) for each parameter set."""
        c = self.predict_coef(prm, members)[:, 0, :]
        return self.basis.state(c)


def members_from(prm: dict, meshes: S.SweepMeshes, period: float) -> list[dict]:
    return S.sweep_members(prm, meshes, period)


def relative_coef_error(pred: np.ndarray, true: np.ndarray) -> np.ndarray:
    d = (pred - true).reshape(pred.shape[0], -1)
    t = true.reshape(true.shape[0], -1)
    return np.linalg.norm(d, axis=1) / np.maximum(np.linalg.norm(t, axis=1), 1e-300)


def refine_parameters(prm: dict, err: np.ndarray, orbits: np.ndarray, count: int, seed: int) -> dict:
    """Extra training draws around the members the network predicts worst, weighted by their orbit cost:
    the top count/4 by err * sqrt(orbits), four draws each, thickness within +-2.3 % (resonances are a few
    per mille wide at low drag) and drag within a factor 1.6, fresh eccentricity and obliquity."""
    rng = np.random.default_rng(seed)
    score = err * np.sqrt(np.maximum(orbits, 1.0))
    pick = np.argsort(score)[::-1][:max(1, count // 4)]
    src = np.repeat(pick, 4)[:count]
    n = src.size
    h = np.clip(prm["h"][src] * 10.0 ** rng.uniform(-0.01, 0.01, n), 100.0, 1e5)
    alpha = np.clip(prm["alpha"][src] * 10.0 ** rng.uniform(-0.2, 0.2, n), 1e-7, 1e-4)
    return {"level": prm["level"][src], "h": h, "alpha": alpha, "ecc": rng.uniform(0.001, 0.01, n),
            "obliq": np.deg2rad(rng.uniform(0.0, 0.5, n))}


def experiment(n_train=4096, n_test=512, level=5, seed_train=3, seed_test=4, epochs=800, batch=128, lr=1e-3,
               round_orbits=10, max_orbits=400, log=print, save=None, tol: float = TOL, refine: int = 0,
               ensemble: int = 1) -> dict:
    """Train on solver runs, then compare orbits to convergence from rest and from the warm start.
    refine > 0: after the first fit, `refine` more training members are drawn around the worst-predicted
    costly ones (refine_parameters), run to convergence from the network's own warm start, and the
    network is trained again on all of them.  ensemble > 1: the warm start is the mean of that many
    networks (Surrogate), and the held-out members also run from the first network alone, on the same
    data, for comparison."""
    t0 = time.time()
    common, period = S.common_params()
    meshes = S.SweepMeshes((level,))
    mesh = meshes.meshes[level]
    basis = MeshBasis(mesh, S.RADIUS)
    ptr = S.draw_parameters(n_train, seed_train, (level,))
    pte = S.draw_parameters(n_test, seed_test, (level,))
    mtr = members_from(ptr, meshes, period)
    mte = members_from(pte, meshes, period)
    log(f"setup {time.time() - t0:.1f} s; training runs ({n_train})")
    t1 = time.time()
    tr = run_to_convergence(common, mesh, mtr, basis, round_orbits=round_orbits, max_orbits=max_orbits, log=log, tol=tol)
    t_data = time.time() - t1
    log(f"training data {t_data:.1f} s, {tr['cell_steps']:.3e} cell-steps")
    sur = Surrogate(basis, ensemble=ensemble)
    t2 = time.time()
    orb_tr = np.where(tr["orbits"] > 0, tr["orbits"], max_orbits + 1)
    losses = sur.fit(ptr, tr["coef"], epochs=epochs, batch=batch, lr=lr, orbits=orb_tr)
    t_fit = time.time() - t2
    log(f"training {t_fit:.1f} s, loss {losses[0]:.3e} -> {losses[-1]:.3e}")
    t_refine = 0.0
    if refine > 0:
        t5 = time.time()
        err_tr = relative_coef_error(sur.predict_coef(ptr)[:, 0], tr["coef"][:, 0])
        pre = refine_parameters(ptr, err_tr, orb_tr, refine, seed_train + 1000)
        mre = members_from(pre, meshes, period)
        v_r, e_r = sur.warm_state(pre)
        rr = run_to_convergence(common, mesh, mre, basis, v0=v_r, eta0=e_r, round_orbits=round_orbits,
                                max_orbits=max_orbits, log=log, tol=tol)
        ptr = {k: np.concatenate([ptr[k], pre[k]]) for k in ptr}
        tr["coef"] = np.concatenate([tr["coef"], rr["coef"]])
        tr["cell_steps"] += rr["cell_steps"]
        # their orbit cost from rest is unknown: the source member's stands in
        src_orbits = orb_tr[np.argsort(err_tr * np.sqrt(np.maximum(orb_tr, 1.0)))[::-1][:max(1, refine // 4)]]
        orb_tr = np.concatenate([orb_tr, np.repeat(src_orbits, 4)[:refine]])
        sur = Surrogate(basis, ensemble=ensemble)
        losses = sur.fit(ptr, tr["coef"], epochs=epochs, batch=batch, lr=lr, orbits=orb_tr)
        t_refine = time.time() - t5
        log(f"refinement: {refine} members around the worst-predicted, {t_refine:.1f} s, loss -> {losses[-1]:.3e}")
    # held-out: zero start (also gives the true converged coefficients) and warm start
    t3 = time.time()
    zero = run_to_convergence(common, mesh, mte, basis, round_orbits=round_orbits, max_orbits=max_orbits, log=log, tol=tol)
    t_zero = time.time() - t3
    v_w, e_w = sur.warm_state(pte)
    t4 = time.time()
    warm = run_to_convergence(common, mesh, mte, None, v0=v_w, eta0=e_w, round_orbits=round_orbits,
                              max_orbits=max_orbits, log=log, tol=tol)
    t_warm = time.time() - t4
    single = None
    if len(sur.nets) > 1:           # the first network alone, for comparison
        v_s, e_s = sur.warm_state(pte, members=1)
        single = run_to_convergence(common, mesh, mte, None, v0=v_s, eta0=e_s, round_orbits=round_orbits,
                                    max_orbits=max_orbits, log=log, tol=tol)
    # the best a degree-8 warm start can do: start from the projection of the converged state itself
    v_t, e_t = basis.state(zero["coef"][:, 0, :])
    best = run_to_convergence(common, mesh, mte, None, v0=v_t, eta0=e_t, round_orbits=round_orbits,
                              max_orbits=max_orbits, log=log, tol=tol)
    pred = sur.predict_coef(pte)
    err = relative_coef_error(pred[:, 0], zero["coef"][:, 0])         # the phase-0 state the warm start loads
    err1 = relative_coef_error(sur.predict_coef(pte, members=1)[:, 0], zero["coef"][:, 0]) if single else err
    if save:        # per member: parameters, orbit counts, prediction error (no coefficient arrays: a few hundred kB)
        np.savez_compressed(save, ptr_h=ptr["h"], ptr_alpha=ptr["alpha"], ptr_ecc=ptr["ecc"], ptr_obliq=ptr["obliq"],
                            pte_h=pte["h"], pte_alpha=pte["alpha"], pte_ecc=pte["ecc"], pte_obliq=pte["obliq"],
                            err_test=err, orbits_train=tr["orbits"], orbits_zero=zero["orbits"],
                            orbits_warm=warm["orbits"], orbits_best=best["orbits"], losses=losses,
                            power_zero=zero["power"], power_warm=warm["power"], err_test_single=err1,
                            orbits_warm_single=single["orbits"] if single else warm["orbits"])
    oz = np.where(zero["orbits"] > 0, zero["orbits"], max_orbits + 1)
    ow = np.where(warm["orbits"] > 0, warm["orbits"], max_orbits + 1)
    ob = np.where(best["orbits"] > 0, best["orbits"], max_orbits + 1)
    both = (zero["orbits"] > 0) & (warm["orbits"] > 0)
    pdiff = np.abs(warm["power"] - zero["power"]) / np.abs(zero["power"])
    res = {
        "n_train": n_train, "n_test": n_test, "level": level, "cells": mesh.n_cells,
        "orbits_zero_median": float(np.median(oz)), "orbits_warm_median": float(np.median(ow)),
        "orbits_zero_mean": float(np.mean(oz)), "orbits_warm_mean": float(np.mean(ow)),
        "orbits_ratio_total": float(np.sum(oz) / np.sum(ow)),
        "orbits_ratio_median_per_case": float(np.median(oz / ow)),
        "frac_cases_3x": float(np.mean(oz >= 3 * ow)),
        "orbits_truncated_truth_median": float(np.median(ob)), "orbits_truncated_truth_mean": float(np.mean(ob)),
        "orbits_ratio_total_truncated_truth": float(np.sum(oz) / np.sum(ob)),
        "converged_power_within_1e3": float(np.mean(pdiff[both] < 1e-3)) if both.any() else None,
        "zero_not_converged": int(np.sum(zero["orbits"] <= 0)), "warm_not_converged": int(np.sum(warm["orbits"] <= 0)),
        "converged_power_rel_diff_median": float(np.median(pdiff[both])) if both.any() else None,
        "converged_power_rel_diff_max": float(np.max(pdiff[both])) if both.any() else None,
        "coef_rel_err_median": float(np.median(err)), "coef_rel_err_p90": float(np.quantile(err, 0.9)),
        "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
        "seconds": {"data": t_data, "train": t_fit, "refine": t_refine, "zero": t_zero, "warm": t_warm},
        "refine": refine, "ensemble": len(sur.nets),
        "loss_weight": "relative squared error x sqrt(zero-start orbits)",
        "epochs": epochs, "batch": batch, "lr": lr, "round_orbits": round_orbits,
        "cell_steps": {"data": tr["cell_steps"], "zero": zero["cell_steps"], "warm": warm["cell_steps"]},
        "max_orbits": max_orbits, "tol": tol,
    }
    if single is not None:
        os1 = np.where(single["orbits"] > 0, single["orbits"], max_orbits + 1)
        res["single_network"] = {"orbits_ratio_total": float(np.sum(oz) / np.sum(os1)),
                                 "orbits_warm_mean": float(np.mean(os1)),
                                 "warm_not_converged": int(np.sum(single["orbits"] <= 0)),
                                 "coef_rel_err_median": float(np.median(err1)),
                                 "coef_rel_err_p90": float(np.quantile(err1, 0.9))}
    return res
