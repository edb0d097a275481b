"""Closed-form solution of the linear LTE with linear drag for the westward
obliquity tide (degree 2, order 1, frequency Omega): the reference's
analyticalLTE, case OBLIQ_WEST (src/analyticalLTE.cpp:22-44 for p_n, q_n, K_n,
L_n; :62-80 for the parameters; :133-181 for the solution), restated in numpy.

Test infrastructure: the oracle's check on the product's analytical initial
state (odis_analytical_state) and the physics pin of the discrete loop.

The closed form keeps only Psi_11 and Phi_21.  Without drag it solves the
continuous equations exactly (Phi_21 = 0, eta = 0: a Rossby-Haurwitz flow); with
drag the neglected coupling to Psi_31 leaves a momentum residual of order
alpha / (2 Omega) relative to the tendency (about 30 % at alpha = 1e-5), so the
pin runs without drag.

With colatitude theta = pi/2 - lat, lambda = lon and w = -Omega:
  lam = w / (2 Omega),  lambs = 4 Omega^2 r^2 / (g h)  (Lamb's parameter)
  L_1 = lam + 1/2 + i alpha / (2 Omega),  K_2 = lam + 1/6 - 6 / (lambs lam) + i alpha / (2 Omega)
  Psi_11 = (Omega r^2 obl / 4) / (q_1(1) - K_2 L_1 / p_2(1)),  Phi_21 = -i L_1 / p_2(1) Psi_11
  u = Re[(-Psi_11 / 3 + i Phi_21) Y_21 e^{-i w t}] / (r sin theta)           (east)
  v = Re[-(i Psi_11 Y_11 + Phi_21 (4 Y_31 - 9 Y_11) / 5) e^{-i w t}] / (r sin theta)   (north)
  eta = Re[i 6 h / (r^2 w) Phi_21 Y_21 e^{-i w t}]
with Y_11 = sin theta e^{i lambda}, Y_21 = 3 cos theta sin theta e^{i lambda},
Y_31 = 3/2 (5 cos^2 theta - 1) sin theta e^{i lambda}; time derivatives are
-i w times the complex amplitudes.
"""
from __future__ import annotations

import numpy as np


def _pn(n, m):
    return (n + 1) * (n + m) / (n * (2 * n + 1))


def _qn(n, m):
    return n * (n + 1 - m) / ((n + 1) * (2 * n + 1))


def coefficients(radius, g, angvel, h, alpha, obliq):
    """(Psi_11, Phi_21, w)."""
    w = -angvel
    lam = w / (2 * angvel)
    lambs = 4 * angvel ** 2 * radius ** 2 / (g * h)
    damp = 1j * alpha / (2 * angvel)
    L1 = lam + 1.0 / 2.0 + damp
    K2 = lam + 1.0 / 6.0 - 6.0 / (lambs * lam) + damp
    U21 = 0.5 * angvel ** 2 * radius ** 2 * obliq
    psi = U21 / (2 * angvel) / (_qn(1, 1) - K2 * L1 / _pn(2, 1))
    phi = -1j * L1 / _pn(2, 1) * psi
    return psi, phi, w


def solution(lat, lon, t, *, radius, g, angvel, h, alpha, obliq):
    """(u_east, v_north, du/dt, dv/dt, eta, deta/dt) at points (lat, lon) (radians) and time t."""
    psi, phi, w = coefficients(radius, g, angvel, h, alpha, obliq)
    th = np.pi * 0.5 - np.asarray(lat, np.float64)
    e = np.exp(1j * np.asarray(lon, np.float64))
    st, ct = np.sin(th), np.cos(th)
    Y11 = st * e
    Y21 = 3 * ct * st * e
    Y31 = 1.5 * (5 * ct ** 2 - 1) * st * e
    ph = np.exp(-1j * w * t)
    U = (-1.0 / 3.0 * psi * Y21 + 1j * phi * Y21) * ph
    V = -(1j * psi * Y11 + phi * (4.0 * Y31 - 9.0 * Y11) / 5.0) * ph
    ETA = 1j * 6.0 / radius ** 2 * h / w * phi * Y21 * ph
    den = radius * st
    return (U.real / den, V.real / den, (-1j * w * U).real / den, (-1j * w * V).real / den,
            ETA.real, (-1j * w * ETA).real)


def state(face_lat, face_lon, nx, ny, node_lat, node_lon, t, dt, **p):
    """The reference's analyticalInitialConditions (src/initialConditions.cpp:150-211): face-normal
    velocity and its time derivative at t, t - dt, t - 2 dt; eta and its derivative likewise."""
    v = eta = None
    cols_v, cols_e = [], []
    with np.errstate(divide="ignore", invalid="ignore"):    # velocities at polar nodes are not used
        for k in range(3):
            u, vn, du, dvn, _, _ = solution(face_lat, face_lon, t - k * dt, **p)
            if k == 0:
                v = u * nx + vn * ny
            cols_v.append(du * nx + dvn * ny)
            _, _, _, _, et, det = solution(node_lat, node_lon, t - k * dt, **p)
            if k == 0:
                eta = et
            cols_e.append(det)
    return v, eta, np.stack(cols_v, axis=1), np.stack(cols_e, axis=1)
