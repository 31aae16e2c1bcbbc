"""Frequency meshes (host side).

Restates src/Frequency/mesh.jl: ``get_mesh`` (mesh.jl:86-121) builds num + 1
frequencies, 0 first, linear up to ``linear`` and logarithmic up to
``upper``; ``Mesh`` (mesh.jl:16-27) bundles the self-energy, s(u)-channel,
t-channel and correlation meshes.  The ``num_*`` fields are array lengths
(num_σ + 1 etc.) exactly as in the reference.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def get_mesh(linear: float, upper: float, num: int, p: float) -> np.ndarray:
    """(num + 1) frequencies: 0, p*num linear points up to ``linear``, the rest log-spaced to ``upper``."""
    if not linear > 0.0:
        raise ValueError("Linear bound must be larger than zero.")
    if not upper > 0.0:
        raise ValueError("Upper bound must be larger than zero.")
    if not linear < upper:
        raise ValueError("Linear bound must be smaller than upper bound.")
    num_lin = int(math.ceil(p * num))
    num_log = num - num_lin
    if not num_log > 0:
        raise ValueError("Number of frequencies is too small.")
    h = linear / num_lin
    xi = (upper / linear) ** (1.0 / num_log)
    mesh = np.zeros(num + 1)
    for i in range(1, num_lin + 1):
        mesh[i] = i * h
    for i in range(1, num_log + 1):
        mesh[num_lin + i] = xi ** i * linear
    return mesh


@dataclass
class Mesh:
    """Frequency meshes of one flow step (mesh.jl:16-27)."""

    num_sigma: int
    num_omega: int
    num_nu: int
    num_chi: int
    sigma: np.ndarray
    omega_s: np.ndarray
    nu_s: np.ndarray
    omega_t: np.ndarray
    nu_t: np.ndarray
    chi: np.ndarray

    def copy(self) -> "Mesh":
        return Mesh(self.num_sigma, self.num_omega, self.num_nu, self.num_chi, self.sigma.copy(),
                    self.omega_s.copy(), self.nu_s.copy(), self.omega_t.copy(), self.nu_t.copy(),
                    self.chi.copy())


# launch! defaults (src/Launcher/Launcher.jl:574-586)
DEFAULT_P_SIGMA = (0.4, 1.5, 1.0)
DEFAULT_P_OMEGA = (0.4, 0.02, 0.05, 0.05, 40.0, 1.0)
DEFAULT_P_NU = (0.4, 0.02, 0.05, 0.03, 30.0, 1.0)
DEFAULT_P_CHI = (0.4, 0.02, 0.05, 0.01, 20.0, 1.0)
DEFAULT_LINS = (5.0, 2.0, 6.0, 4.0, 4.0)
DEFAULT_BOUNDS = (0.5, 50.0, 200.0, 150.0, 100.0)


def initial_mesh(Lam: float, num_sigma: int, num_omega: int, num_nu: int, num_chi: int,
                 p_sigma=DEFAULT_P_SIGMA, p_omega_s=DEFAULT_P_OMEGA, p_nu_s=DEFAULT_P_NU,
                 p_omega_t=DEFAULT_P_OMEGA, p_nu_t=DEFAULT_P_NU, p_chi=DEFAULT_P_CHI,
                 lins=DEFAULT_LINS, bounds=DEFAULT_BOUNDS) -> Mesh:
    """Meshes that ``launch!`` builds at cutoff Λ (Launcher.jl:667-673)."""
    b = max(Lam, bounds[0])
    sigma = get_mesh(lins[1] * Lam, bounds[1] * b, num_sigma, p_sigma[0]) * p_sigma[2]
    omega_s = get_mesh(lins[2] * Lam, bounds[2] * b, num_omega, p_omega_s[0]) * p_omega_s[5]
    nu_s = get_mesh(lins[3] * Lam, bounds[3] * b, num_nu, p_nu_s[0]) * p_nu_s[5]
    omega_t = get_mesh(lins[2] * Lam, bounds[2] * b, num_omega, p_omega_t[0]) * p_omega_t[5]
    nu_t = get_mesh(lins[3] * Lam, bounds[3] * b, num_nu, p_nu_t[0]) * p_nu_t[5]
    chi = get_mesh(lins[4] * Lam, bounds[4] * b, num_chi, p_chi[0]) * p_chi[5]
    return Mesh(num_sigma + 1, num_omega + 1, num_nu + 1, num_chi + 1, sigma, omega_s, nu_s,
                omega_t, nu_t, chi)
