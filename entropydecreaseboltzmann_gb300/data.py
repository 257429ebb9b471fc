"""Velocity grids and seeded synthetic initial data (numpy, FP64).

Grid: x_i = -R + i h, h = 2R/N (CalQ/BKW.h:124-133), row-major [i][j][k].
The Bobylev-Krook-Wu (BKW) solution is that of CalQ/BKW.h:114-116 and
CalQ/testfft.cpp:11-16 written with s = K(t) = 1 - exp(-t/6):
    f(v) = (2 pi s)^(-3/2) exp(-v^2/(2s)) ((5s-3)/(2s) + (1-s) v^2/(2 s^2)).
"""
from __future__ import annotations

import numpy as np


def grid(N: int, R: float):
    h = 2.0 * R / N
    x = -R + h * np.arange(N)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return h, X.reshape(-1), Y.reshape(-1), Z.reshape(-1)


def K(t):
    return 1.0 - np.exp(-np.asarray(t, dtype=np.float64) / 6.0)


def bkw_f(s, v2):
    return (2.0 * np.pi * s) ** -1.5 * np.exp(-v2 / (2.0 * s)) * (
        (5.0 * s - 3.0) / (2.0 * s) + (1.0 - s) / (2.0 * s * s) * v2)


def bkw_dfdt(s, v2):
    """d f / d t of the BKW solution (ds/dt = (1-s)/6)."""
    P = (2.0 * np.pi * s) ** -1.5 * np.exp(-v2 / (2.0 * s))
    G = (5.0 * s - 3.0) / (2.0 * s) + (1.0 - s) / (2.0 * s * s) * v2
    dP = -1.5 / s + v2 / (2.0 * s * s)
    dG = 1.5 / (s * s) - v2 / s ** 3 + v2 / (2.0 * s * s)
    return P * (dP * G + dG) * (1.0 - s) / 6.0


def bkw_grid(N: int, R: float, t: float):
    """BKW solution at time t (s = K(t)) on the grid, N^3 reals."""
    h, X, Y, Z = grid(N, R)
    return bkw_f(K(t), X * X + Y * Y + Z * Z)


def maxwellian(N, R, rho, u, T):
    h, X, Y, Z = grid(N, R)
    v2 = (X - u[0]) ** 2 + (Y - u[1]) ** 2 + (Z - u[2]) ** 2
    return rho * (2.0 * np.pi * T) ** -1.5 * np.exp(-v2 / (2.0 * T))


def mass(f, N, R):
    h = 2.0 * R / N
    return float(np.sum(f) * h ** 3)


def bkw_bump_batch(S: int, N: int, R: float, seed: int, t0_range=(5.5, 8.0),
                   amp_max=0.05, width=0.5):
    """S solves: BKW at a seeded t0 ~ U[t0_range] plus a Gaussian bump of
    amplitude U[0, amp_max] * mass, centre U[-1,1]^3, width `width`; mass
    renormalised to 1.  Returns (F0 [S, N^3], t0 [S], amp [S])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h, X, Y, Z = grid(N, R)
    t0 = rng.uniform(*t0_range, size=S)
    amp = rng.uniform(0.0, amp_max, size=S)
    ctr = rng.uniform(-1.0, 1.0, size=(S, 3))
    out = np.empty((S, N ** 3))
    for s in range(S):
        f = bkw_f(K(t0[s]), X * X + Y * Y + Z * Z)
        m = np.sum(f) * h ** 3
        v2c = (X - ctr[s, 0]) ** 2 + (Y - ctr[s, 1]) ** 2 + (Z - ctr[s, 2]) ** 2
        bump = np.exp(-v2c / (2.0 * width * width)) * (2.0 * np.pi * width * width) ** -1.5
        f = f + amp[s] * m * bump
        out[s] = f / (np.sum(f) * h ** 3)
    return out, t0, amp


def maxwellian_mixture_batch(S: int, N: int, R: float, seed: int, kmin=1, kmax=3,
                             u_range=2.0, T_range=(0.5, 1.5)):
    """S solves: mixtures of kmin..kmax isotropic Maxwellians with Dirichlet(1)
    weights, drifts U[-u_range, u_range]^3, temperatures U[T_range]; mass 1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.empty((S, N ** 3))
    for s in range(S):
        k = int(rng.integers(kmin, kmax + 1))
        w = rng.dirichlet(np.ones(k)) if k > 1 else np.ones(1)
        f = np.zeros(N ** 3)
        for j in range(k):
            u = rng.uniform(-u_range, u_range, size=3)
            T = rng.uniform(*T_range)
            f += maxwellian(N, R, w[j], u, T)
        out[s] = f / mass(f, N, R)
    return out


def two_maxwellians(N: int, R: float, seed: int):
    """Mixture of two isotropic Maxwellians, mass split 0.5/0.5, drifts
    U[-2,2]^3, temperatures U[0.5,1.5]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    f = np.zeros(N ** 3)
    for _ in range(2):
        u = rng.uniform(-2.0, 2.0, size=3)
        T = rng.uniform(0.5, 1.5)
        f += maxwellian(N, R, 0.5, u, T)
    return f
