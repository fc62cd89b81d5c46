"""Seeded synthetic workloads of the batched and serving modes.

Mixed batches: grid sides drawn independently, log-uniform in [64, 1024] and
rounded to multiples of 16; half blasts (centre U[0.2, 0.8]^2, radius
U[0.05, 0.2], rho = 1, p = 0.1 outside, inside pressure ratio log-uniform in
[10, 1e4], reflecting walls), half four-quadrant Riemann problems (each
quadrant rho U[0.1, 2], p U[0.02, 2], |u|, |v| U[0, 1.5] with random signs,
split at (0.5, 0.5), absorbing walls); t_end U[0.05, 0.25], gamma 1.4, HLLC,
CFL 0.8.  Shocked bubbles (serving mix): a shock of Mach U[1.2, 3] from the
left into gas at rest (rho = 1, p = 1) holding a circular bubble of density
ratio U[0.1, 10], post-shock state from the Rankine-Hugoniot relations.
"""
from __future__ import annotations

import struct

import numpy as np

from . import HydroParams, PRECISION_FP32C, make_params


def f32(v: float) -> float:
    return struct.unpack("f", struct.pack("f", float(v)))[0]


def _centres(nx, ny, xmin=0.0, ymin=0.0, xmax=1.0, ymax=1.0):
    dx = (f32(xmax) - f32(xmin)) / nx
    dy = (f32(ymax) - f32(ymin)) / ny
    x = f32(xmin) + dx / 2 + (np.arange(nx + 4) - 2) * dx
    y = f32(ymin) + dy / 2 + (np.arange(ny + 4) - 2) * dy
    return np.meshgrid(x, y)


def four_quadrant_state(nx, ny, prim, gamma=1.4, split=(0.5, 0.5)):
    """prim: 4 x (rho, p, u, v) for quadrants 0 (x>=xt, y>=yt), 1 (x<xt,
    y>=yt), 2 (x<xt, y<yt), 3 (x>=xt, y<yt) -- the reference's numbering."""
    X, Y = _centres(nx, ny)
    region = np.where(X < split[0], np.where(Y < split[1], 2, 1), np.where(Y < split[1], 3, 0))
    U = np.zeros((4, ny + 4, nx + 4))
    for r in range(4):
        rho, p, u, v = prim[r]
        m = region == r
        U[0][m] = rho
        U[2][m] = rho * u
        U[3][m] = rho * v
        U[1][m] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return U


def blast_state(nx, ny, cx, cy, radius, p_in, p_out=0.1, rho=1.0, gamma=1.4):
    X, Y = _centres(nx, ny)
    inside = (X - cx) ** 2 + (Y - cy) ** 2 < radius * radius
    U = np.zeros((4, ny + 4, nx + 4))
    U[0] = rho
    U[1] = np.where(inside, p_in, p_out) / (gamma - 1.0)
    return U


def shocked_bubble_state(nx, ny, mach, density_ratio, gamma=1.4, shock_x=0.15, bubble=(0.45, 0.5, 0.15)):
    """Pre-shock gas rho = 1, p = 1 at rest; post-shock state behind a shock
    of the given Mach number (normal-shock relations); bubble of density
    density_ratio at the same pressure."""
    g = gamma
    r1, p1 = 1.0, 1.0
    c1 = np.sqrt(g * p1 / r1)
    M2 = mach * mach
    r2 = r1 * (g + 1) * M2 / ((g - 1) * M2 + 2)
    p2 = p1 * (2 * g * M2 - (g - 1)) / (g + 1)
    us = mach * c1
    u2 = us * (1 - r1 / r2)
    X, Y = _centres(nx, ny)
    U = np.zeros((4, ny + 4, nx + 4))
    post = X < shock_x
    inb = (X - bubble[0]) ** 2 + (Y - bubble[1]) ** 2 < bubble[2] ** 2
    rho = np.where(post, r2, np.where(inb, density_ratio * r1, r1))
    p = np.where(post, p2, p1)
    u = np.where(post, u2, 0.0)
    U[0] = rho
    U[2] = rho * u
    U[1] = p / (g - 1) + 0.5 * rho * u * u
    return U


class Solve:
    """One request: parameters, initial state, t_end."""

    def __init__(self, kind, params: HydroParams, u0: np.ndarray, t_end: float):
        self.kind = kind
        self.params = params
        self.u0 = u0
        self.t_end = t_end

    @property
    def cells(self):
        return self.params.nx * self.params.ny


def _side(rng, lo=64, hi=1024):
    s = np.exp(rng.uniform(np.log(lo), np.log(hi)))
    return int(min(hi, max(lo, 16 * round(s / 16))))


def mixed_batch(n: int, seed: int = 0, *, max_side: int = 1024, bubbles: bool = False,
                precision: int = PRECISION_FP32C, riemann: str = "hllc"):
    """n solves: blasts and four-quadrant problems (and shocked bubbles when
    `bubbles`), in a seeded order."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx, ny = _side(rng, 64, max_side), _side(rng, 64, max_side)
        t_end = float(rng.uniform(0.05, 0.25))
        kind = ("blast", "four_quadrant", "shocked_bubble")[k % 3] if bubbles else \
            ("blast", "four_quadrant")[k % 2]
        if kind == "blast":
            cx, cy = rng.uniform(0.2, 0.8, size=2)
            radius = rng.uniform(0.05, 0.2)
            ratio = np.exp(rng.uniform(np.log(10.0), np.log(1e4)))
            p = make_params(nx, ny, problem="blast", riemann=riemann, gamma0=1.4, cfl=0.8,
                            bc=(1, 1, 1, 1), precision=precision)
            u0 = blast_state(nx, ny, cx, cy, radius, 0.1 * ratio, gamma=p.gamma0)
        elif kind == "four_quadrant":
            prim = []
            for _ in range(4):
                rho = rng.uniform(0.1, 2.0)
                pr = rng.uniform(0.02, 2.0)
                u = rng.uniform(0.0, 1.5) * rng.choice([-1.0, 1.0])
                v = rng.uniform(0.0, 1.5) * rng.choice([-1.0, 1.0])
                prim.append((rho, pr, u, v))
            p = make_params(nx, ny, problem="four_quadrant", riemann=riemann, gamma0=1.4, cfl=0.8,
                            bc=(2, 2, 2, 2), precision=precision)
            u0 = four_quadrant_state(nx, ny, prim, gamma=p.gamma0)
        else:
            mach = rng.uniform(1.2, 3.0)
            ratio = rng.uniform(0.1, 10.0)
            p = make_params(nx, ny, problem="shocked_bubble", riemann=riemann, gamma0=1.4, cfl=0.8,
                            bc=(2, 2, 1, 1), precision=precision)
            u0 = shocked_bubble_state(nx, ny, mach, ratio, gamma=p.gamma0)
        out.append(Solve(kind, p, u0, t_end))
    return out
