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


def shocked_bubble_state(nx, ny, p):
    """The shocked-bubble state of parameters p (the reference's
    [shocked_bubble] states: post-shock gas left of shock_loc, a bubble at
    rest, pre-shock gas at rest elsewhere)."""
    g = p.gamma0
    X, Y = _centres(nx, ny, p.xmin, p.ymin, p.xmax, p.ymax)
    U = np.zeros((4, ny + 4, nx + 4))
    post = X < p.shock_loc
    inb = np.sqrt((X - p.bubble_center_x) ** 2 + (Y - p.bubble_center_y) ** 2) < p.bubble_radius
    rho = np.where(post, p.postshock_density, np.where(inb, p.bubble_density, p.preshock_density))
    pr = np.where(post, p.postshock_pressure, np.where(inb, p.bubble_pressure, p.preshock_pressure))
    u = np.where(post, p.postshock_velocity, 0.0)
    U[0] = rho
    U[2] = rho * u
    U[1] = pr / (g - 1) + 0.5 * rho * u * u
    return U


class Solve:
    """One request: parameters, initial state, t_end.  u0 None: the initial
    condition is described by the parameters and built on the device."""

    def __init__(self, kind, params: HydroParams, u0, t_end: float):
        self.kind = kind
        self.params = params
        self.u0 = u0
        self.t_end = t_end

    @property
    def cells(self):
        return self.params.nx * self.params.ny

    def host_state(self) -> np.ndarray:
        """The initial state on the host (the generator's own arrays)."""
        return self.u0 if self.u0 is not None else _host_state(self)


def _host_state(s: "Solve") -> np.ndarray:
    p = s.params
    if s.kind == "blast":
        return blast_state(p.nx, p.ny, p.blast_center_x, p.blast_center_y, p.blast_radius,
                           p.blast_pressure_in, p.blast_pressure_out, rho=p.blast_density_in, gamma=p.gamma0)
    if s.kind == "four_quadrant":
        prim = [tuple(p.fq_state[q][v] for v in range(4)) for q in range(4)]
        return four_quadrant_state(p.nx, p.ny, prim, gamma=p.gamma0, split=(p.fq_split_x, p.fq_split_y))
    if s.kind == "shocked_bubble":
        return shocked_bubble_state(p.nx, p.ny, p)
    raise ValueError("no host generator for " + s.kind)


def _side(rng, lo=64, hi=1024):
    s = np.exp(rng.uniform(np.log(lo), np.log(hi)))
    return int(min(hi, max(lo, 16 * round(s / 16))))


def shock_states(mach, gamma=1.4):
    """Post-shock (rho, p, u) behind a normal shock of the given Mach number
    running into gas at rest with rho = 1, p = 1 (Rankine-Hugoniot)."""
    g = gamma
    M2 = mach * mach
    r2 = (g + 1) * M2 / ((g - 1) * M2 + 2)
    p2 = (2 * g * M2 - (g - 1)) / (g + 1)
    u2 = mach * np.sqrt(g) * (1 - 1 / r2)
    return r2, p2, u2


def mixed_batch(n: int, seed: int = 0, *, max_side: int = 1024, bubbles: bool = False,
                precision: int = PRECISION_FP32C, riemann: str = "hllc", device_init: bool = True):
    """n solves: blasts and four-quadrant problems (and shocked bubbles when
    `bubbles`), in a seeded order.  Each initial condition is carried by its
    parameters (the reference's [blast] and [shocked_bubble] states, the
    four-quadrant states and split) and built on the device at admission;
    device_init=False attaches the host-generated arrays instead."""
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
            p.blast_center_x, p.blast_center_y, p.blast_radius = float(cx), float(cy), float(radius)
            p.blast_density_in = p.blast_density_out = 1.0
            p.blast_pressure_in, p.blast_pressure_out = 0.1 * float(ratio), 0.1
            p.blast_total_energy_inside = 0.0
        elif kind == "four_quadrant":
            p = make_params(nx, ny, problem="four_quadrant", riemann=riemann, gamma0=1.4, cfl=0.8,
                            bc=(2, 2, 2, 2), precision=precision)
            p.fq_split_x = p.fq_split_y = 0.5
            for q in range(4):
                rho = rng.uniform(0.1, 2.0)
                pr = rng.uniform(0.02, 2.0)
                u = rng.uniform(0.0, 1.5) * rng.choice([-1.0, 1.0])
                v = rng.uniform(0.0, 1.5) * rng.choice([-1.0, 1.0])
                for i, val in enumerate((rho, pr, u, v)):
                    p.fq_state[q][i] = float(val)
        else:
            mach = rng.uniform(1.2, 3.0)
            ratio = rng.uniform(0.1, 10.0)
            p = make_params(nx, ny, problem="shocked_bubble", riemann=riemann, gamma0=1.4, cfl=0.8,
                            bc=(2, 2, 1, 1), precision=precision)
            r2, p2, u2 = shock_states(float(mach), p.gamma0)
            p.shock_loc = 0.15
            p.bubble_center_x, p.bubble_center_y, p.bubble_radius = 0.45, 0.5, 0.15
            p.bubble_density, p.bubble_pressure = float(ratio), 1.0
            p.preshock_density, p.preshock_pressure = 1.0, 1.0
            p.postshock_density, p.postshock_pressure, p.postshock_velocity = r2, p2, u2
        s = Solve(kind, p, None, t_end)
        if not device_init:
            s.u0 = _host_state(s)
        out.append(s)
    return out
