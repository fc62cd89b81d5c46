"""The CPU oracle against golden fixtures produced by the reference itself
(tests/golden/make_golden.py runs the reference's own sources).  Bit-exact:
the oracle is a restatement of the reference's FP64 arithmetic in the same
operation order, built with -ffp-contract=off."""
import hashlib
import json
import os

import numpy as np
import pytest

import _cases as C
from oracle import pyoracle as po


def _params_for(text, riemann="hllc"):
    kw = C.oracle_kwargs(text)
    kw["riemann"] = riemann  # the reference runs riemann_hllc whatever the key says
    return po.make_params(**kw)


@pytest.mark.parametrize("name", sorted(C.run_cases().keys()))
def test_oracle_runs_bitwise(runs, name):
    text = str(runs[f"{name}__ini"])
    p = _params_for(text)
    nmax, tend = C.run_limits(text)
    nsteps = int(runs[f"{name}__nsteps"])
    u, dts, t, ns = po.run(p, runs[f"{name}__u0"], min(nmax, C.run_cases()[name]["nsteps"]), tend)
    assert ns == nsteps
    assert np.array_equal(dts, runs[f"{name}__dt"])
    assert t == float(runs[f"{name}__t"])
    assert np.array_equal(u, runs[f"{name}__u"])


def test_oracle_c1_implode_1000_steps(golden_dir):
    g = json.load(open(os.path.join(golden_dir, "c1.json")))
    p = _params_for(g["ini"])
    u0 = C.implode_diag_state(256, 256, C.f32(1.4))
    u, dts, t, ns = po.run(p, u0, 1000, C.f32(10.0))
    assert ns == g["nsteps"] == 1000
    assert [float(x).hex() for x in dts] == g["dt_hex"]
    assert hashlib.sha256(np.ascontiguousarray(u).tobytes()).hexdigest() == g["sha256_state"]


def _kat_params(kat, key):
    return _params_for(str(kat[key]))


def test_oracle_primitives(kat):
    p = _kat_params(kat, "ini_slope2")
    q, c = po.primitives(p, kat["prim_u"])
    assert np.array_equal(q, kat["prim_q"]) and np.array_equal(c, kat["prim_c"])


@pytest.mark.parametrize("st", [1, 2])
def test_oracle_slopes(kat, st):
    p = _kat_params(kat, f"ini_slope{st}")
    dqx, dqy = po.slopes(p, kat["slope_q5"])
    assert np.array_equal(dqx, kat[f"slope{st}_dqx"]) and np.array_equal(dqy, kat[f"slope{st}_dqy"])


@pytest.mark.parametrize("face", [0, 1, 2, 3])
def test_oracle_trace(kat, face):
    p = _kat_params(kat, "ini_slope2")
    out = po.trace(p, kat["trace_q"], kat["trace_dqx"], kat["trace_dqy"],
                   float(kat["trace_dtdx"]), float(kat["trace_dtdy"]), face)
    assert np.array_equal(out, kat[f"trace_face{face}"])


@pytest.mark.parametrize("solver", ["hllc", "approx"])
def test_oracle_riemann(kat, solver):
    p = _kat_params(kat, "ini_slope2")
    f = po.riemann(p, solver, kat["riemann_ql"], kat["riemann_qr"])
    assert np.array_equal(f, kat[f"riemann_{solver}"])


@pytest.mark.parametrize("tag", ["1111", "2222", "3333", "1231", "3123"])
def test_oracle_boundaries_and_dt(kat, tag):
    p = _kat_params(kat, f"bc{tag}_ini")
    u = po.make_boundaries(p, kat[f"bc{tag}_u0"])
    assert np.array_equal(u, kat[f"bc{tag}_u"])
    assert po.compute_dt(p, kat[f"bc{tag}_u0"]) == float(kat[f"bc{tag}_dt"])


def test_oracle_hll_properties():
    """HLL is not in the reference: check consistency (F(q,q) = physical flux),
    upwinding of supersonic states and Galilean mirror symmetry."""
    p = po.make_params(8, 8, gamma0=1.4)
    rng = np.random.default_rng(5)
    q = np.stack([np.exp(rng.normal(0, 1, 200)), np.exp(rng.normal(0, 1, 200)),
                  rng.normal(0, 1, 200), rng.normal(0, 1, 200)], axis=1)
    f = po.riemann(p, "hll", q, q)
    r, pr, u, v = q.T
    E = pr / (p.gamma0 - 1) + 0.5 * r * u * u + 0.5 * r * v * v
    phys = np.stack([r * u, (E + pr) * u, r * u * u + pr, r * u * v], axis=1)
    assert np.allclose(f, phys, rtol=1e-13, atol=1e-13)
    ql = q.copy(); qr = q[::-1].copy()
    ql[:, 2] = 20.0; qr[:, 2] = 20.0   # supersonic to the right: F = F(qL)
    fl = po.riemann(p, "hll", ql, ql)
    assert np.array_equal(po.riemann(p, "hll", ql, qr), fl)
    # mirror x -> -x: F(qL, qR) = -M F(M qR, M qL) with M flipping u
    ql = q; qr = q[::-1].copy()
    M = np.array([1, 1, -1, 1.0])
    a = po.riemann(p, "hll", ql, qr)
    b = po.riemann(p, "hll", qr * M, ql * M)
    assert np.allclose(a, -(b * M), rtol=1e-12, atol=1e-12)
