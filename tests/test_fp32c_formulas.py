"""Two rewritings of the FP32C step, checked in FP32 arithmetic on the CPU
(numpy float32, the kernel's formulas restated):

- the slope limiter as slope_type times the minmod of q - qm, qp - q and
  (qp - qm) / (2 slope_type), the minmod taken as the median of
  min(a, b, c), 0 and max(a, b, c), against the reference's form
  (src/HydroBaseFunctor.h:421-455);
- HLLC's sampling as one choice between a side's own state and its star
  state, which needs SL > 0 => u* > 0 and SR <= 0 => u* <= 0 for the wave
  speeds and u* of riemann_hllc (src/HydroBaseFunctor.h:704-809).
"""
import numpy as np
import pytest

f32 = np.float32


def reference_slope(q, qp, qm, st):
    """slope_unsplit_hydro_2d_scalar, one direction, in float32."""
    dlft = f32(st) * (q - qm)
    drgt = f32(st) * (qp - q)
    dcen = f32(0.5) * (qp - qm)
    dsgn = np.where(dcen >= 0, f32(1), f32(-1))
    slop = np.minimum(np.abs(dlft), np.abs(drgt))
    dlim = np.where(dlft * drgt <= 0, f32(0), slop)
    return dsgn * np.minimum(dlim, np.abs(dcen))


def minmod_slope(q, qp, qm, st):
    """The kernel's slope2 (the slope divided by st), times st."""
    a = q - qm
    b = qp - q
    c = f32(0.5 / st) * (qp - qm)
    lo = np.minimum(np.minimum(a, b), c)
    hi = np.maximum(np.maximum(a, b), c)
    return f32(st) * np.maximum(lo, np.minimum(hi, f32(0)))


@pytest.mark.parametrize("st", [1.0, 2.0])
def test_minmod_limiter_equals_reference_form(st):
    rng = np.random.default_rng(11)
    n = 400_000
    # magnitudes where the reference's product test cannot underflow, plus
    # exact ties, zeros and sign changes
    mag = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), size=(3, n)))
    sgn = rng.choice([-1.0, 1.0], size=(3, n))
    q, qp, qm = (mag * sgn).astype(f32)
    k = n // 8
    qp[:k] = q[:k]                    # a flat side
    qm[k:2 * k] = q[k:2 * k]
    q[2 * k:3 * k] = 0
    qm[3 * k:4 * k] = qp[3 * k:4 * k]  # central difference 0
    got = minmod_slope(q, qp, qm, st)
    want = reference_slope(q, qp, qm, st)
    assert np.array_equal(got, want)   # values; the sign of a zero may differ


def hllc_speeds(rl, ul, pl, rr, ur, pr, gamma=f32(1.4), smallc2=f32(1e-20)):
    """Wave speeds and u* of riemann_hllc in float32 (the kernel's order)."""
    cl = np.sqrt(np.maximum(gamma * pl / rl, smallc2))
    cr = np.sqrt(np.maximum(gamma * pr / rr, smallc2))
    cmax = np.maximum(cl, cr)
    SL = np.minimum(ul, ur) - cmax
    SR = np.maximum(ul, ur) + cmax
    rcl = rl * (ul - SL)
    rcr = rr * (SR - ur)
    ustar = (rcr * ur + (rcl * ul + (pl - pr))) / (rcr + rcl)
    return SL, SR, ustar


def test_hllc_outer_waves_fix_the_sign_of_ustar():
    rng = np.random.default_rng(12)
    n = 1_000_000
    r = np.exp(rng.uniform(np.log(1e-4), np.log(1e2), size=(2, n))).astype(f32)
    p = np.exp(rng.uniform(np.log(1e-6), np.log(1e3), size=(2, n))).astype(f32)
    u = rng.uniform(-30, 30, size=(2, n)).astype(f32)
    SL, SR, ustar = hllc_speeds(r[0], u[0], p[0], r[1], u[1], p[1])
    sup_l, sup_r = SL > 0, SR <= 0
    assert sup_l.sum() > 1000 and sup_r.sum() > 1000  # both supersonic cases are sampled
    assert np.all(ustar[sup_l] > 0)
    assert np.all(ustar[sup_r] <= 0)
    # so the reference's four-way sampling (SL > 0: left state; else u* > 0
    # or SR > 0: a star state; else right state) takes a side's own state
    # exactly when the one-choice form does, on the side u* picks
    lft = ustar > 0
    S = np.where(lft, SL, SR)
    ref_own_state = (SL > 0) | ~(lft | (SR > 0))
    one_choice_own_state = (S > 0) == lft
    assert np.array_equal(ref_own_state, one_choice_own_state)
