"""Batched solves: each result is the same alone and in the mix (bit for
bit), equals the single-simulation FP32C path, respects its own t_end, and
admission follows the pool's free bytes."""
import numpy as np
import pytest

import _cases as C

import euler2d_kokkos_gb300 as e2d
from euler2d_kokkos_gb300 import workloads as W

pytestmark = pytest.mark.gpu

POOL = 2 << 30


def run_to_end(batch, max_iters=100000, chunk=16):
    n = 1
    it = 0
    while n > 0 and it < max_iters:
        n = batch.run(chunk)
        it += chunk
    return it


def small_mix(n=10, seed=7):
    return W.mixed_batch(n, seed=seed, max_side=192)


def test_batch_mix_equals_alone(gpu_lib):
    solves = small_mix()
    with e2d.Batch(pool_bytes=POOL) as b:
        ids = [b.admit(s.params, s.t_end, s.u0) for s in solves]
        run_to_end(b)
        mixed = [b.get_state(i) for i in ids]
        ends = [b.query(i) for i in ids]
    for s, got, (t, ns, active) in zip(solves, mixed, ends):
        assert not active and t == s.t_end
        with e2d.Batch(pool_bytes=POOL) as alone:
            i = alone.admit(s.params, s.t_end, s.u0)
            run_to_end(alone)
            assert np.array_equal(alone.get_state(i), got)
            assert alone.query(i)[1] == ns


def test_batch_equals_single_simulation_path(gpu_lib):
    s = small_mix(2, seed=3)[1]
    with e2d.Batch(pool_bytes=POOL) as b:
        i = b.admit(s.params, s.t_end, s.u0)
        run_to_end(b)
        got = b.get_state(i)
        t_b, n_b, _ = b.query(i)
    with e2d.HydroRun(s.params) as h:  # the same initial condition, built on the device
        t, ns = 0.0, 0
        while t < s.t_end:
            t, ns, tr = h.step_n(64, s.t_end, t, ns)
            if len(tr) == 0:
                break
        single = h.current(ns)
    assert (t, ns) == (t_b, n_b)
    assert np.array_equal(got, single)


def test_batch_tuning_does_not_change_results(gpu_lib):
    """Register variants, cp.async and TMA row staging (4, 6) and strip
    heights give the same bits; the 300-wide solve has interior strips, the
    ones TMA stages."""
    wide = e2d.make_params(300, 96, problem="implode", riemann="hllc", gamma0=1.4, cfl=0.8,
                           implode_shape=1, precision=e2d.PRECISION_FP32C)
    solves = small_mix(6, seed=11) + [W.Solve("implode", wide, None, 0.02)]
    outs = []
    for tuning in [(1, [16, 32, 64]), (0, [64, 16, 32]), (1, [8, 8, 8]), (4, [32, 32, 32]),
                   (6, [16, 64, 32])]:
        with e2d.Batch(pool_bytes=POOL) as b:
            b.set_tuning(*tuning)
            ids = [b.admit(s.params, s.t_end, s.u0) for s in solves]
            run_to_end(b)
            outs.append([b.get_state(i) for i in ids])
    for other in outs[1:]:
        for a, c in zip(outs[0], other):
            assert np.array_equal(a, c)


def test_batch_autotune_keeps_results(gpu_lib):
    solves = small_mix(6, seed=12)
    with e2d.Batch(pool_bytes=POOL) as b:
        ids = [b.admit(s.params, s.t_end, s.u0) for s in solves]
        b.autotune(2)
        run_to_end(b)
        tuned = [b.get_state(i) for i in ids]
    with e2d.Batch(pool_bytes=POOL) as b:
        ids = [b.admit(s.params, s.t_end, s.u0) for s in solves]
        run_to_end(b)
        plain = [b.get_state(i) for i in ids]
    for a, c in zip(tuned, plain):
        assert np.array_equal(a, c)


def test_batch_admission_by_free_bytes(gpu_lib):
    s = small_mix(1, seed=5)[0]
    need = e2d.Batch.instance_bytes(s.params)
    with e2d.Batch(pool_bytes=3 * need) as b:
        a = b.admit(s.params, s.t_end, s.u0)
        c = b.admit(s.params, s.t_end, s.u0)
        free, _ = b.free_bytes()
        with pytest.raises(e2d.E2DError) as ei:
            for _ in range(4):
                b.admit(s.params, s.t_end, s.u0)
        assert ei.value.status == 2  # E2D_ENOMEM
        b.release(a)
        d = b.admit(s.params, s.t_end, s.u0)  # room again
        run_to_end(b)
        assert np.array_equal(b.get_state(c), b.get_state(d))


def test_batch_fp32c_accuracy_vs_fp64(gpu_lib):
    """A batched FP32C solve against the FP64 path (bit-identical to the
    reference) at the same final time: relative L1 of density <= 1e-5."""
    s = small_mix(2, seed=9)[0]
    with e2d.Batch(pool_bytes=POOL) as b:
        i = b.admit(s.params, s.t_end, s.u0)
        run_to_end(b)
        got = b.get_state(i)
    p64 = s.params.copy()
    p64.precision = e2d.PRECISION_FP64
    with e2d.HydroRun(p64.init()) as h:
        t, ns = 0.0, 0
        while t < s.t_end:
            t, ns, tr = h.step_n(256, s.t_end, t, ns)
            if len(tr) == 0:
                break
        ref = h.current(ns)
    rho, rref = got[0, 2:-2, 2:-2], ref[0, 2:-2, 2:-2]
    assert np.abs(rho - rref).sum() / np.abs(rref).sum() < 1e-5


def test_run_batched_and_serve_complete_every_solve(gpu_lib):
    """The batched driver and the Poisson serving loop finish every request;
    a kept final state equals the same solve run alone."""
    from euler2d_kokkos_gb300 import serving

    solves = small_mix(8, seed=21)
    st, states = serving.run_batched(solves, pool_bytes=POOL, keep={0, 5})
    assert st.solves == len(solves) and st.cell_updates > 0
    for k in (0, 5):
        with e2d.Batch(pool_bytes=POOL) as alone:
            i = alone.admit(solves[k].params, solves[k].t_end, solves[k].u0)
            run_to_end(alone)
            assert np.array_equal(alone.get_state(i), states[k])
    sv = serving.serve(solves, rate_per_s=500.0, pool_bytes=POOL)
    assert sv.solves == len(solves) and len(sv.latencies) == len(solves)
    assert sv.cell_updates == st.cell_updates
    pct = sv.percentiles()
    assert 0 < pct["p50_s"] <= pct["p95_s"] <= pct["p99_s"] <= pct["max_s"]
    seq = serving.run_one_at_a_time(solves[:2])
    assert seq.solves == 2 and seq.cell_updates > 0


def test_serve_results_equal_each_solve_alone(gpu_lib):
    """Continuous batching keeps results: requests of uneven size arriving
    while others run (staggered Poisson arrivals; FP32C and FP64 requests
    mixed) end where each ends when run alone -- an FP32C request bit for
    bit as the same solve alone in a batch (and within 1e-5 relative L1 of
    density of the FP64 path), an FP64 request bit for bit as the single
    FP64 path, which is bit-identical to the reference."""
    from euler2d_kokkos_gb300 import serving

    solves = small_mix(6, seed=51) + W.mixed_batch(2, seed=52, max_side=160, precision=e2d.PRECISION_FP64)
    order = [0, 6, 1, 2, 7, 3, 4, 5]  # FP64 requests arrive between FP32C ones
    solves = [solves[k] for k in order]
    st = serving.serve(solves, rate_per_s=150.0, pool_bytes=POOL, keep=set(range(len(solves))))
    assert st.solves == len(solves) and not st.failed and not st.rejected
    assert st.peak_live >= 2  # requests overlapped on the GPU
    assert sorted(st.states) == list(range(len(solves)))
    for k, s in enumerate(solves):
        got = st.states[k]
        if s.params.precision == e2d.PRECISION_FP64 or k in st.escalated:
            p64 = s.params.copy()
            p64.precision = e2d.PRECISION_FP64
            with e2d.HydroRun(p64.init(), init_problem=s.u0 is None) as h:
                if s.u0 is not None:
                    h.set_state(0, s.u0)
                t, n = 0.0, 0
                while t < s.t_end:
                    t, n, _ = h.step_n(64, s.t_end, t, n, want_trace=False)
                assert np.array_equal(h.current(n), got), k
            continue
        with e2d.Batch(pool_bytes=POOL) as alone:
            i = alone.admit(s.params, s.t_end, s.u0)
            run_to_end(alone)
            assert np.array_equal(alone.get_state(i), got), k
        p64 = s.params.copy()
        p64.precision = e2d.PRECISION_FP64
        with e2d.HydroRun(p64.init(), init_problem=s.u0 is None) as h:
            if s.u0 is not None:
                h.set_state(0, s.u0)
            t, n = 0.0, 0
            while t < s.t_end:
                t, n, _ = h.step_n(256, s.t_end, t, n, want_trace=False)
            ref = h.current(n)
        rho, rref = got[0, 2:-2, 2:-2], ref[0, 2:-2, 2:-2]
        assert np.abs(rho - rref).sum() / np.abs(rref).sum() < 1e-5, k


def test_device_initial_conditions_equal_host_generators(gpu_lib):
    """The parametrised initial conditions built on the device at admission
    equal the host generators' arrays: bit for bit for blasts and
    four-quadrant problems, to rounding for shocked bubbles (whose energy the
    reference's initialiser sums in another order)."""
    solves = W.mixed_batch(9, seed=4, max_side=160, bubbles=True, precision=e2d.PRECISION_FP64)
    for s in solves:
        with e2d.HydroRun(s.params) as h:
            dev = h.get_state(0)
        host = s.host_state()
        if s.kind == "shocked_bubble":
            assert np.allclose(dev, host, rtol=1e-14, atol=0)
            assert np.array_equal(dev[0], host[0]) and np.array_equal(dev[2], host[2])
        else:
            assert np.array_equal(dev[:, 2:-2, 2:-2], host[:, 2:-2, 2:-2]), s.kind
    # a host array and the device initialiser give the same batched result
    s = W.mixed_batch(2, seed=4, max_side=128)[1]
    outs = []
    for u0 in (None, s.host_state()):
        with e2d.Batch(pool_bytes=POOL) as b:
            i = b.admit(s.params, s.t_end, u0)
            run_to_end(b)
            outs.append(b.get_state(i))
    assert np.array_equal(outs[0], outs[1])


def test_batch_fp64_instances_equal_single_fp64_path(gpu_lib):
    """FP64 instances of uneven size (with FP32C instances in the same
    batch) each end bit for bit where the single FP64 path (bit-identical to
    the reference) ends, after the same number of steps; the FP32C instances
    are unchanged by the FP64 ones sharing their batch."""
    fp64 = W.mixed_batch(4, seed=31, max_side=160, precision=e2d.PRECISION_FP64)
    fp32 = small_mix(3, seed=32)
    with e2d.Batch(pool_bytes=POOL) as b:
        ids64 = [b.admit(s.params, s.t_end) for s in fp64]
        ids32 = [b.admit(s.params, s.t_end) for s in fp32]
        run_to_end(b)
        got64 = [(b.get_state(i), b.query(i)) for i in ids64]
        got32 = [b.get_state(i) for i in ids32]
    for s, (u, (t, ns, active)) in zip(fp64, got64):
        assert not active and t == s.t_end
        with e2d.HydroRun(s.params) as h:
            tt, n = 0.0, 0
            while tt < s.t_end:
                tt, n, _ = h.step_n(64, s.t_end, tt, n, want_trace=False)
            assert (tt, n) == (t, ns)
            assert np.array_equal(h.current(n), u)
    for s, u in zip(fp32, got32):
        with e2d.Batch(pool_bytes=POOL) as alone:
            i = alone.admit(s.params, s.t_end)
            run_to_end(alone)
            assert np.array_equal(alone.get_state(i), u)


def test_batch_error_paths(gpu_lib):
    s = small_mix(1, seed=41)[0]
    with e2d.Batch(pool_bytes=POOL) as b:
        p_hll = s.params.copy()
        p_hll.riemannSolverType = e2d.RIEMANN["hll"]
        with pytest.raises(e2d.E2DError) as ei:
            b.admit(p_hll, s.t_end)  # the batch runs HLLC
        assert ei.value.status == 1
        for call in (lambda: b.query(3), lambda: b.get_state(3), lambda: b.release(3)):
            with pytest.raises(e2d.E2DError) as ei:
                call()  # slot 3 was never admitted
            assert ei.value.status == 1
        assert b.run(0) == 0  # nothing admitted: nothing active
        i = b.admit(s.params, s.t_end)
        assert b.run(0) == 1
        b.release(i)
        with pytest.raises(e2d.E2DError):
            b.query(i)
    with pytest.raises(e2d.E2DError) as ei:
        e2d.Batch(pool_bytes=1 << 20, max_instances=0)
    assert ei.value.status == 1


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
def test_batch_nonfinite_instance_is_isolated(gpu_lib, precision):
    """A solve whose state holds a NaN is stopped and reported (E2D_ENUMERIC
    from query); the other solves of the batch finish as they do alone."""
    prec = e2d.PRECISION_FP32C if precision == "fp32c" else e2d.PRECISION_FP64
    good, bad = W.mixed_batch(2, seed=51, max_side=128, precision=prec, device_init=False)
    u_bad = bad.u0.copy()
    u_bad[0, 10, 10] = np.nan
    with e2d.Batch(pool_bytes=POOL) as b:
        ig = b.admit(good.params, good.t_end, good.u0)
        ib = b.admit(bad.params, bad.t_end, u_bad)
        run_to_end(b)
        with pytest.raises(e2d.E2DError) as ei:
            b.query(ib)
        assert ei.value.status == 3  # E2D_ENUMERIC
        t, ns, active = b.query(ig)
        assert not active and t == good.t_end
        mixed = b.get_state(ig)
    with e2d.Batch(pool_bytes=POOL) as alone:
        i = alone.admit(good.params, good.t_end, good.u0)
        run_to_end(alone)
        assert np.array_equal(alone.get_state(i), mixed)


def test_serving_nonfinite_policies(gpu_lib):
    """A FP32C solve whose initial state holds a NaN: "drop" records it as
    failed; "fp64" admits it again as an FP64 instance, which stops too (the
    NaN is in its input), and then records it.  The other solve completes
    either way, and the stopped solve's updates are kept out of cell_updates."""
    from euler2d_kokkos_gb300 import serving

    good, bad = W.mixed_batch(2, seed=51, max_side=128, device_init=False)
    bad.u0 = bad.u0.copy()
    bad.u0[0, 10, 10] = np.nan
    with e2d.Batch(pool_bytes=POOL) as alone:
        alone.admit(good.params, good.t_end, good.u0)
        run_to_end(alone)
        good_updates = alone.stats()[0]
    for policy in ("drop", "fp64"):
        st, _ = serving.run_batched([good, bad], pool_bytes=POOL, autotune=False, on_nonfinite=policy)
        assert st.solves == 1 and st.failed == [1], policy
        assert st.escalated == ([1] if policy == "fp64" else []), policy
        assert st.wasted_cell_updates > 0 and st.cell_updates == good_updates, policy


BREAKDOWN_T_END, BREAKDOWN_STATES = C.BREAKDOWN_T_END, C.BREAKDOWN_STATES


def test_fp32_breakdown_is_rerun_in_fp64(gpu_lib):
    """run_batched stops the FP32C solve of the flow above with
    E2D_ENUMERIC, runs it again in FP64 and returns the FP64 path's state bit
    for bit."""
    from euler2d_kokkos_gb300 import serving

    p = e2d.make_params(416, 1824, problem="four_quadrant", riemann="hllc", gamma0=1.4, cfl=0.8,
                        bc=(2, 2, 2, 2), precision=e2d.PRECISION_FP32C)
    p.fq_split_x = p.fq_split_y = 0.5
    for q in range(4):
        for v in range(4):
            p.fq_state[q][v] = BREAKDOWN_STATES[q][v]
    s = W.Solve("four_quadrant", p, None, BREAKDOWN_T_END)
    st, states = serving.run_batched([s], pool_bytes=POOL, autotune=False, keep={0})
    assert st.escalated == [0] and st.failed == [] and st.solves == 1
    p64 = p.copy()
    p64.precision = e2d.PRECISION_FP64
    with e2d.HydroRun(p64.init()) as h:
        t, ns = 0.0, 0
        while t < BREAKDOWN_T_END:
            prev = ns
            t, ns, _ = h.step_n(256, BREAKDOWN_T_END, t, ns, want_trace=False)
            assert ns > prev
        assert np.array_equal(h.current(ns), states[0])
