"""The request service (pars_gpu_service_*): reference `settings` messages in,
curve buffers / FTLE fields out, with admission, batching and two lanes.

Bars:
* every result is the same alone and in the mix: a batch of mixed requests
  submitted together gives, request by request, exactly (bit for bit) what the
  same request gives when it is alone in the service;
* a streamline request with mode "streamlines_reference" (the reference's
  frozen-velocity scheme) returns the reference's buffers: bit-exact vertices,
  indices and rgb colours against the oracle;
* an FTLE request equals the context path (flow map + FTLE) on the same
  dataset, bit for bit.
"""
import numpy as np
import pytest

from conftest import assert_colors_equal

pytestmark = pytest.mark.gpu


def _requests():
    base = {"particle_tracing_integrator": "runge_kutta_4", "color_generation_free_parameter": 0.75}
    reqs = []
    for k, (stride, iters, color, step) in enumerate([(3, 302, "rgb", 0.01), (2, 152, "hsv_constant_s", 0.02),
                                                      (4, 502, "hsl_constant_l", 0.01), (5, 82, "rgb", 0.05),
                                                      (2, 202, "hsv_constant_v", 0.01), (6, 1002, "rgb", 0.01)]):
        reqs.append(dict(base, mode="streamlines", dataset_filepath="abc40" if k % 2 == 0 else "abc28",
                         seed_generation_stride=[stride] * 3, seed_generation_iterations=iters,
                         color_generation_mode=color, particle_tracing_step_size=step))
    for k, (stride, iters) in enumerate([(1, 101), (2, 201), (1, 61), (3, 301)]):
        reqs.append(dict(base, mode="ftle", dataset_filepath="abc40" if k % 2 else "abc28",
                         seed_generation_stride=[stride] * 3, seed_generation_iterations=iters,
                         particle_tracing_step_size=0.01))
    return reqs


def _result(svc, ticket, kind):
    return svc.streamlines(ticket) if kind == "streamlines" else svc.ftle(ticket)


def _same(a, b, kind):
    if kind == "ftle":
        return np.array_equal(a, b, equal_nan=True)
    return len(a) == len(b) and all(np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1], equal_nan=True)
                                    and np.array_equal(x[2], y[2]) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def service():
    from pars_gb300 import native, workloads as W
    svc = native.Service(0, budget_bytes=24 << 30, lanes=2, max_batch=16)
    svc.add_dataset("abc40", W.abc_field(40, noise_sigma=0.01, seed=4))
    svc.add_dataset("abc28", W.abc_field(28))
    yield svc
    svc.close()


def test_results_are_the_same_alone_and_in_the_mix(service):
    from pars_gb300.requests import encode_settings
    reqs = _requests()
    tickets = [service.submit(encode_settings(r)) for r in reqs]
    for t in tickets:
        assert service.wait(t) == 2
    mixed = [_result(service, t, "ftle" if "ftle" in r["mode"] else "streamlines") for t, r in zip(tickets, reqs)]
    infos = [service.info(t) for t in tickets]
    assert all(i.status == 0 for i in infos)
    assert all(i.latency_ms >= i.run_ms >= 0 for i in infos)
    for t in tickets:
        service.release(t)
    for r, m in zip(reqs, mixed):
        kind = "ftle" if "ftle" in r["mode"] else "streamlines"
        t = service.submit(encode_settings(r))
        assert service.wait(t) == 2
        alone = _result(service, t, kind)
        service.release(t)
        assert _same(alone, m, kind), r


def test_reference_mode_streamlines_match_the_oracle(service, port):
    from pars_gb300 import workloads as W
    from pars_gb300.requests import encode_settings
    f = W.abc_field(28)
    req = {"mode": "streamlines_reference", "dataset_filepath": "abc28", "seed_generation_stride": [3, 3, 3],
           "seed_generation_iterations": 202, "particle_tracing_integrator": "runge_kutta_4",
           "particle_tracing_step_size": 0.01, "color_generation_mode": "rgb"}
    t = service.submit(encode_settings(req))
    assert service.wait(t) == 2
    got = service.streamlines(t)
    service.release(t)
    seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(3)).astype(np.float32), 202)
    expected = port.trace_single(f, seeds, 2, 0.01, "rgb", 0.5)
    assert len(got) == len(expected.batches)
    for (v, c, i), e in zip(got, expected.batches):
        assert np.array_equal(v, e["vertices"])
        assert np.array_equal(i, e["indices"])
        assert_colors_equal(c, e["colors"])


@pytest.mark.parametrize("mode,ftle_mode,stages", [("ftle", 0, 1), ("ftle_fractional_anisotropy", 1, 1), ("ftle_reference", 0, 0)])
def test_ftle_request_equals_the_context_path(service, ctx, mode, ftle_mode, stages):
    """A mode containing "fractional_anisotropy" asks for the anisotropy map
    (ftle_map_generator.cpp:51-54) instead of the FTLE; one containing
    "reference" integrates with the reference's frozen scheme."""
    from pars_gb300 import native, workloads as W
    from pars_gb300.requests import encode_settings
    f = W.abc_field(40, noise_sigma=0.01, seed=4)
    req = {"mode": mode, "dataset_filepath": "abc40", "seed_generation_stride": [1, 1, 1],
           "seed_generation_iterations": 151, "particle_tracing_integrator": "runge_kutta_4",
           "particle_tracing_step_size": 0.01}
    t = service.submit(encode_settings(req))
    assert service.wait(t) == 2
    got = service.ftle(t)
    steps = service.info(t).steps
    service.release(t)
    h = ctx.upload_field(f)
    fm, s = ctx.flow_map_generate(h, 151, 1.0, native.RUNGE_KUTTA_4, stages, 0.01)
    expected = ctx.ftle_generate(fm, np.float32(0.01) * 151, ftle_mode, shape=tuple(f.dims))
    assert steps == s
    assert np.array_equal(got, expected)
    ctx.release_field(fm)
    ctx.release_field(h)


def test_unknown_dataset_and_oversized_requests_are_rejected(service):
    from pars_gb300 import native
    from pars_gb300.requests import encode_settings
    with pytest.raises(native.ParsGpuError) as e:
        service.submit(encode_settings({"mode": "ftle", "dataset_filepath": "missing", "seed_generation_stride": [1, 1, 1],
                                        "seed_generation_iterations": 11, "particle_tracing_integrator": "runge_kutta_4",
                                        "particle_tracing_step_size": 0.01}))
    assert e.value.status == -5
    with pytest.raises(native.ParsGpuError) as e:
        service.submit(encode_settings({"mode": "streamlines", "dataset_filepath": "abc40", "seed_generation_stride": [1, 1, 1],
                                        "seed_generation_iterations": 2_000_000, "particle_tracing_integrator": "runge_kutta_4",
                                        "particle_tracing_step_size": 0.01}))
    assert e.value.status == -6


def test_held_results_move_to_host_when_they_block_the_queue(service):
    """With a budget that holds only a few requests' results, requests that are
    submitted together and collected only at the end all finish (the held
    results move to host memory) and give the same buffers."""
    from pars_gb300 import native, workloads as W
    from pars_gb300.requests import encode_settings
    req = {"mode": "streamlines", "dataset_filepath": "abc40", "seed_generation_stride": [3, 3, 3],
           "seed_generation_iterations": 302, "particle_tracing_integrator": "runge_kutta_4",
           "particle_tracing_step_size": 0.01, "color_generation_mode": "rgb"}
    t = service.submit(encode_settings(req))
    assert service.wait(t) == 2
    expected = service.streamlines(t)
    service.release(t)
    small = native.Service(0, budget_bytes=200 << 20, lanes=2, max_batch=4)
    try:
        small.add_dataset("abc40", W.abc_field(40, noise_sigma=0.01, seed=4))
        tickets = [small.submit(encode_settings(req)) for _ in range(12)]
        for t in tickets:
            assert small.wait(t, timeout_ms=120_000) == 2
        for t in tickets:
            assert _same(small.streamlines(t), expected, "streamlines")
            small.release(t)
    finally:
        small.close()


def test_released_results_are_gone(service):
    from pars_gb300 import native
    from pars_gb300.requests import encode_settings
    t = service.submit(encode_settings({"mode": "ftle", "dataset_filepath": "abc28", "seed_generation_stride": [2, 2, 2],
                                        "seed_generation_iterations": 21, "particle_tracing_integrator": "runge_kutta_4",
                                        "particle_tracing_step_size": 0.01}))
    assert service.wait(t) == 2
    assert np.isfinite(service.ftle(t)).any()
    service.release(t)
    with pytest.raises(native.ParsGpuError) as e:
        service.ftle(t)
    assert e.value.status == -5


def test_shared_curve_buffers_outlive_released_neighbours(service):
    """Streamline requests of one batch share its curve buffers: releasing some
    of them, and running more batches meanwhile, leaves the others' results
    intact; once all are released the buffers serve later batches."""
    from pars_gb300.requests import encode_settings
    reqs = [r for r in _requests() if r["mode"] == "streamlines"][:4]
    tickets = [service.submit(encode_settings(r)) for r in reqs]
    for t in tickets:
        assert service.wait(t) == 2
    first = [service.streamlines(t) for t in tickets]
    for t in tickets[:3]:
        service.release(t)
    for r in reqs[:3]:                       # more batches while the fourth is held
        t = service.submit(encode_settings(r))
        assert service.wait(t) == 2
        service.release(t)
    assert _same(service.streamlines(tickets[3]), first[3], "streamlines")
    service.release(tickets[3])
    again = [service.submit(encode_settings(r)) for r in reqs]
    for t, expected in zip(again, first):
        assert service.wait(t) == 2
        assert _same(service.streamlines(t), expected, "streamlines")
        service.release(t)


def test_profile_reports_kernels_and_phases(service):
    from pars_gb300.requests import encode_settings
    service.profile_enable(True)
    reqs = _requests()
    tickets = [service.submit(encode_settings(r)) for r in reqs]
    for t in tickets:
        assert service.wait(t) == 2
        service.release(t)
    for name in ("trace_streamlines", "color_generate", "batch_advect_horizon", "ftle_fused",
                 "streamlines.trace", "streamlines.index_color", "ftle.advect"):
        ms, count = service.profile_get(name)
        assert count >= 1 and ms > 0.0, name
    requests, batches = service.profile_get("batches.streamlines")   # (requests held, batches)
    assert requests == 6.0 and 1 <= batches <= 6
    service.profile_enable(False)


def test_requests_with_the_other_integrators_equal_the_context_path(service, ctx):
    """A Dormand-Prince streamline request and an Adams-Bashforth-Moulton FTLE
    request (re-sampled stages) give what the context path gives, bit for bit,
    also when they share their batches with RK4 requests."""
    from pars_gb300 import native, workloads as W
    from pars_gb300.requests import encode_settings
    f = W.abc_field(28)
    stream = {"mode": "streamlines", "dataset_filepath": "abc28", "seed_generation_stride": [4, 4, 4],
              "seed_generation_iterations": 152, "particle_tracing_integrator": "runge_kutta_dormand_prince_5",
              "particle_tracing_step_size": 0.01, "color_generation_mode": "rgb"}
    ftle = {"mode": "ftle", "dataset_filepath": "abc28", "seed_generation_stride": [1, 1, 1],
            "seed_generation_iterations": 81, "particle_tracing_integrator": "adams_bashforth_moulton_2",
            "particle_tracing_step_size": 0.01}
    mix = [r for r in _requests()][:3] + [stream, ftle] + [r for r in _requests()][-2:]
    tickets = [service.submit(encode_settings(r)) for r in mix]
    for t in tickets:
        assert service.wait(t) == 2
    got_curves = service.streamlines(tickets[3])
    got_ftle = service.ftle(tickets[4])
    for t in tickets:
        service.release(t)
    h = ctx.upload_field(f)
    seeds = ctx.seed_generate(f.offset, f.size, (f.spacing * np.float32(4)).astype(np.float32), 152)
    s = ctx.trace(h, seeds, native.INTEGRATORS["runge_kutta_dormand_prince_5"], native.STAGES_RESAMPLED, 0.01)
    ctx.curves_index()
    ctx.curves_color("rgb")
    expected = [(b["vertices"], b["colors"], b["indices"]) for b in ctx.curves(s["batches"], True, True, True)]
    assert _same(got_curves, expected, "streamlines")
    fm, _ = ctx.flow_map_generate(h, 81, 1.0, native.INTEGRATORS["adams_bashforth_moulton_2"], native.STAGES_RESAMPLED, 0.01)
    expected_ftle = ctx.ftle_generate(fm, np.float32(0.01) * 81, 0, shape=tuple(f.dims))
    assert np.array_equal(got_ftle, expected_ftle, equal_nan=True)
    ctx.release_field(fm)
    ctx.release_field(h)


def test_requests_admitted_mid_flight_equal_their_results_alone(service):
    """Continuous admission: while a long FTLE request runs on one lane, the
    requests submitted after it has started are admitted by the other lane
    and run at the same time on the device; each gives bit for bit what it
    gives alone."""
    import time
    from pars_gb300.requests import encode_settings
    long_request = {"mode": "ftle", "dataset_filepath": "abc40", "seed_generation_stride": [1, 1, 1],
                    "seed_generation_iterations": 20001, "particle_tracing_integrator": "runge_kutta_4",
                    "particle_tracing_step_size": 0.001}
    reqs = _requests()
    t_long = service.submit(encode_settings(long_request))
    t0 = time.perf_counter()
    while service.wait(t_long, 0) == 0:      # queued: wait until it runs
        time.sleep(0.0005)
    submitted, tickets = [], []
    for r in reqs:
        submitted.append(time.perf_counter())
        tickets.append(service.submit(encode_settings(r)))
    for t in tickets + [t_long]:
        assert service.wait(t) == 2
    long_info = service.info(t_long)
    long_end = t0 + long_info.latency_ms / 1e3
    started = [s + service.info(t).queue_ms / 1e3 for s, t in zip(submitted, tickets)]
    assert sum(s < long_end for s in started) >= 1, "no request started while the long one ran"
    mixed = [_result(service, t, "ftle" if "ftle" in r["mode"] else "streamlines") for t, r in zip(tickets, reqs)]
    for t in tickets + [t_long]:
        service.release(t)
    for r, m in zip(reqs, mixed):
        kind = "ftle" if "ftle" in r["mode"] else "streamlines"
        t = service.submit(encode_settings(r))
        assert service.wait(t) == 2
        alone = _result(service, t, kind)
        service.release(t)
        assert _same(alone, m, kind), r


def test_ftle_requests_join_the_running_engine_and_leave_first():
    """One lane, continuous engine with 64-step horizons: FTLE requests
    submitted while a long FTLE request runs join its launch sequence and are
    handed out before it completes (with run-to-completion batches on one
    lane they would wait for it); each result equals the same request run as
    a one-launch batch (horizon 0), bit for bit."""
    import time
    from pars_gb300 import native, workloads as W
    from pars_gb300.requests import encode_settings
    svc = native.Service(0, budget_bytes=8 << 30, lanes=1, max_batch=16)
    try:
        svc.add_dataset("abc40", W.abc_field(40, noise_sigma=0.01, seed=4))
        svc.add_dataset("abc28", W.abc_field(28))
        svc.set_horizon(64)
        base = {"particle_tracing_integrator": "runge_kutta_4", "particle_tracing_step_size": 0.01}
        long_request = dict(base, mode="ftle", dataset_filepath="abc40", seed_generation_stride=[1, 1, 1],
                            seed_generation_iterations=20001, particle_tracing_step_size=0.001)
        short = [dict(base, mode="ftle", dataset_filepath="abc28", seed_generation_stride=[2, 2, 2],
                      seed_generation_iterations=201),
                 dict(base, mode="ftle_reference", dataset_filepath="abc28", seed_generation_stride=[1, 1, 1],
                      seed_generation_iterations=101),
                 dict(base, mode="ftle_fractional_anisotropy", dataset_filepath="abc40",
                      seed_generation_stride=[3, 3, 3], seed_generation_iterations=151),
                 dict(base, mode="ftle", dataset_filepath="abc28", seed_generation_stride=[2, 2, 2],
                      seed_generation_iterations=101, particle_tracing_integrator="runge_kutta_dormand_prince_5")]
        t_long = svc.submit(encode_settings(long_request))
        t_long_submitted = time.perf_counter()
        for _ in range(200000):
            if svc.wait(t_long, 0) != 0:
                break
            time.sleep(0.0005)
        submitted, tickets = [], []
        for r in short:
            submitted.append(time.perf_counter())
            tickets.append(svc.submit(encode_settings(r)))
        for t in tickets + [t_long]:
            assert svc.wait(t) == 2
        long_end = t_long_submitted + svc.info(t_long).latency_ms / 1e3
        ends = [s + svc.info(t).latency_ms / 1e3 for s, t in zip(submitted, tickets)]
        print(f"\nlong request done at {long_end - t_long_submitted:.3f} s; short ones at "
              + ", ".join(f"{e - t_long_submitted:.3f}" for e in ends))
        assert all(e < long_end for e in ends), "a request waited for the long one"
        joined = [svc.ftle(t) for t in tickets]
        long_result = svc.ftle(t_long)
        for t in tickets + [t_long]:
            svc.release(t)
        svc.set_horizon(0)
        for r, got in zip(short + [long_request], joined + [long_result]):
            t = svc.submit(encode_settings(r))
            assert svc.wait(t) == 2
            assert np.array_equal(svc.ftle(t), got, equal_nan=True), r["mode"]
            svc.release(t)
    finally:
        svc.close()
