"""The GPU ray tracer (pars_gpu_ray_tracer_*, the counterpart of
pars::ray_tracer, pars/source/stages/ray_tracer.cpp) against its CPU
restatement in the oracle.

Bars:
* every image equals the oracle's byte for byte (the kernel and the
  restatement round the same FP32 operations in the same order, and the
  closest hit is the smallest (distance, segment) pair whatever the BVH's
  shape): curves with and without colours, with a volume, several batches,
  degenerate (zero-length) segments, a camera inside the volume, accumulated
  jittered frames, one segment, no segments;
* the context's device-resident curves render like the same curves given as
  host batches;
* frames accumulate across trace calls; a camera change starts again;
* re-tracing the context's curves after set_integral_curves is an error;
* the service renders the requests that carry an image size, each image equal
  to the oracle's render of the request's own curves and volume.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _curves(port, n=32, stride=4, iterations=202, color="hsv_constant_s", seed_field=None):
    from pars_gb300 import workloads as W
    f = seed_field or W.abc_field(n)
    st = (f.spacing * np.float32(stride)).astype(np.float32)
    seeds = port.seed_generate(f.offset, f.size, st, iterations)
    c = port.trace_single(f, seeds, 2, 0.01, color, 0.75)
    return f, [(b["vertices"], b["colors"], b["indices"]) for b in c.batches]


def _render_gpu(ctx, batches, radius, camera, size, frames=1, volume=None):
    ctx.ray_tracer_set_integral_curves_host(batches, radius)
    if volume is not None:
        ctx.ray_tracer_set_volume(*volume)
    else:
        ctx.ray_tracer_clear_volume()
    ctx.ray_tracer_set_image_size(*size)
    ctx.ray_tracer_set_camera(*camera)
    ctx.ray_tracer_trace(frames)
    return ctx.ray_tracer_serialize()


def _assert_same(got, expected):
    diff = np.any(got != expected, axis=-1)
    assert not diff.any(), f"{int(diff.sum())} of {diff.size} pixels differ; first at {np.argwhere(diff)[:3].tolist()}"


CAMERA = ((3.14, 3.14, 14.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
OBLIQUE = ((-4.0, 9.5, 11.0), (0.55, -0.45, -0.7), (0.1, 1.0, 0.0))


@pytest.mark.parametrize("case", ["colours", "white", "volume", "frames", "oblique", "inside"])
def test_images_equal_the_oracle(ctx, port, case):
    f, batches = _curves(port)
    vol = None
    camera, frames, radius, size = CAMERA, 1, 0.05, (96, 72)
    if case == "white":
        batches = [(v, None, i) for v, _, i in batches]
    if case in ("volume", "inside"):
        vol = ((np.linalg.norm(f.xyz, axis=-1) / 3.0).astype(np.float32), f.offset, f.spacing)
    if case == "frames":
        frames = 5
    if case == "oblique":
        camera, radius, size = OBLIQUE, 0.08, (101, 67)
    if case == "inside":
        camera = ((3.0, 3.2, 2.9), (0.3, -0.2, 1.0), (0.0, 1.0, 0.0))
    got = _render_gpu(ctx, batches, radius, camera, size, frames, vol)
    expected, _ = port.render(batches, radius, camera, size, frames=frames, volume=vol)
    assert got.shape == (size[1], size[0], 4)
    _assert_same(got, expected)
    assert (got[..., :3] > 0).any()


def test_edge_cases_equal_the_oracle(ctx, port):
    rng = np.random.default_rng(5)
    # several batches, zero-length segments, a batch without indices
    v1 = rng.uniform(0, 4, (40, 4)).astype(np.float32)
    v1[10] = v1[11]                       # degenerate segment 10
    c1 = rng.uniform(0, 1, (40, 4)).astype(np.float32)
    i1 = np.arange(0, 39, dtype=np.int32)
    v2 = rng.uniform(1, 3, (7, 4)).astype(np.float32)
    i2 = np.array([0, 2, 5], np.int32)
    c2 = rng.uniform(0, 1, (7, 4)).astype(np.float32)
    v3 = rng.uniform(0, 1, (3, 4)).astype(np.float32)
    batches = [(v1, c1, i1), (v3, np.ones_like(v3), np.zeros(0, np.int32)), (v2, c2, i2)]
    cam = ((2.0, 2.0, 9.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    for radius in (0.02, 0.3):
        got = _render_gpu(ctx, batches, radius, cam, (80, 60), 3)
        expected, _ = port.render(batches, radius, cam, (80, 60), frames=3)
        _assert_same(got, expected)
    # one segment; no segments (volume only, then nothing at all)
    one = [(v2[:2], c2[:2], np.array([0], np.int32))]
    _assert_same(_render_gpu(ctx, one, 0.5, cam, (40, 30)), port.render(one, 0.5, cam, (40, 30))[0])
    vol = (rng.uniform(0, 1, (9, 7, 8)).astype(np.float32), np.zeros(3, np.float32), np.full(3, 0.5, np.float32))
    _assert_same(_render_gpu(ctx, [], 0.5, cam, (40, 30), 2, vol), port.render([], 0.5, cam, (40, 30), frames=2, volume=vol)[0])
    empty = _render_gpu(ctx, [], 0.5, cam, (40, 30))
    assert (empty[..., :3] == 0).all() and (empty[..., 3] == 255).all()


def test_context_curves_render_like_host_curves(ctx, port):
    from pars_gb300 import native, workloads as W
    f = W.abc_field(40)
    seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(3)).astype(np.float32), 302)
    h = ctx.upload_field(f)
    s = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 0.01)
    ctx.curves_index()
    ctx.curves_color("hsl_constant_l", 0.6)
    ctx.ray_tracer_clear_volume()
    ctx.ray_tracer_set_image_size(120, 90)
    ctx.ray_tracer_set_camera(*OBLIQUE)
    ctx.ray_tracer_set_integral_curves(0.04)
    ctx.ray_tracer_trace(2)
    device = ctx.ray_tracer_serialize()
    host = ctx.curves(s["batches"], vertices=True, colors=True, indices=True)
    batches = [(b["vertices"], b["colors"], b["indices"]) for b in host]
    ctx.ray_tracer_set_integral_curves_host(batches, 0.04)
    ctx.ray_tracer_trace(2)
    _assert_same(ctx.ray_tracer_serialize(), device)
    expected, _ = port.render(batches, 0.04, OBLIQUE, (120, 90), frames=2)
    _assert_same(device, expected)
    # re-tracing replaces the curves the tracer was given
    ctx.ray_tracer_set_integral_curves(0.04)
    ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 0.01)
    with pytest.raises(native.ParsGpuError) as e:
        ctx.ray_tracer_trace(1)
    assert e.value.status == -9
    ctx.release_field(h)


def test_frames_accumulate_until_the_camera_changes(ctx, port):
    _, batches = _curves(port, n=24, stride=3)
    ctx.ray_tracer_set_integral_curves_host(batches, 0.06)
    ctx.ray_tracer_clear_volume()
    ctx.ray_tracer_set_image_size(64, 48)
    ctx.ray_tracer_set_camera(*CAMERA)
    ctx.ray_tracer_trace(1)
    ctx.ray_tracer_trace(3)
    assert ctx.ray_tracer_frames() == 4
    split = ctx.ray_tracer_serialize()
    ctx.ray_tracer_set_camera(*CAMERA)
    assert ctx.ray_tracer_frames() == 0
    ctx.ray_tracer_trace(4)
    _assert_same(split, ctx.ray_tracer_serialize())
    _assert_same(split, port.render(batches, 0.06, CAMERA, (64, 48), frames=4)[0])


def test_many_segments(ctx, port):
    """A scene of about a million capsules (deep BVH, many equal Morton codes
    where curves crowd) at a small resolution."""
    from pars_gb300 import workloads as W
    f, batches = _curves(port, n=64, stride=2, iterations=62, color="rgb")
    assert sum(len(i) for _, _, i in batches) > 900_000
    cam = ((3.1, 3.3, 10.5), (0.02, -0.03, -1.0), (0.0, 1.0, 0.0))
    got = _render_gpu(ctx, batches, 0.01, cam, (128, 96), 2)
    expected, _ = port.render(batches, 0.01, cam, (128, 96), frames=2)
    _assert_same(got, expected)


def test_scene_of_segment_pairs(ctx, port):
    """A scene above 2 M capsules, whose BVH leaves hold runs of two
    consecutive segments of a curve (split at curve breaks and at even start
    vertices): each segment's own box and capsule are still tested, so the
    image equals the oracle's."""
    f, batches = _curves(port, n=64, stride=2, iterations=102, color="rgb")
    assert sum(len(i) for _, _, i in batches) > 2_300_000
    cam = ((3.2, 3.0, 10.0), (-0.03, 0.02, -1.0), (0.0, 1.0, 0.0))
    got = _render_gpu(ctx, batches, 0.01, cam, (128, 96), 2)
    expected, _ = port.render(batches, 0.01, cam, (128, 96), frames=2)
    _assert_same(got, expected)


def test_service_renders_requests_that_ask_for_an_image(port):
    """Streamline requests with raytracing settings come back with the image
    ray_tracer::serialize would reply with (pipeline.cpp:264-337): each equals
    the oracle's render of the request's own curves (and volume); a "volume"
    request renders the volume alone; without an image size there is none."""
    from pars_gb300 import native, workloads as W
    from pars_gb300.requests import encode_settings
    f = W.abc_field(32)
    speed = np.linalg.norm(f.xyz, axis=-1)
    vol = (speed / speed.max()).astype(np.float32)
    svc = native.Service(0, budget_bytes=8 << 30, lanes=1, max_batch=8)
    try:
        svc.add_dataset("abc32", f)
        svc.add_volume("speed", vol, f.offset, f.spacing)
        view = {"raytracing_camera_position": list(OBLIQUE[0]), "raytracing_camera_forward": list(OBLIQUE[1]),
                "raytracing_camera_up": list(OBLIQUE[2]), "raytracing_image_size": [96, 64],
                "raytracing_streamline_radius": 0.06, "raytracing_iterations": 2}
        base = {"dataset_filepath": "abc32", "seed_generation_stride": [4, 4, 4], "seed_generation_iterations": 152,
                "particle_tracing_integrator": "runge_kutta_4", "particle_tracing_step_size": 0.01,
                "color_generation_mode": "hsv_constant_s", "color_generation_free_parameter": 0.75}
        cases = [dict(base, mode="streamlines", **view),
                 dict(base, mode="streamlines_reference volume", volume_type="speed", **dict(view, raytracing_iterations=1)),
                 dict(base, mode="volume", volume_type="speed", **view),
                 dict(base, mode="streamlines")]
        tickets = [svc.submit(encode_settings(r)) for r in cases]
        for t in tickets:
            assert svc.wait(t, timeout_ms=120_000) == 2
        for r, t in zip(cases, tickets):
            image = svc.image(t)
            if "raytracing_image_size" not in r:
                assert image is None and tuple(svc.info(t).image_size) == (0, 0)
                continue
            curves = svc.streamlines(t)
            if r["mode"] == "volume":
                assert curves == [] or all(len(i) == 0 for _, _, i in curves)
            volume = (vol, f.offset, f.spacing) if "volume" in r["mode"] else None
            expected, _ = port.render(curves, 0.06, OBLIQUE, (96, 64), frames=r["raytracing_iterations"], volume=volume)
            assert tuple(svc.info(t).image_size) == (96, 64)
            _assert_same(image, expected)
            msg = native.image_encode(image)
            assert len(msg) == 96 * 64 * 4 + 8      # size: 0a 02 60 40; data: 12 + 3-byte length
        for t in tickets:
            svc.release(t)
    finally:
        svc.close()
