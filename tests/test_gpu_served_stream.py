"""The served mixed stream at its own sizes: the stream's first 24 requests
(seed 4: streamline and FTLE requests on its 8 resident datasets, ABC or
double-gyre fields of edge 64-512, 200-2000 RK4 steps; streamline requests
reply with a 960x540 ray-traced image, the pars_service reply) submitted
together to the two-lane service, against the same requests run one at a
time through the plain single-request C ABI (seeds + trace + index + colour +
ray tracer, or flow map + FTLE).

Bar: every reply is bit-identical to the plain path's — images byte for byte,
FTLE fields bit for bit, the same particle-steps — although the service traces
streamline requests as blocks of shared batches and advects FTLE requests in
the continuous engine's horizon launches, admitted while others run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIDTH, HEIGHT = 960, 540


def _stream(count):
    from pars_gb300 import workloads as W
    from pars_gb300.requests import encode_settings
    f32 = np.float32
    ds, reqs = W.served_stream_config(seed=4, requests=count)
    out = []
    for r in reqs:
        d = ds[r["dataset"]]
        step = 0.01 if d["kind"] == "abc" else 0.05
        iterations = r["steps"] + (2 if r["kind"] == "streamlines" else 1)
        extent = np.array([2 * np.pi] * 3 if d["kind"] == "abc" else [2.0, 1.0, 1.0])
        camera = (float(extent[0] / 2), float(extent[1] / 2), float(-1.6 * extent.max()))
        radius = float(f32(0.1) * f32(extent[0] / (d["edge"] - 1)))
        message = {"mode": r["kind"], "dataset_filepath": d["name"], "seed_generation_stride": [r["stride"]] * 3,
                   "seed_generation_iterations": iterations, "particle_tracing_integrator": "runge_kutta_4",
                   "particle_tracing_step_size": step, "color_generation_mode": "hsv_constant_s",
                   "color_generation_free_parameter": 0.75}
        if r["kind"] == "streamlines":
            message.update({"raytracing_camera_position": list(camera), "raytracing_camera_forward": [0.0, 0.0, 1.0],
                            "raytracing_camera_up": [0.0, 1.0, 0.0], "raytracing_image_size": [WIDTH, HEIGHT],
                            "raytracing_streamline_radius": radius, "raytracing_iterations": 1})
        out.append({"kind": r["kind"], "dataset": r["dataset"], "stride": r["stride"], "iterations": iterations,
                    "step": step, "camera": camera, "radius": radius, "message": encode_settings(message)})
    return ds, out


def _plain(ctx, field, spec):
    """One request through the plain single-request C ABI; returns (reply, steps)."""
    from pars_gb300 import native
    f32 = np.float32
    xyz, offset, size, spacing = field
    edge = xyz.shape[0]
    h = ctx.upload_field_device(xyz.data_ptr(), (edge,) * 3, offset, size, spacing)
    try:
        if spec["kind"] == "streamlines":
            seeds = ctx.seed_generate(offset, size, (spacing * f32(spec["stride"])).astype(f32), spec["iterations"])
            summary = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, spec["step"])
            ctx.curves_index()
            ctx.curves_color("hsv_constant_s", 0.75)
            ctx.ray_tracer_set_image_size(WIDTH, HEIGHT)
            ctx.ray_tracer_set_camera(spec["camera"], (0.0, 0.0, 1.0), (0.0, 1.0, 0.0))
            ctx.ray_tracer_clear_volume()
            ctx.ray_tracer_set_integral_curves(spec["radius"])
            ctx.ray_tracer_trace(1)
            return ctx.ray_tracer_serialize(), summary["steps"]
        fm, steps = ctx.flow_map_generate(h, spec["iterations"], float(f32(1.0) / f32(spec["stride"])), native.RUNGE_KUTTA_4,
                                          native.STAGES_RESAMPLED, spec["step"])
        t = float(f32(spec["step"]) * f32(spec["iterations"]))
        shape = tuple(ctx.field_info(fm)["shape"])
        out = ctx.ftle_generate(fm, t, native.FTLE_REGULAR, shape=shape)
        ctx.release_field(fm)
        return out, steps
    finally:
        ctx.release_field(h)


def test_served_stream_replies_equal_the_plain_path(ctx):
    import torch
    from pars_gb300 import native, workloads as W
    ds, specs = _stream(24)
    fields = []
    for d in ds:
        gen = W.abc_device if d["kind"] == "abc" else W.gyre_snapshot_device
        fields.append(gen(torch, d["edge"]))
    torch.cuda.synchronize()
    svc = native.Service(0, budget_bytes=96 << 30, lanes=2, max_batch=64)
    try:
        for d, (xyz, offset, size, spacing) in zip(ds, fields):
            svc.add_dataset_device(d["name"], xyz.data_ptr(), (d["edge"],) * 3, offset, size, spacing)
        tickets = [svc.submit(s["message"]) for s in specs]
        served = []
        for t, s in zip(tickets, specs):
            assert svc.wait(t) == 2
            info = svc.info(t)
            assert info.status == 0, info.status
            reply = svc.image(t) if s["kind"] == "streamlines" else svc.ftle(t)
            served.append((reply, info.steps))
            svc.release(t)
    finally:
        svc.close()
    kinds = {s["kind"] for s in specs}
    assert kinds == {"streamlines", "ftle"}
    for s, (reply, steps) in zip(specs, served):
        expected, expected_steps = _plain(ctx, fields[s["dataset"]], s)
        assert steps == expected_steps, (s["kind"], s["dataset"], steps, expected_steps)
        if s["kind"] == "streamlines":
            assert reply.shape == expected.shape and np.array_equal(reply, expected), ("image", s["dataset"], s["stride"])
        else:
            assert np.array_equal(reply, expected, equal_nan=True), ("ftle", s["dataset"], s["stride"])
    print(f"\n{len(specs)} requests ({sum(s['kind'] == 'ftle' for s in specs)} FTLE) on datasets of edge "
          f"{sorted(d['edge'] for d in ds)}: every reply equals the plain path's")
