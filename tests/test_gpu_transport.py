"""pars_service's wire protocol end to end: a ZMTP 3.0 PAIR peer (what the
reference's clients use) sends `settings` messages to the service's
transport and receives `image` messages, byte-identical to the images the
service gives the same requests through the C ABI; a request without an
image (FTLE) is answered with an empty image; a ZMTP 3.1 PING is answered
with a PONG; a message split over several frames is one request."""
import threading

import numpy as np
import pytest

from test_render_cpu import decode_image
from zmtp_peer import Peer, command

pytestmark = pytest.mark.gpu


def _messages():
    from pars_gb300.requests import encode_settings
    base = {"particle_tracing_integrator": "runge_kutta_4", "color_generation_mode": "hsv_constant_s",
            "color_generation_free_parameter": 0.75, "dataset_filepath": "abc28", "particle_tracing_step_size": 0.01}
    image = {"raytracing_camera_position": [3.1, 3.1, -9.0], "raytracing_camera_forward": [0.0, 0.0, 1.0],
             "raytracing_camera_up": [0.0, 1.0, 0.0], "raytracing_image_size": [96, 64], "raytracing_streamline_radius": 0.02,
             "raytracing_iterations": 1}
    return [encode_settings(dict(base, mode="streamlines", seed_generation_stride=[3] * 3, seed_generation_iterations=202, **image)),
            encode_settings(dict(base, mode="ftle", seed_generation_stride=[2] * 3, seed_generation_iterations=101)),
            encode_settings(dict(base, mode="streamlines", seed_generation_stride=[4] * 3, seed_generation_iterations=402, **image))]


def test_zmtp_pair_peer_gets_the_services_images():
    from pars_gb300 import native, workloads as W
    svc = native.Service(0, budget_bytes=8 << 30, lanes=1, max_batch=8)
    svc.add_dataset("abc28", W.abc_field(28))
    messages = _messages()
    expected = []
    for m in messages:
        t = svc.submit(m)
        assert svc.wait(t) == 2
        img = svc.image(t)
        expected.append(None if img is None else img.tobytes())
        svc.release(t)
    listener, port = native.transport_listen("127.0.0.1", 0)
    served = {}
    server = threading.Thread(target=lambda: served.setdefault("n", svc.serve(listener)))
    server.start()
    peer = Peer(port, version=(3, 1))
    peer.sock.sendall(command(b"PING", b"\x00\x0a" + b"ctx"))
    flags, body = peer.read_frame()
    assert flags & 0x04 and body == b"\x04PONG" + b"ctx"
    replies = []
    for k, m in enumerate(messages):
        peer.send(m, parts=1 + k)
        replies.append(peer.receive())
    peer.close()
    server.join(120)
    native.transport_close(listener)
    assert served["n"] == len(messages)
    for reply, want in zip(replies, expected):
        size, data = decode_image(reply)
        if want is None:
            assert size in ([], [0, 0]) and data == b""
        else:
            assert size == [96, 64] and data == want
    svc.close()
