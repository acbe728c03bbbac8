"""The service's transport without a GPU: the listener binds and closes, and
the test's ZMTP peer frames messages as ZeroMQ RFC 23 writes them."""
import socket

from zmtp_peer import SIGNATURE, command, frame, greeting, parse_frame, ready


def test_listener_binds_a_free_port_and_closes():
    from pars_gb300 import native
    listener, port = native.transport_listen("127.0.0.1", 0)
    assert 0 < port < 65536
    probe = socket.create_connection(("127.0.0.1", port), timeout=5)   # the kernel accepts into the backlog
    probe.close()
    native.transport_close(listener)


def test_frames_follow_the_specification():
    assert len(greeting()) == 64 and greeting()[:10] == SIGNATURE and greeting()[10:12] == b"\x03\x00"
    assert frame(b"abc") == b"\x00\x03abc"
    assert frame(b"abc", more=True) == b"\x01\x03abc"
    long_body = bytes(300)
    assert frame(long_body)[:9] == b"\x02" + (300).to_bytes(8, "big")
    assert command(b"PING", b"\x00\x00") == b"\x04\x07\x04PING\x00\x00"
    assert ready().startswith(b"\x04") and b"\x0bSocket-Type\x00\x00\x00\x04PAIR" in ready()
    flags, body, rest = parse_frame(frame(long_body) + b"\x00\x00")
    assert flags == 0x02 and body == long_body and rest == b"\x00\x00"
