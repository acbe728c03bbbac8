"""A ZMTP 3.0 PAIR peer in Python for the transport tests (test
infrastructure): the client side of ZeroMQ RFC 23 with the NULL mechanism —
what a ZeroMQ PAIR socket that connects to pars_service does on the wire."""
import socket
import struct

SIGNATURE = b"\xff" + b"\x00" * 8 + b"\x7f"


def greeting(version=(3, 0), as_server=False):
    return SIGNATURE + bytes(version) + b"NULL".ljust(20, b"\x00") + bytes([1 if as_server else 0]) + b"\x00" * 31


def frame(body, more=False, command=False):
    flags = (0x01 if more else 0) | (0x04 if command else 0)
    if len(body) <= 255:
        return bytes([flags, len(body)]) + body
    return bytes([flags | 0x02]) + struct.pack(">Q", len(body)) + body


def command(name, data=b""):
    return frame(bytes([len(name)]) + name + data, command=True)


def ready(socket_type=b"PAIR"):
    return command(b"READY", bytes([11]) + b"Socket-Type" + struct.pack(">I", len(socket_type)) + socket_type)


def parse_frame(buffer):
    """(flags, body, rest) of the first frame in `buffer`, or None if incomplete."""
    if len(buffer) < 2:
        return None
    flags = buffer[0]
    if flags & 0x02:
        if len(buffer) < 9:
            return None
        n, start = struct.unpack(">Q", buffer[1:9])[0], 9
    else:
        n, start = buffer[1], 2
    if len(buffer) < start + n:
        return None
    return flags, buffer[start:start + n], buffer[start + n:]


class Peer:
    def __init__(self, port, host="127.0.0.1", version=(3, 0), socket_type=b"PAIR", timeout=120.0):
        self.sock = socket.create_connection((host, port), timeout=timeout)
        self.buffer = b""
        self.sock.sendall(greeting(version))
        theirs = self._read_exact(64)
        assert theirs[:10] == SIGNATURE and theirs[10] == 3 and theirs[12:16] == b"NULL", theirs
        self.sock.sendall(ready(socket_type))
        flags, body = self.read_frame()
        assert flags & 0x04 and body[:6] == b"\x05READY", body
        self.server_ready = body

    def _read_exact(self, n):
        while len(self.buffer) < n:
            chunk = self.sock.recv(1 << 20)
            if not chunk:
                raise ConnectionError("peer closed")
            self.buffer += chunk
        out, self.buffer = self.buffer[:n], self.buffer[n:]
        return out

    def read_frame(self):
        while True:
            parsed = parse_frame(self.buffer)
            if parsed:
                flags, body, self.buffer = parsed
                return flags, body
            chunk = self.sock.recv(1 << 20)
            if not chunk:
                raise ConnectionError("peer closed")
            self.buffer += chunk

    def send(self, message, parts=1):
        """A message, split into `parts` frames."""
        step = max(1, -(-len(message) // parts))
        pieces = [message[i:i + step] for i in range(0, len(message), step)] or [b""]
        self.sock.sendall(b"".join(frame(p, more=k + 1 < len(pieces)) for k, p in enumerate(pieces)))

    def receive(self):
        out = b""
        while True:
            flags, body = self.read_frame()
            if flags & 0x04:
                continue
            out += body
            if not flags & 0x01:
                return out

    def close(self):
        self.sock.close()
