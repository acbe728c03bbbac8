"""Host side of the ray tracer without a GPU: the `image` message encoder of
the C ABI, and the CPU restatement (oracle) checked against closed-form
shading of a single sphere and against its own frame accumulation."""
import numpy as np


def _varint(buf, i):
    v, shift = 0, 0
    while True:
        b = buf[i]
        i += 1
        v |= (b & 0x7F) << shift
        shift += 7
        if b < 0x80:
            return v, i


def decode_image(message):
    """Minimal proto3 reader for pars.image (size = 1 packed int32, data = 2)."""
    size, data, i = [], b"", 0
    while i < len(message):
        key, i = _varint(message, i)
        field, wire = key >> 3, key & 7
        assert wire == 2
        n, i = _varint(message, i)
        chunk = message[i:i + n]
        i += n
        if field == 1:
            j = 0
            while j < len(chunk):
                v, j = _varint(chunk, j)
                size.append(v)
        elif field == 2:
            data = bytes(chunk)
    return size, data


def test_image_message_round_trip():
    from pars_gb300 import native
    rgba = np.arange(300 * 200 * 4, dtype=np.uint32).astype(np.uint8).reshape(200, 300, 4)
    msg = native.image_encode(rgba)
    size, data = decode_image(msg)
    assert size == [300, 200]
    assert data == rgba.tobytes()
    # hand-built: 2 x 1 image -> 0a 02 02 01 12 08 <8 bytes>
    tiny = np.arange(8, dtype=np.uint8).reshape(1, 2, 4)
    assert native.image_encode(tiny) == bytes([0x0A, 0x02, 0x02, 0x01, 0x12, 0x08]) + bytes(range(8))


def _srgb_byte(c):
    s = np.where(c <= 0.0031308, 12.92 * c, 1.055 * np.power(c, 1 / 2.4) - 0.055)
    return np.clip(np.floor(s * 255 + 0.5), 0, 255)


def test_oracle_shades_a_sphere_as_the_closed_form(port):
    """A zero-length segment is a sphere; the pixel through its centre sees
    the normal pointing back at the camera.  Shading in FP64: base 0.8 c,
    ambient 1, per light base (n.L) (1, 1, 0.8) + 0.7 (n.h)^10 (1, 1, 0.8)."""
    c = np.array([0.2, 0.5, 0.9, 1.0], np.float32)
    v = np.array([[0.0, 0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0]], np.float32)
    cam = ((0.0, 0.0, 5.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    img, _ = port.render([(v, np.stack([c, c]), np.array([0], np.int32))], 1.0, cam, (5, 5))
    n = np.array([0.0, 0.0, 1.0])
    view = np.array([0.0, 0.0, 1.0])
    base = 0.8 * c[:3].astype(np.float64)
    out = base.copy()
    for d in ([1.0, 1.0, -0.5], [-1.0, 0.0, 0.5]):
        L = -np.array(d) / np.linalg.norm(d)
        ndl = n @ L
        if ndl > 0:
            out += base * ndl * np.array([1, 1, 0.8])
            hv = (L + view) / np.linalg.norm(L + view)
            if n @ hv > 0:
                out += 0.7 * (n @ hv) ** 10 * np.array([1, 1, 0.8])
    expected = _srgb_byte(np.clip(out, 0, 1))
    assert np.abs(img[2, 2, :3].astype(int) - expected).max() <= 1
    assert img[2, 2, 3] == 255
    assert (img[0, 0, :3] == 0).all()          # corner rays miss the sphere


def test_oracle_frames_accumulate(port):
    from pars_gb300 import workloads as W
    f = W.abc_field(16)
    seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(4)).astype(np.float32), 52)
    c = port.trace_single(f, seeds, 2, 0.01, "rgb", 0.5)
    batches = [(b["vertices"], b["colors"], b["indices"]) for b in c.batches]
    cam = ((3.0, 3.0, 12.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    both, _ = port.render(batches, 0.1, cam, (48, 32), frames=3)
    _, acc = port.render(batches, 0.1, cam, (48, 32), frames=1)
    split, _ = port.render(batches, 0.1, cam, (48, 32), frames=2, accum=acc, first_frame=1)
    assert np.array_equal(both, split)
