"""Encoder for the reference's request message, proto3 `pars.settings`
(pars/proto/settings.proto:5-27), without a protobuf dependency.

Scalars equal to their proto3 default are omitted and repeated scalars are
packed, as a proto3 serializer writes them.
"""
import struct

# field name -> (number, kind)
FIELDS = {
    "mode": (1, "string"),
    "volume_type": (2, "string"),
    "dataset_filepath": (3, "string"),
    "seed_generation_stride": (4, "repeated_int32"),
    "seed_generation_iterations": (5, "int32"),
    "particle_tracing_integrator": (6, "string"),
    "particle_tracing_step_size": (7, "float"),
    "particle_tracing_load_balance": (8, "bool"),
    "color_generation_mode": (9, "string"),
    "color_generation_free_parameter": (10, "float"),
    "raytracing_camera_position": (11, "repeated_float"),
    "raytracing_camera_forward": (12, "repeated_float"),
    "raytracing_camera_up": (13, "repeated_float"),
    "raytracing_image_size": (14, "repeated_int32"),
    "raytracing_streamline_radius": (15, "float"),
    "raytracing_iterations": (16, "int32"),
}


def _varint(value):
    value &= (1 << 64) - 1   # negative int32 -> 10-byte two's complement varint
    out = bytearray()
    while True:
        byte = value & 0x7F
        value >>= 7
        if value:
            out.append(byte | 0x80)
        else:
            out.append(byte)
            return bytes(out)


def _key(number, wire_type):
    return _varint((number << 3) | wire_type)


def encode_settings(settings):
    """settings: dict with any of FIELDS -> bytes, fields in number order."""
    out = bytearray()
    for name, (number, kind) in sorted(FIELDS.items(), key=lambda x: x[1][0]):
        if name not in settings:
            continue
        value = settings[name]
        if kind == "string":
            if value:
                data = value.encode()
                out += _key(number, 2) + _varint(len(data)) + data
        elif kind in ("int32", "bool"):
            if value:
                out += _key(number, 0) + _varint(int(value))
        elif kind == "float":
            if value != 0.0:
                out += _key(number, 5) + struct.pack("<f", value)
        elif kind == "repeated_int32":
            if len(value):
                data = b"".join(_varint(int(v)) for v in value)
                out += _key(number, 2) + _varint(len(data)) + data
        elif kind == "repeated_float":
            if len(value):
                data = b"".join(struct.pack("<f", v) for v in value)
                out += _key(number, 2) + _varint(len(data)) + data
    return bytes(out)
