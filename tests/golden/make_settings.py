"""Writes tests/golden/settings.npz: `pars.settings` requests serialized by
the protobuf library itself, from a descriptor built with the field names,
numbers and types of the reference's pars/proto/settings.proto:5-27, and the
JSON forms protobuf's json_format writes and reads (the benchmark's settings
files, service.cpp:72-77).  The fixtures pin the library's settings decoder,
its JSON reader and pars_gb300.requests' encoder.
Needs the `protobuf` package (present in the development container):

    python tests/golden/make_settings.py
"""
import json
import os

import numpy as np
from google.protobuf import descriptor_pb2, descriptor_pool, json_format, message_factory

HERE = os.path.dirname(os.path.abspath(__file__))

SCHEMA = [  # name, number, type, repeated
    ("mode", 1, "string", False), ("volume_type", 2, "string", False), ("dataset_filepath", 3, "string", False),
    ("seed_generation_stride", 4, "int32", True), ("seed_generation_iterations", 5, "int32", False),
    ("particle_tracing_integrator", 6, "string", False), ("particle_tracing_step_size", 7, "float", False),
    ("particle_tracing_load_balance", 8, "bool", False), ("color_generation_mode", 9, "string", False),
    ("color_generation_free_parameter", 10, "float", False), ("raytracing_camera_position", 11, "float", True),
    ("raytracing_camera_forward", 12, "float", True), ("raytracing_camera_up", 13, "float", True),
    ("raytracing_image_size", 14, "int32", True), ("raytracing_streamline_radius", 15, "float", False),
    ("raytracing_iterations", 16, "int32", False),
]
TYPES = {"string": descriptor_pb2.FieldDescriptorProto.TYPE_STRING, "int32": descriptor_pb2.FieldDescriptorProto.TYPE_INT32,
         "float": descriptor_pb2.FieldDescriptorProto.TYPE_FLOAT, "bool": descriptor_pb2.FieldDescriptorProto.TYPE_BOOL}


def settings_class():
    f = descriptor_pb2.FileDescriptorProto(name="settings.proto", package="pars", syntax="proto3")
    m = f.message_type.add(name="settings")
    for name, number, kind, repeated in SCHEMA:
        field = m.field.add(name=name, number=number, type=TYPES[kind])
        field.label = (descriptor_pb2.FieldDescriptorProto.LABEL_REPEATED if repeated
                       else descriptor_pb2.FieldDescriptorProto.LABEL_OPTIONAL)
    pool = descriptor_pool.DescriptorPool()
    pool.Add(f)
    return message_factory.GetMessageClass(pool.FindMessageTypeByName("pars.settings"))


CASES = [
    {"mode": "streamlines", "volume_type": "retardation", "dataset_filepath": "abc64", "seed_generation_stride": [4, 4, 4],
     "seed_generation_iterations": 1002, "particle_tracing_integrator": "runge_kutta_4", "particle_tracing_step_size": 0.01,
     "particle_tracing_load_balance": True, "color_generation_mode": "hsv_constant_s", "color_generation_free_parameter": 0.75,
     "raytracing_camera_position": [0.5, -1.25, 3.0], "raytracing_camera_forward": [0.0, 0.0, 1.0],
     "raytracing_camera_up": [0.0, 1.0, 0.0], "raytracing_image_size": [1080, 1920],
     "raytracing_streamline_radius": 0.1, "raytracing_iterations": 1},
    {"mode": "ftle", "dataset_filepath": "/data/field.h5", "seed_generation_stride": [1, 1, 1],
     "seed_generation_iterations": 2000, "particle_tracing_integrator": "runge_kutta_4", "particle_tracing_step_size": 0.5},
    {"mode": "streamlines_reference", "dataset_filepath": "x", "seed_generation_stride": [2, -3, 70000],
     "seed_generation_iterations": -5, "particle_tracing_step_size": -0.25, "raytracing_iterations": 300},
]


JSON_VARIANTS = [
    '{"seedGenerationIterations": "1002", "particleTracingStepSize": "0.5", "mode": "ftle"}',
    '{"raytracing_camera_position": ["NaN", 1, "-Infinity"], "raytracingImageSize": [1920, "1080"], "volume_type": null}',
    '{"particleTracingLoadBalance": true, "colorGenerationFreeParameter": 7.5e-1, "dataset_filepath": "a\\u00e9b\\n"}',
    '{"seed_generation_stride": [], "raytracingIterations": 0, "particle_tracing_step_size": -0.0}',
]


def main():
    cls = settings_class()
    out = {}
    for k, case in enumerate(CASES):
        msg = cls()
        for name, value in case.items():
            if isinstance(value, list):
                getattr(msg, name).extend(value)
            else:
                setattr(msg, name, value)
        out[f"case{k}"] = np.frombuffer(msg.SerializeToString(), np.uint8)
        out[f"case{k}_json"] = np.array(json.dumps(case))
        out[f"case{k}_protojson"] = np.array(json_format.MessageToJson(msg))
    # JSON that json_format.Parse accepts, with the message it makes
    for k, text in enumerate(JSON_VARIANTS):
        out[f"variant{k}_json"] = np.array(text)
        out[f"variant{k}"] = np.frombuffer(json_format.Parse(text, cls()).SerializeToString(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "settings.npz"), **out)
    print("wrote settings.npz")


if __name__ == "__main__":
    main()
