"""The `settings` request message: the library's decoder and the Python
encoder against protobuf-serialized fixtures (tests/golden/make_settings.py)."""
import json

import numpy as np
import pytest

from conftest import golden


def cases():
    g = golden("settings.npz")
    return [(g[f"case{k}"].tobytes(), json.loads(str(g[f"case{k}_json"]))) for k in range(3)]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_encoder_matches_protobuf(k):
    from pars_gb300.requests import encode_settings
    data, case = cases()[k]
    assert encode_settings(case) == data


@pytest.mark.parametrize("k", [0, 1, 2])
def test_library_decodes_protobuf_bytes(k):
    from pars_gb300 import native
    data, case = cases()[k]
    s = native.decode_settings(data)
    assert s.mode.decode() == case.get("mode", "")
    assert s.dataset_filepath.decode() == case.get("dataset_filepath", "")
    assert s.particle_tracing_integrator.decode() == case.get("particle_tracing_integrator", "")
    assert list(s.seed_generation_stride) == (case.get("seed_generation_stride", []) + [0, 0, 0])[:3]
    assert s.seed_generation_iterations == case.get("seed_generation_iterations", 0)
    assert s.particle_tracing_step_size == np.float32(case.get("particle_tracing_step_size", 0.0))
    assert s.particle_tracing_load_balance == int(case.get("particle_tracing_load_balance", False))
    assert s.color_generation_free_parameter == np.float32(case.get("color_generation_free_parameter", 0.0))
    assert list(s.raytracing_image_size) == (case.get("raytracing_image_size", []) + [0, 0])[:2]
    assert s.raytracing_iterations == case.get("raytracing_iterations", 0)


def test_decoder_accepts_unpacked_repeated_and_unknown_fields():
    from pars_gb300 import native
    # field 4 unpacked (two varints), an unknown field 99 (varint), field 7 float
    msg = bytes([0x20, 0x03, 0x20, 0x05, 0x98, 0x06, 0x07]) + bytes([0x3D]) + np.float32(0.5).tobytes()
    s = native.decode_settings(msg)
    assert list(s.seed_generation_stride)[:2] == [3, 5]
    assert s.particle_tracing_step_size == np.float32(0.5)


@pytest.mark.parametrize("bad", [b"\x0a\x05ab", b"\x20", b"\x3d\x00\x00", b"\x0f"])
def test_decoder_rejects_malformed_messages(bad):
    from pars_gb300 import native
    with pytest.raises(native.ParsGpuError):
        native.decode_settings(bad)


def test_json_settings_make_the_protobuf_message():
    """pars_gpu_settings_from_json against protobuf's json_format: the JSON the
    runtime writes (lowerCamelCase), the snake_case files the benchmark
    generator writes, and the variants json_format.Parse accepts (numeric
    strings, NaN / -Infinity, null, escapes, -0.0) give the runtime's bytes."""
    from pars_gb300 import native
    g = golden("settings.npz")
    for k in range(3):
        expected = g[f"case{k}"].tobytes()
        assert native.settings_from_json(str(g[f"case{k}_protojson"])) == expected
        assert native.settings_from_json(str(g[f"case{k}_json"])) == expected
    for k in range(4):
        assert native.settings_from_json(str(g[f"variant{k}_json"])) == g[f"variant{k}"].tobytes(), k


def test_json_settings_errors():
    from pars_gb300 import native
    for bad in ('{"mode": 3}', '{"unknown_field": 1}', '{"seedGenerationIterations": 1.5}', '[1, 2]',
                '{"mode": "x",}', '{"raytracingImageSize": [1e20]}', '{"particleTracingStepSize": 1e39}', '{"mode": "x"} y'):
        with pytest.raises(native.ParsGpuError) as e:
            native.settings_from_json(bad)
        assert e.value.status == -1, bad
