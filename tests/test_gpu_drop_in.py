"""The C++ drop-in (include/pa_gpu.hpp) driven the way pars::pipeline drives
the reference stages (tests/cpp/drop_in_pipeline.cpp), compiled with g++ and
checked against the oracle: bit-exact curves and indices, hsv colours within
2e-6, the ray tracer's `image` reply byte-identical to the CPU restatement's
render of the same curves, FTLE within 1e-4 of the FP64 evaluation of the
same flow map."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, assert_colors_equal

pytestmark = pytest.mark.gpu


def test_cpp_drop_in_pipeline_matches_oracle(port):
    from pars_gb300 import native, workloads as W
    f = W.abc_field(32)
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drop_in_pipeline")
        lib_dir = os.path.dirname(native.LIBRARY_PATH)
        subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "drop_in_pipeline.cpp"), "-L" + lib_dir, "-lpars_gpu",
                        "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
        field_path = os.path.join(tmp, "field.bin")
        f.xyz.tofile(field_path)
        iterations, step, stride = 302, 0.01, 2
        r = subprocess.run([exe, field_path, *map(str, f.dims), repr(float(f.spacing[0])), str(stride), str(iterations),
                            repr(step), tmp], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(stride)).astype(np.float32), iterations)
        expected = port.trace_single(f, seeds, 2, step, "hsv_constant_s", 0.75)
        meta = open(os.path.join(tmp, "curves.txt")).read().split()
        assert int(meta[0]) == len(expected.batches)
        for b, e in enumerate(expected.batches):
            v = np.fromfile(os.path.join(tmp, f"vertices_{b}.bin"), np.float32).reshape(-1, 4)
            i = np.fromfile(os.path.join(tmp, f"indices_{b}.bin"), np.int32)
            c = np.fromfile(os.path.join(tmp, f"colors_{b}.bin"), np.float32).reshape(-1, 4)
            assert np.array_equal(v, e["vertices"])
            assert np.array_equal(i, e["indices"])
            assert_colors_equal(c, e["colors"], 2e-6)
        from test_render_cpu import decode_image
        size, data = decode_image(open(os.path.join(tmp, "image.bin"), "rb").read())
        assert size == [64, 48]
        batches = []
        for b in range(len(expected.batches)):
            v = np.fromfile(os.path.join(tmp, f"vertices_{b}.bin"), np.float32).reshape(-1, 4)
            c = np.fromfile(os.path.join(tmp, f"colors_{b}.bin"), np.float32).reshape(-1, 4)
            i = np.fromfile(os.path.join(tmp, f"indices_{b}.bin"), np.int32)
            batches.append((v, c, i))
        image, _ = port.render(batches, 0.05, ((3.0, 3.2, 13.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0)), (64, 48), frames=2)
        assert data == image.tobytes()
        flow, _ = port.flow_map(f, iterations, 1.0, 2, step)
        ftle = np.fromfile(os.path.join(tmp, "ftle.bin"), np.float32).reshape(tuple(f.dims))
        ref = port.ftle_fp64(flow, f.spacing, step * (iterations - 1))
        floor = 1e-2 * np.abs(ref).max()
        big = np.abs(ref) >= floor
        assert (np.abs(ftle[big] - ref[big]) / np.abs(ref[big])).max() <= 1e-4
