"""Polyline export (pars_gpu_export_vtk / pars_gpu_curves_export_vtk), the
counterpart of data_io::save_integral_curves (pa/source/stages/data_io.cpp:
142-196): the .vtp file read back holds exactly the points, colour bytes and
polylines that the reference's loop assembles, including a run that spans two
batches, empty runs, a last run without a termination vertex (its points kept,
no line) and colours the reference never writes (NaN -> 0)."""
import re

import numpy as np
import pytest

T = np.array([-2, -2, -2, 0], np.float32)


def read_vtp(path):
    data = open(path, "rb").read()
    head, raw = data.split(b"<AppendedData encoding=\"raw\">\n   _", 1)
    head = head.decode()
    arrays = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)"[^>]*offset="(\d+)"', head):
        kind, name, off = m.group(1), m.group(2), int(m.group(3))
        n = int(np.frombuffer(raw[off:off + 8], np.uint64)[0])
        dtype = {"UInt8": np.uint8, "Float32": np.float32, "Int64": np.int64}[kind]
        arrays[name] = np.frombuffer(raw[off + 8:off + 8 + n], dtype)
    counts = re.search(r'NumberOfPoints="(\d+)".*NumberOfLines="(\d+)"', head)
    return arrays, int(counts.group(1)), int(counts.group(2))


def expected(batches):
    """The reference's loop (data_io.cpp:160-181), restated."""
    points, colors, lines, line = [], [], [], []
    for v, c in batches:
        for j in range(len(v)):
            if not np.array_equal(v[j], T):
                line.append(len(points))
                points.append(v[j, :3])
                col = np.zeros(3) if c is None else c[j, :3].astype(np.float64) * 255.0
                colors.append([0 if not (x > 0) else (255 if x >= 255 else int(np.floor(x + 0.5))) for x in col])
            elif line:
                lines.append(line)
                line = []
    return np.array(points, np.float32).reshape(-1, 3), np.array(colors, np.uint8).reshape(-1, 3), lines


def test_export_matches_the_reference_loop(tmp_path):
    from pars_gb300 import native
    rng = np.random.default_rng(4)
    v1 = rng.uniform(0, 1, (12, 4)).astype(np.float32)
    v1[[3, 4, 8]] = T                        # a run of 3, an empty run, a run of 3, then an open run
    c1 = rng.uniform(-0.1, 1.1, (12, 4)).astype(np.float32)
    c1[5, 0] = np.nan
    v2 = rng.uniform(0, 1, (6, 4)).astype(np.float32)
    v2[[2, 5]] = T                           # ends the open run of batch 1, then a run of 2
    v3 = rng.uniform(0, 1, (4, 4)).astype(np.float32)   # no termination vertex: points without a line
    batches = [(v1, c1), (v2, None), (v3, rng.uniform(0, 1, (4, 4)).astype(np.float32))]
    path = str(tmp_path / "streamlines.vtp")
    native.export_vtk(path, batches)
    arrays, npoints, nlines = read_vtp(path)
    points, colors, lines = expected(batches)
    assert npoints == len(points) and nlines == len(lines) == 4
    assert np.array_equal(arrays["Points"].reshape(-1, 3), points)
    assert np.array_equal(arrays["Colors"].reshape(-1, 3), colors)
    ends = np.cumsum([len(l) for l in lines])
    assert np.array_equal(arrays["offsets"], ends)
    assert np.array_equal(arrays["connectivity"], np.concatenate(lines))


def test_empty_export(tmp_path):
    from pars_gb300 import native
    path = str(tmp_path / "empty.vtp")
    native.export_vtk(path, [])
    arrays, npoints, nlines = read_vtp(path)
    assert npoints == 0 and nlines == 0 and len(arrays["Points"]) == 0


@pytest.mark.gpu
def test_device_curves_export_like_host_curves(tmp_path, ctx, port):
    from pars_gb300 import native, workloads as W
    f = W.abc_field(24)
    seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(4)).astype(np.float32), 82)
    h = ctx.upload_field(f)
    s = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_FROZEN, 0.01)
    ctx.curves_index()
    ctx.curves_color("hsv_constant_s", 0.75)
    device = str(tmp_path / "device.vtp")
    ctx.curves_export_vtk(device)
    host = [(b["vertices"], b["colors"]) for b in ctx.curves(s["batches"], vertices=True, colors=True)]
    host_path = str(tmp_path / "host.vtp")
    native.export_vtk(host_path, host)
    assert open(device, "rb").read() == open(host_path, "rb").read()
    ctx.release_field(h)
