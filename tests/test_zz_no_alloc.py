"""The allocation-free FTLE entry point (pars_gpu_ftle_no_alloc).

It serves callers that may not allocate device memory — a plugin inside a host
application that owns the GPU's memory, or a path that cannot afford the
synchronisation of cudaMalloc/cudaFree.  The test calls it through the C ABI
twice in a row, on two different fields (so a stale flow map or step counter
left in the shared static scratch by the first call would show up in the
second), and checks each result against the context-based entry points
(pars_gpu_field_upload_device + pars_gpu_flow_map_generate +
pars_gpu_ftle_generate): FTLE within the relative 1e-4 used by the other FTLE
tests and the same step count.  (Frozen stages run the same flow-map kernel
on both paths; re-sampled RK4 runs the batched engine on the context path, so
there the two agree to rounding, not bit for bit.)  The
caller's input and output buffers are allocated by the caller (torch here),
as the entry point expects.  The file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, field_dev, field, out_dev, steps_dev, stream, iterations, step, time, stage_mode):
    shape = np.ascontiguousarray(field.dims, np.int32)
    return lib.pars_gpu_ftle_no_alloc(field_dev.data_ptr(), shape.ctypes.data, field.offset.ctypes.data, field.size.ctypes.data,
                                      field.spacing.ctypes.data, iterations, 2, stage_mode, step, time, 0,
                                      out_dev.data_ptr(), steps_dev.data_ptr() if steps_dev is not None else None, stream)


def _reference(ctx, field, iterations, step, time, stage_mode):
    h = ctx.upload_field(field)
    fm, steps = ctx.flow_map_generate(h, iterations, 1.0, 2, stage_mode, step)
    ftle = ctx.ftle_generate(fm, time, 0, shape=tuple(field.dims))
    ctx.release_field(fm)
    ctx.release_field(h)
    return ftle, steps


def test_no_alloc_ftle_matches_context_path_twice():
    import torch
    from pars_gb300 import native, workloads as W

    lib = native.library()
    ctx = native.Context(0)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream().cuda_stream
    iterations, step = 121, 0.01
    time = step * (iterations - 1)
    fields = [W.abc_field(40, noise_sigma=0.01, seed=0), W.abc_field(48, noise_sigma=0.02, seed=5)]
    for stage_mode, field in zip((native.STAGES_RESAMPLED, native.STAGES_FROZEN), fields):
        field_dev = torch.from_numpy(field.xyz).cuda()
        out_dev = torch.full(tuple(field.dims), float("nan"), dtype=torch.float32, device="cuda")
        steps_dev = torch.zeros(1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        status = _call(lib, field_dev, field, out_dev, steps_dev, stream, iterations, step, time, stage_mode)
        assert status == 0
        torch.cuda.synchronize()
        got = out_dev.cpu().numpy()
        expected, steps = _reference(ctx, field, iterations, step, time, stage_mode)
        assert int(steps_dev.item()) == steps
        floor = 1e-2 * np.abs(expected).max()
        big = np.abs(expected) >= floor
        assert (np.abs(got[big] - expected[big]) / np.abs(expected[big])).max() <= 1e-4
        assert np.abs(got[~big] - expected[~big]).max() <= 1e-4 * floor
    ctx.close()


def test_no_alloc_rejects_fields_beyond_its_static_scratch():
    import torch
    from pars_gb300 import native, workloads as W

    lib = native.library()
    field = W.abc_field(65)   # 65^3 > 64^3 voxels
    field_dev = torch.zeros(8, dtype=torch.float32, device="cuda")
    out_dev = torch.zeros(8, dtype=torch.float32, device="cuda")
    status = _call(lib, field_dev, field, out_dev, None, torch.cuda.current_stream().cuda_stream, 11, 0.01, 0.1,
                   native.STAGES_RESAMPLED)
    assert status == -6   # PARS_ERR_BUDGET


def test_no_alloc_rejects_overflowing_geometry_on_a_device():
    """Shapes whose voxel or seed products overflow, or that exceed the static
    scratch, return their status before any launch, with a device current."""
    import torch
    from test_cabi import NO_ALLOC_BAD_GEOMETRY
    from pars_gb300 import native

    lib = native.library()
    torch.cuda.set_device(0)
    dev = torch.zeros(16, dtype=torch.float32, device="cuda")
    for shape, size, spacing, status in NO_ALLOC_BAD_GEOMETRY:
        shape = np.array(shape, np.int32)
        offset = np.zeros(3, np.float32)
        size = np.array(size, np.float32)
        spacing = np.array(spacing, np.float32)
        got = lib.pars_gpu_ftle_no_alloc(dev.data_ptr(), shape.ctypes.data, offset.ctypes.data, size.ctypes.data,
                                         spacing.ctypes.data, 11, 2, 1, 0.01, 0.1, 0, dev.data_ptr(), None,
                                         torch.cuda.current_stream().cuda_stream)
        assert got == status, (shape, got)
    torch.cuda.synchronize()
    assert torch.isfinite(dev).all() and (dev == 0).all()
