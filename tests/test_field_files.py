"""Field files (pars_gpu_raw_* / _scalar_load / _ftle_save / _field_load),
the counterpart of pa::data_io (pa/source/stages/data_io.cpp).

Bars: a rank's block is the partitioner's ghosted hyperslab of the dataset,
bit for bit, with the spacing divided by its maximum and offset / size as
data_io.cpp:108-114 compute them in FP32; FTLE blocks written by every rank
assemble the whole field (data_io.cpp:117-140); malformed files are rejected.
The vector-field load (device) is checked in the GPU test at the end."""
import os

import numpy as np
import pytest


def _expected_block(data, ranks, rank, spacing):
    from pars_gb300 import native
    p = native.partition(ranks, rank, data.shape[:3])
    o, g, b = p["offset"], p["ghosted"], p["block"]
    block = data[o[0]:o[0] + g[0], o[1]:o[1] + g[1], o[2]:o[2] + g[2]]
    sp = np.asarray(spacing, np.float32)
    sp = (sp / sp.max()).astype(np.float32)
    return block, (o.astype(np.float32) * sp).astype(np.float32), sp, (b.astype(np.float32) * sp).astype(np.float32), p


def test_scalar_blocks_are_the_ghosted_hyperslabs(tmp_path):
    from pars_gb300 import native
    rng = np.random.default_rng(2)
    data = rng.standard_normal((23, 17, 29)).astype(np.float32)
    path = str(tmp_path / "volume.praw")
    native.raw_write(path, data, (0.5, 2.0, 1.25))
    components, shape, spacing = native.raw_info(path)
    assert components == 1 and shape == (23, 17, 29) and np.array_equal(spacing, np.float32([0.5, 2.0, 1.25]))
    for ranks in (1, 2, 6, 8):
        for rank in range(ranks):
            values, offset, sp, size = native.scalar_load(path, ranks, rank)
            block, eo, esp, esize, _ = _expected_block(data, ranks, rank, (0.5, 2.0, 1.25))
            assert np.array_equal(values, block)
            assert np.array_equal(offset, eo) and np.array_equal(sp, esp) and np.array_equal(size, esize)


def test_ftle_blocks_assemble_the_field(tmp_path):
    from pars_gb300 import native
    rng = np.random.default_rng(3)
    domain = (20, 14, 9)
    full = rng.standard_normal(domain).astype(np.float32)
    path = str(tmp_path / "ftle_forward.praw")
    ranks = 4
    for rank in range(ranks):
        p = native.partition(ranks, rank, domain)
        o, b = p["offset"], p["block"]
        native.ftle_save(path, domain, o, full[o[0]:o[0] + b[0], o[1]:o[1] + b[1], o[2]:o[2] + b[2]], (1.0, 1.0, 1.0))
    values, _, _, _ = native.scalar_load(path)
    assert np.array_equal(values, full)
    with pytest.raises(native.ParsGpuError):
        native.ftle_save(path, (21, 14, 9), (0, 0, 0), full[:2, :2, :2])      # another domain


def test_malformed_files_are_rejected(tmp_path):
    from pars_gb300 import native
    missing = str(tmp_path / "missing.praw")
    with pytest.raises(native.ParsGpuError) as e:
        native.raw_info(missing)
    assert e.value.status == -5
    bad = tmp_path / "bad.praw"
    bad.write_bytes(b"NOTRAW01" + bytes(56))
    with pytest.raises(native.ParsGpuError) as e:
        native.raw_info(str(bad))
    assert e.value.status == -1
    short = str(tmp_path / "short.praw")
    native.raw_write(short, np.zeros((4, 4, 4), np.float32), (1, 1, 1))
    with open(short, "r+b") as f:
        f.truncate(64 + 100)
    with pytest.raises(native.ParsGpuError):
        native.scalar_load(short)
    vec = str(tmp_path / "vectors.praw")
    native.raw_write(vec, np.zeros((4, 4, 4, 3), np.float32), (1, 1, 1))
    with pytest.raises(native.ParsGpuError):
        native.scalar_load(vec)                                    # a vector file is not a scalar field


@pytest.mark.gpu
def test_vector_field_load_matches_the_upload(tmp_path, ctx):
    """A loaded block equals the same hyperslab uploaded directly (values,
    offset, size, spacing), and traces identically."""
    from pars_gb300 import native, workloads as W
    f = W.abc_field(40, noise_sigma=0.01, seed=9)
    path = str(tmp_path / "abc40.praw")
    native.raw_write(path, f.xyz, (0.3, 0.3, 0.6))
    for ranks, rank in ((1, 0), (8, 5)):
        h, part = ctx.field_load(path, ranks, rank)
        block, offset, sp, size, _ = _expected_block(f.xyz, ranks, rank, (0.3, 0.3, 0.6))
        info = ctx.field_info(h)
        assert tuple(info["shape"]) == block.shape[:3]
        assert np.array_equal(info["offset"], offset) and np.array_equal(info["spacing"], sp) and np.array_equal(info["size"], size)
        assert np.array_equal(ctx.download_field(h), block)
        ref = ctx.upload_field(W.Field(block, offset, sp, size))
        seeds = np.zeros(64, native.PARTICLE_DTYPE)
        rng = np.random.default_rng(rank)
        seeds["position"][:, :3] = offset + rng.uniform(0.1, 0.9, (64, 3)).astype(np.float32) * size
        seeds["remaining_iterations"] = 80
        seeds["vector_field_index"] = -1
        a = ctx.trace(h, seeds, native.RUNGE_KUTTA_4, native.STAGES_FROZEN, 0.01)
        va = ctx.curves(a["batches"])
        b = ctx.trace(ref, seeds, native.RUNGE_KUTTA_4, native.STAGES_FROZEN, 0.01)
        vb = ctx.curves(b["batches"])
        assert a["steps"] == b["steps"] and all(np.array_equal(x["vertices"], y["vertices"]) for x, y in zip(va, vb))
        ctx.release_field(h)
        ctx.release_field(ref)
