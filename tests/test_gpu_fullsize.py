"""Accuracy and parity at the sizes the benchmark numbers are quoted on.

* FTLE workload (256^3 ABC + N(0, 0.01) noise, seed 0; one seed per vertex,
  re-sampled RK4, h = 0.01, at most 500 steps): the batched engine's end
  points and step counts for 16,777,216 seeds, checked on a strided sample of
  about 100,000 seeds against the FP64 oracle of the same scheme on the same
  FP32 grid values: every seed with the oracle's step count within 1e-3 cell
  widths, the others (an exit one step earlier or later) ending next to the
  domain boundary.  Then the FTLE of an interior 48^3 window against the FP64
  FTLE of an FP64 flow map of the window and its one-voxel halo: relative
  error <= 1e-4 where |FTLE| >= 1 % of the window's maximum (absolute below),
  on voxels whose seven-point stencil took the oracle's step counts.
* Partitioned domain (512^3 Arnold-Beltrami + 8 Fourier modes, seed 1; 4x4x4
  blocks on one GPU; Gaussian-mixture seeds, seed 2; h = 0.005, 2000 steps):
  a 20,000-seed subsample (every 50th of the 1,000,000 seeds), the
  reference's frozen scheme, bit-exact per (block, round) batch against the
  oracle's round-by-round restatement of particle_tracer::trace with the
  block exchange (particle_tracer.cpp:253-409).
* Batched pathlines (32 unsteady double gyres, edge 32-256, 16-64 slices,
  2.9 M seeds, seed 3; RK4 in space-time, h = 0.01, 1000 steps): all 32 jobs
  in one launch, step totals consistent, six fields' strided seeds within
  1e-3 cells of the FP64 unsteady oracle.
"""
import numpy as np
import pytest

from test_gpu_parity import compare, gpu_curves

pytestmark = pytest.mark.gpu

N = 256
ITERATIONS = 501          # at most 500 steps
STEP = 0.01
T = 5.0


@pytest.fixture(scope="module")
def ftle_workload(ctx):
    """The 256^3 field, the engine's end points / step counts of every seed,
    and the flow map + FTLE through the context path (the bench's calls)."""
    import torch
    from pars_gb300 import native, workloads as W
    f = W.abc_field(N, noise_sigma=0.01, seed=0)
    h = ctx.upload_field(f)
    count = N ** 3
    end = torch.empty((count, 4), dtype=torch.float32, device="cuda")
    steps = torch.empty(count, dtype=torch.int32, device="cuda")
    j = native.BatchJob()
    j.field, j.integrator, j.stage_mode, j.max_steps, j.step_size = h, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, ITERATIONS - 1, STEP
    j.seeds, j.seed_count = None, 0
    for a in range(3):
        j.lattice_offset[a] = float(f.offset[a])
        j.lattice_stride[a] = float(f.spacing[a])
        j.lattice_count[a] = N
    j.end_positions, j.end_steps = end.data_ptr(), steps.data_ptr()
    total = ctx.batch_advect([j])[0]
    torch.cuda.synchronize()
    fm, fm_steps = ctx.flow_map_generate(h, ITERATIONS, 1.0, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, STEP)
    flow = ctx.download_field(fm)
    ftle = ctx.ftle_generate(fm, T, native.FTLE_REGULAR, shape=(N, N, N))
    out = {"field": f, "end": end[:, :3].cpu().numpy().reshape(N, N, N, 3), "steps": steps.cpu().numpy().reshape(N, N, N),
           "total": total, "flow": flow, "fm_steps": fm_steps, "ftle": ftle}
    ctx.release_field(fm)
    ctx.release_field(h)
    del end, steps
    torch.cuda.empty_cache()
    return out


def _lattice(f, idx):
    """FP32 seed positions of C-order lattice indices (offset + stride * index)."""
    ijk = np.stack(np.unravel_index(idx, tuple(f.dims)), -1).astype(np.float32)
    return (f.offset + ijk * f.spacing).astype(np.float32).astype(np.float64)


def test_engine_flow_map_is_the_context_flow_map(ftle_workload):
    w = ftle_workload
    assert w["total"] == w["fm_steps"] == int(w["steps"].sum(dtype=np.int64))
    assert np.array_equal(w["end"], w["flow"])


def test_ftle_workload_end_points_within_1e3_cells_of_fp64(ftle_workload, port):
    w = ftle_workload
    f = w["field"]
    idx = np.arange(0, N ** 3, 167)                       # 100,462 seeds over the whole grid
    end64, steps64, _ = port.advect_fp64(f, _lattice(f, idx), ITERATIONS - 1, integrator=2, mode=1, step=STEP)
    steps32 = w["steps"].reshape(-1)[idx]
    end32 = w["end"].reshape(-1, 3)[idx].astype(np.float64)
    cell = float(f.spacing[0])
    same = steps32 == steps64
    err = np.linalg.norm(end32[same] - end64[same], axis=1) / cell
    print(f"\n{same.sum()} of {len(idx)} seeds with the oracle's step count; end-point error (cells): "
          f"max {err.max():.3g}, p99.9 {np.percentile(err, 99.9):.3g}, median {np.median(err):.3g}")
    assert same.mean() > 0.999
    assert err.max() <= 1e-3, f"max end-point error {err.max()} cells"
    # a differing count is an exit decided one step apart: both end next to the domain boundary
    lo = f.offset.astype(np.float64)
    hi = lo + (f.dims - 1) * f.spacing.astype(np.float64)
    reach = 2 * 6.0 * STEP / cell                         # two steps at the field's largest speed, in cells
    for k in np.nonzero(~same)[0]:
        for p in (end32[k], end64[k]):
            gap = np.minimum(np.abs(p - lo), np.abs(p - hi)).min() / cell
            outside = np.any(p < lo) or np.any(p > hi)
            assert outside or gap <= reach, (idx[k], steps32[k], steps64[k], gap)


def test_ftle_workload_interior_window_within_1e4_of_fp64(ftle_workload, port):
    w = ftle_workload
    f = w["field"]
    a, b = 104, 152                                       # the 48^3 window; its halo is [103, 153)
    halo = np.arange(a - 1, b + 1)
    I, J, K = np.meshgrid(halo, halo, halo, indexing="ij")
    idx = np.ravel_multi_index((I.ravel(), J.ravel(), K.ravel()), (N, N, N))
    end64, steps64, _ = port.advect_fp64(f, _lattice(f, idx), ITERATIONS - 1, integrator=2, mode=1, step=STEP)
    m = len(halo)
    flow64 = end64.reshape(m, m, m, 3)
    # the FP64 FTLE of the FP64 flow map (central differences inside the halo
    # block are the full grid's central differences)
    ref = ftle_fp64_of_fp64_flow(flow64, f.spacing, T)[1:-1, 1:-1, 1:-1]
    got = w["ftle"][a:b, a:b, a:b].astype(np.float64)
    # voxels whose stencil took the oracle's step counts
    equal = (w["steps"][a - 1:b + 1, a - 1:b + 1, a - 1:b + 1] == steps64.reshape(m, m, m))
    stencil = (equal[1:-1, 1:-1, 1:-1] & equal[:-2, 1:-1, 1:-1] & equal[2:, 1:-1, 1:-1] & equal[1:-1, :-2, 1:-1]
               & equal[1:-1, 2:, 1:-1] & equal[1:-1, 1:-1, :-2] & equal[1:-1, 1:-1, 2:])
    assert stencil.mean() > 0.99
    floor = 1e-2 * np.abs(ref).max()
    big = (np.abs(ref) >= floor) & stencil
    small = (np.abs(ref) < floor) & stencil
    rel = np.abs(got[big] - ref[big]) / np.abs(ref[big])
    print(f"\nFTLE window: {stencil.sum()} of {stencil.size} voxels compared; relative error max {rel.max():.3g}, "
          f"median {np.median(rel):.3g}; FTLE range [{ref.min():.3g}, {ref.max():.3g}]")
    assert rel.max() <= 1e-4, rel.max()
    if small.any():
        assert np.abs(got[small] - ref[small]).max() <= 1e-4 * floor


def ftle_fp64_of_fp64_flow(flow64, spacing, time):
    """FTLE of an FP64 flow map in FP64: central differences (2h), C = J^T J,
    its largest eigenvalue (numpy's symmetric solver), 0.5 log(lambda) / |T|.
    One-sided differences at the block's faces (those voxels are the halo and
    are not compared)."""
    h = spacing.astype(np.float64)
    J = np.empty(flow64.shape[:3] + (3, 3))
    for axis in range(3):
        d = np.gradient(flow64, h[axis], axis=axis, edge_order=1)
        J[..., :, axis] = d
    C = np.einsum("...ki,...kj->...ij", J, J)
    lam = np.linalg.eigvalsh(C)[..., -1]
    return 0.5 * np.log(lam) / abs(time)


def test_partitioned_domain_512_frozen_matches_oracle(ctx, port):
    import torch
    from pars_gb300 import native, workloads as W
    n, ranks = 512, 64
    xyz, spacing = W.beltrami_fourier_device(torch, n, seed=1)
    info = native.partition(ranks, 0, (n, n, n))
    every, remaining = 50, 2002
    seeds_all, offsets_all = W.gaussian_mixture_seeds(1_000_000, n, spacing, info, remaining=remaining, seed=2)
    take = np.arange(0, len(seeds_all), every)
    seeds = seeds_all[take]
    owner = np.searchsorted(offsets_all, take, side="right") - 1
    offsets = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=ranks))]).astype(np.int64)
    d = ctx.domain_create_device(xyz.data_ptr(), (n, n, n), spacing, ranks)
    host = W.Field(xyz.cpu().numpy(), np.zeros(3, np.float32), spacing)
    del xyz
    torch.cuda.empty_cache()
    s = ctx.trace_domain(d, seeds, offsets, native.RUNGE_KUTTA_4, native.STAGES_FROZEN, 0.005)
    got = gpu_curves(ctx, s, "rgb")
    ctx.domain_release(d)
    expected = port.trace_multi(host, ranks, offsets, seeds, 2, 0.005, "rgb", 0.5)
    print(f"\n{len(seeds)} seeds, {s['rounds']} rounds, {s['batches']} batches, {s['steps']} steps")
    assert s["rounds"] > 1
    assert s["steps"] == expected.steps
    compare(got, expected.batches)


def test_pathline_workload_all_32_fields_in_one_launch(ctx, port):
    """The batched-pathline workload as the benchmark runs it: 32 unsteady
    double gyres (edge 32-256 log-uniform, 16-64 slices, 2.9 M seeds, seed 3)
    in one launch, RK4 in space-time, h = 0.01, 1000 steps.  Every job's step
    total equals the sum of its per-seed counts; on up to six of the fields of
    edge <= 96 (their slices copied to the host), 400 strided seeds each
    against the FP64 unsteady oracle: more than 99 % with the oracle's step
    count, and those within 1e-3 cells."""
    import torch
    from pars_gb300 import native, workloads as W
    specs = W.pathline_batch_config(seed=3)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    jobs, keep, handles = [], [], []
    for spec in specs:
        n, slices, c = spec["edge"], spec["slices"], spec["seeds"]
        xyz, offset, spacing, t0, dt = W.double_gyre_device(torch, n, slices)
        h = ctx.upload_unsteady_field_device(xyz.data_ptr(), (n, n, n), slices, offset,
                                             np.array([n, n, n], np.float32) * spacing, spacing, t0, dt)
        handles.append(h)
        host = xyz.cpu().numpy() if n <= 96 and sum(k[1] is not None for k in keep) < 6 else None
        del xyz
        seeds = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
        seeds[:, 0] = 0.05 + 1.9 * torch.rand(c, device="cuda", generator=gen)
        seeds[:, 1] = 0.05 + 0.9 * torch.rand(c, device="cuda", generator=gen)
        seeds[:, 2] = 0.05 + 0.9 * torch.rand(c, device="cuda", generator=gen)
        end = torch.empty((c, 4), dtype=torch.float32, device="cuda")
        steps = torch.empty(c, dtype=torch.int32, device="cuda")
        j = native.BatchJob()
        j.field, j.integrator, j.stage_mode, j.max_steps, j.step_size = h, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 1000, 0.01
        j.time_begin, j.seeds, j.seed_count = 0.0, seeds.data_ptr(), c
        j.end_positions, j.end_steps = end.data_ptr(), steps.data_ptr()
        jobs.append(j)
        keep.append((spec, host, offset, spacing, t0, dt, seeds, end, steps))
    torch.cuda.empty_cache()
    totals = ctx.batch_advect(jobs)
    first = [(end.clone(), steps.clone()) for *_, end, steps in keep]
    # a second run gives the same bits (inputs made on the caller's stream are
    # complete before the context reads them)
    assert ctx.batch_advect(jobs) == totals
    for (e, st), (*_, end, steps) in zip(first, keep):
        assert torch.equal(e, end) and torch.equal(st, steps)
    del first
    checked = 0
    for (spec, host, offset, spacing, t0, dt, seeds, end, steps), total in zip(keep, totals):
        assert int(steps.sum(dtype=torch.int64).item()) == total
        if host is None:
            continue
        idx = np.linspace(0, spec["seeds"] - 1, 400).astype(np.int64)
        s = seeds.cpu().numpy()[idx, :3]
        e64, s64 = port.advect_unsteady_fp64(host, offset, spacing, t0, dt, s, 0.0, 0.01, 1000)
        got_steps = steps.cpu().numpy()[idx]
        got = end.cpu().numpy()[idx, :3].astype(np.float64)
        same = got_steps == s64
        assert same.mean() > 0.99, (spec, same.mean())
        err = np.linalg.norm(got[same] - e64[same], axis=1) / float(spacing.min())
        assert err.max() <= 1e-3, (spec, err.max())
        checked += 1
    print(f"\n{len(specs)} fields, {sum(s['seeds'] for s in specs)} seeds, {sum(totals)} steps; {checked} fields checked against FP64")
    assert checked >= 4
    for h in handles:
        ctx.release_field(h)
