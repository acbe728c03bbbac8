"""Batched advection in one persistent launch (pars_gpu_batch_advect).

Bars:
* pathlines on unsteady double-gyre fields (classical RK4 in space-time, time
  interpolation between slices, FP64 time of each step): end points within
  1e-3 cells of the FP64 oracle for every particle with the oracle's step
  count;
* a job's results do not depend on what else is in the batch: each job run
  alone equals the same job inside a mixed batch, bit for bit, for every
  launch shape the autotuner can pick;
* a re-sampled flow map computed through the batched engine equals the
  per-seed result of an explicit-seed batch job on the same lattice.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch_buffers():
    import torch
    return torch


def _job(native, field, seeds_dev, count, end_dev, steps_dev, max_steps, step, time_begin=0.0):
    j = native.BatchJob()
    j.field = field
    j.integrator = native.RUNGE_KUTTA_4
    j.stage_mode = native.STAGES_RESAMPLED
    j.max_steps = max_steps
    j.step_size = step
    j.time_begin = time_begin
    j.seeds = seeds_dev.data_ptr()
    j.seed_count = count
    j.end_positions = end_dev.data_ptr()
    j.end_steps = steps_dev.data_ptr() if steps_dev is not None else None
    return j


def _gyre_fields(ctx, specs):
    from pars_gb300 import workloads as W
    out = []
    for n, slices in specs:
        xyz, offset, spacing, t0, dt = W.double_gyre_slices(n, slices)
        h = ctx.upload_unsteady_field(xyz, offset, spacing, t0, dt)
        out.append((h, xyz, offset, spacing, t0, dt))
    return out


def _seeds(rng, count, n):
    p = np.zeros((count, 4), np.float32)
    p[:, 0] = rng.uniform(0.05, 1.95, count)
    p[:, 1] = rng.uniform(0.05, 0.95, count)
    p[:, 2] = rng.uniform(0.05, 0.95, count)
    return p


def test_pathlines_match_fp64_oracle(ctx, port):
    from pars_gb300 import native
    torch = _torch_buffers()
    rng = np.random.default_rng(3)
    fields = _gyre_fields(ctx, [(20, 9), (33, 17), (26, 12)])
    counts = [700, 2500, 300]
    step, max_steps = 0.02, 400
    jobs, keep = [], []
    for (h, *_), c in zip(fields, counts):
        s = _seeds(rng, c, 0)
        sd = torch.from_numpy(s).cuda()
        ed = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
        st = torch.zeros(c, dtype=torch.int32, device="cuda")
        jobs.append(_job(native, h, sd, c, ed, st, max_steps, step, time_begin=0.5))
        keep.append((s, sd, ed, st))
    got_steps = ctx.batch_advect(jobs)
    for (h, xyz, offset, spacing, t0, dt), (s, sd, ed, st), total in zip(fields, keep, got_steps):
        end = ed.cpu().numpy()[:, :3].astype(np.float64)
        steps = st.cpu().numpy()
        assert int(steps.sum()) == total
        e64, s64 = port.advect_unsteady_fp64(xyz, offset, spacing, t0, dt, s[:, :3], 0.5, step, max_steps)
        same = steps == s64
        assert same.mean() > 0.99
        cell = float(spacing.min())
        err = np.linalg.norm(end[same] - e64[same], axis=1) / cell
        assert err.max() <= 1e-3, err.max()
    for h, *_ in fields:
        ctx.release_field(h)


@pytest.mark.parametrize("variant", [-1, 0, 1, 2, 3])
def test_job_results_do_not_depend_on_the_batch(ctx, variant):
    from pars_gb300 import native, workloads as W
    torch = _torch_buffers()
    rng = np.random.default_rng(7)
    steady = W.abc_field(40, noise_sigma=0.01, seed=1)
    hs = ctx.upload_field(steady)
    unsteady = _gyre_fields(ctx, [(24, 10)])[0][0]
    specs = [(hs, 3000, lambda c: np.concatenate([rng.uniform(0.1, 6.1, (c, 3)), np.zeros((c, 1))], 1).astype(np.float32)),
             (unsteady, 1500, lambda c: _seeds(rng, c, 0)),
             (hs, 700, lambda c: np.concatenate([rng.uniform(0.1, 6.1, (c, 3)), np.zeros((c, 1))], 1).astype(np.float32))]
    made = []
    for h, c, gen in specs:
        s = gen(c)
        made.append((h, c, torch.from_numpy(s).cuda()))

    def run(indices):
        outs, jobs = [], []
        for i in indices:
            h, c, sd = made[i]
            ed = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
            st = torch.zeros(c, dtype=torch.int32, device="cuda")
            jobs.append(_job(native, h, sd, c, ed, st, 300, 0.01))
            outs.append((ed, st))
        steps = ctx.batch_advect(jobs, variant)
        return [(ed.cpu().numpy(), st.cpu().numpy(), n) for (ed, st), n in zip(outs, steps)]

    mixed = run([0, 1, 2])
    for k in range(3):
        alone = run([k])[0]
        assert np.array_equal(alone[0], mixed[k][0])
        assert np.array_equal(alone[1], mixed[k][1])
        assert alone[2] == mixed[k][2]
    ctx.release_field(hs)
    ctx.release_field(unsteady)


def test_resampled_flow_map_equals_explicit_seed_job(ctx, port):
    from pars_gb300 import native, workloads as W
    torch = _torch_buffers()
    f = W.abc_field(36, noise_sigma=0.01, seed=2)
    h = ctx.upload_field(f)
    fm, steps = ctx.flow_map_generate(h, 201, 1.0, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 0.01)
    flow = ctx.download_field(fm)
    seeds = port.seed_generate(f.offset, f.size, f.spacing, 201)
    s = np.ascontiguousarray(seeds["position"])
    sd = torch.from_numpy(s).cuda()
    ed = torch.zeros((len(s), 4), dtype=torch.float32, device="cuda")
    n = ctx.batch_advect([_job(native, h, sd, len(s), ed, None, 200, 0.01)])[0]
    assert n == steps
    assert np.array_equal(ed.cpu().numpy()[:, :3].reshape(flow.shape), flow)
    ctx.release_field(fm)
    ctx.release_field(h)


def test_frozen_jobs_match_the_oracle_bit_for_bit_in_a_mixed_batch(ctx, port):
    """Frozen-scheme jobs (the reference's arithmetic; a weighted-sum, a
    tableau and the two-step Adams-Bashforth scheme with its per-particle
    history) run as their own job class next to a re-sampled job: each frozen
    job's end points equal the oracle's frozen flow map (reference semantics)
    bit for bit, and the re-sampled job equals itself run alone."""
    from pars_gb300 import native, workloads as W
    torch = _torch_buffers()
    f = W.abc_field(24, noise_sigma=0.01, seed=5)
    h = ctx.upload_field(f)
    # the seed lattice of flow_map_generator at scale 1 (seed_generator.cpp:11)
    counts = [int(np.float32(f.size[i]) / np.float32(f.spacing[i])) for i in range(3)]
    n = int(np.prod(counts))
    max_steps, step = 120, 0.02

    def lattice_job(integrator, stage_mode):
        j = native.BatchJob()
        j.field = h
        j.integrator = integrator
        j.stage_mode = stage_mode
        j.max_steps = max_steps
        j.step_size = step
        j.seeds = None
        for i in range(3):
            j.lattice_offset[i] = float(f.offset[i])
            j.lattice_stride[i] = float(f.spacing[i])
            j.lattice_count[i] = counts[i]
        out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        j.end_positions = out.data_ptr()
        j.end_steps = None
        return j, out

    frozen = [native.RUNGE_KUTTA_4, native.INTEGRATORS["runge_kutta_dormand_prince_5"], native.INTEGRATORS["adams_bashforth_2"]]
    jobs, outs = [], []
    for k in frozen:
        j, o = lattice_job(k, native.STAGES_FROZEN)
        jobs.append(j); outs.append(o)
    rj, ro = lattice_job(native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED)
    steps = ctx.batch_advect(jobs + [rj])
    for k, o, s in zip(frozen, outs, steps):
        flow, ref_steps = port.flow_map(f, max_steps + 1, 1.0, k, step)
        assert s == ref_steps
        expected = flow[:counts[0], :counts[1], :counts[2]].reshape(-1, 3)
        assert np.array_equal(o.cpu().numpy()[:, :3], expected), k
    alone_j, alone_o = lattice_job(native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED)
    alone_steps = ctx.batch_advect([alone_j])
    assert alone_steps[0] == steps[-1]
    assert torch.equal(alone_o, ro)
    assert ctx.batch_tuned(2)[0] >= 0
    ctx.release_field(h)
