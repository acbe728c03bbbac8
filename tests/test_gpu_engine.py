"""Continuous batched advection (pars_gpu_engine_submit / pars_gpu_engine_advance).

The engine's horizon launches park every warp after a fixed number of steps
and resume it in the next launch, and jobs submitted between launches join
the running table.  Bar: every job's end positions, step counts and total
steps equal the one-launch engine's (pars_gpu_batch_advect) bit for bit,
whatever the horizon (fixed, or chosen by the engine for launches of about
2 ms: iterations 0) and whenever the job was submitted, for the three job
classes (re-sampled steady, re-sampled unsteady, frozen with the reference's
multistep history).
"""
import numpy as np
import pytest

from test_gpu_batch import _gyre_fields, _job, _seeds

pytestmark = pytest.mark.gpu


def _lattice_job(native, torch, f, h, integrator, stage_mode, max_steps, step):
    counts = [int(np.float32(f.size[i]) / np.float32(f.spacing[i])) for i in range(3)]
    n = int(np.prod(counts))
    j = native.BatchJob()
    j.field, j.integrator, j.stage_mode, j.max_steps, j.step_size = h, integrator, stage_mode, max_steps, step
    j.seeds = None
    for i in range(3):
        j.lattice_offset[i] = float(f.offset[i])
        j.lattice_stride[i] = float(f.spacing[i])
        j.lattice_count[i] = counts[i]
    end = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    steps = torch.zeros(n, dtype=torch.int32, device="cuda")
    j.end_positions, j.end_steps = end.data_ptr(), steps.data_ptr()
    return j, end, steps


def _workload(ctx):
    """Seven jobs over the three classes: (job factory, outputs) pairs, so that
    each run writes into fresh buffers."""
    import torch
    from pars_gb300 import native, workloads as W
    rng = np.random.default_rng(11)
    steady = W.abc_field(40, noise_sigma=0.01, seed=1)
    hs = ctx.upload_field(steady)
    small = W.abc_field(24, noise_sigma=0.01, seed=5)
    hsmall = ctx.upload_field(small)
    hu = _gyre_fields(ctx, [(24, 10)])[0][0]
    explicit = [(hs, np.concatenate([rng.uniform(0.1, 6.1, (3000, 3)), np.zeros((3000, 1))], 1).astype(np.float32)),
                (hu, _seeds(rng, 1500, 0)),
                (hs, np.concatenate([rng.uniform(0.1, 6.1, (700, 3)), np.zeros((700, 1))], 1).astype(np.float32))]
    explicit = [(h, torch.from_numpy(s).cuda()) for h, s in explicit]

    def make():
        jobs = []
        for h, sd in explicit:
            c = sd.shape[0]
            ed = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
            st = torch.zeros(c, dtype=torch.int32, device="cuda")
            jobs.append((_job(native, h, sd, c, ed, st, 300, 0.01), ed, st))
        for integrator in (native.RUNGE_KUTTA_4, native.INTEGRATORS["adams_bashforth_2"],
                           native.INTEGRATORS["runge_kutta_dormand_prince_5"]):
            jobs.append(_lattice_job(native, torch, small, hsmall, integrator, native.STAGES_FROZEN, 120, 0.02))
        jobs.append(_lattice_job(native, torch, steady, hs, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 250, 0.01))
        return jobs

    return make, (hs, hsmall, hu)


def _run_engine(ctx, jobs, iterations, first_wave):
    """Submits jobs[:first_wave], advances twice, submits the rest, then
    advances until every job is reported; returns {index: steps} and the
    number of launches."""
    tickets = {}
    for k in range(first_wave):
        tickets[ctx.engine_submit(jobs[k][0])] = k
    steps, advances, open_at_second_wave = {}, 0, None
    for _ in range(2):
        done, _left = ctx.engine_advance(iterations)
        advances += 1
        steps.update({tickets[t]: s for t, s in done})
    open_at_second_wave = _left
    for k in range(first_wave, len(jobs)):
        tickets[ctx.engine_submit(jobs[k][0])] = k
    for _ in range(200000):
        done, left = ctx.engine_advance(iterations)
        advances += 1
        steps.update({tickets[t]: s for t, s in done})
        if left == 0:
            break
    assert len(steps) == len(jobs)
    return steps, advances, open_at_second_wave


@pytest.mark.parametrize("iterations", [7, 64, 1000, 0])
def test_engine_horizons_equal_one_launch(ctx, iterations):
    make, handles = _workload(ctx)
    alone = []
    for j, ed, st in make():
        n = ctx.batch_advect([j])[0]
        alone.append((ed.cpu().numpy(), st.cpu().numpy(), n))
    jobs = make()
    steps, advances, open_mid = _run_engine(ctx, jobs, iterations, first_wave=3)
    print(f"\nhorizon {iterations}: {advances} advances; {open_mid} jobs open when the second wave was submitted")
    if 0 < iterations < 100:
        assert open_mid > 0          # the second wave joined a running table
        assert advances > 10
    for k, (j, ed, st) in enumerate(jobs):
        e, s, n = alone[k]
        assert steps[k] == n, k
        assert np.array_equal(st.cpu().numpy(), s), k
        assert np.array_equal(ed.cpu().numpy(), e), k
    for h in handles:
        ctx.release_field(h)


def test_engine_full_gpu_horizon_on_a_lattice(ctx):
    """Every resident warp parks (262,144 seeds on a 64^3 lattice, horizons of
    50 steps): the parked groups fill the buffers and are resumed exactly."""
    import torch
    from pars_gb300 import native, workloads as W
    f = W.abc_field(65, noise_sigma=0.01, seed=3)
    h = ctx.upload_field(f)
    j, ed, st = _lattice_job(native, torch, f, h, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 400, 0.01)
    n = ctx.batch_advect([j])[0]
    e, s = ed.cpu().numpy(), st.cpu().numpy()
    j2, ed2, st2 = _lattice_job(native, torch, f, h, native.RUNGE_KUTTA_4, native.STAGES_RESAMPLED, 400, 0.01)
    t = ctx.engine_submit(j2)
    total, advances = None, 0
    for _ in range(100000):
        done, left = ctx.engine_advance(50)
        advances += 1
        for ticket, steps in done:
            assert ticket == t
            total = steps
        if left == 0:
            break
    assert advances >= 8
    assert total == n
    assert np.array_equal(st2.cpu().numpy(), s)
    assert np.array_equal(ed2.cpu().numpy(), e)
    ctx.release_field(h)


def test_engine_edge_cases(ctx):
    import torch
    from pars_gb300 import native, workloads as W
    assert ctx.engine_advance(16) == ([], 0)
    with pytest.raises(native.ParsGpuError):
        ctx.engine_advance(-1)
    f = W.abc_field(16, noise_sigma=0.0, seed=0)
    h = ctx.upload_field(f)
    sd = torch.zeros((1, 4), dtype=torch.float32, device="cuda")
    ed = torch.zeros((1, 4), dtype=torch.float32, device="cuda")
    empty = _job(native, h, sd, 0, ed, None, 100, 0.01)
    t = ctx.engine_submit(empty)
    done, left = ctx.engine_advance(16)
    assert done == [(t, 0)] and left == 0
    # completions beyond the caller's capacity are returned by later calls
    tickets = [ctx.engine_submit(_job(native, h, sd, 0, ed, None, 100, 0.01)) for _ in range(3)]
    first, left = ctx.engine_advance(16, capacity=2)
    assert [d[0] for d in first] == tickets[:2] and left == 1
    rest, left = ctx.engine_advance(16, capacity=2)
    assert [d[0] for d in rest] == tickets[2:] and left == 0
    ctx.release_field(h)


def test_engine_table_grows_while_jobs_are_parked(ctx):
    """200 small jobs of all three classes (120 re-sampled steady, 40
    unsteady, 40 frozen), submitted in waves of 40 between 16-step launches,
    so that the steady table grows past its first 64 slots while earlier jobs
    are parked: the counters move with the table and every job equals the
    one-launch engine."""
    import torch
    from pars_gb300 import native, workloads as W
    rng = np.random.default_rng(21)
    steady = W.abc_field(24, noise_sigma=0.01, seed=7)
    hs = ctx.upload_field(steady)
    hu = _gyre_fields(ctx, [(20, 9)])[0][0]
    specs = []
    for k in range(200):
        kind = {3: 1, 4: 2}.get(k % 5, 0)
        c = int(rng.integers(50, 400))
        if kind == 1:
            seeds = _seeds(rng, c, 0)
        else:
            seeds = np.concatenate([rng.uniform(0.2, 6.0, (c, 3)), np.zeros((c, 1))], 1).astype(np.float32)
        specs.append((kind, torch.from_numpy(seeds).cuda(), c))

    def job(kind, sd, c):
        ed = torch.zeros((c, 4), dtype=torch.float32, device="cuda")
        st = torch.zeros(c, dtype=torch.int32, device="cuda")
        j = _job(native, hu if kind == 1 else hs, sd, c, ed, st, 200, 0.01)
        if kind == 2:
            j.stage_mode = native.STAGES_FROZEN
            j.integrator = native.INTEGRATORS["adams_bashforth_2"]
        return j, ed, st

    alone = []
    for kind, sd, c in specs:
        j, ed, st = job(kind, sd, c)
        n = ctx.batch_advect([j])[0]
        alone.append((ed.cpu().numpy(), st.cpu().numpy(), n))
    made = [job(kind, sd, c) for kind, sd, c in specs]
    tickets, got = {}, {}
    open_before_growth = None
    for wave in range(5):
        for k in range(40 * wave, 40 * wave + 40):
            tickets[ctx.engine_submit(made[k][0])] = k
        done, left = ctx.engine_advance(16)
        for t, s in done:
            got[tickets[t]] = s
        if wave == 1:
            open_before_growth = left
    assert open_before_growth >= 64      # the third wave's steady jobs grow a table that still runs
    for _ in range(100000):
        done, left = ctx.engine_advance(16)
        for t, s in done:
            got[tickets[t]] = s
        if left == 0:
            break
    assert len(got) == len(specs)
    for k, (j, ed, st) in enumerate(made):
        e, s, n = alone[k]
        assert got[k] == n, k
        assert np.array_equal(st.cpu().numpy(), s), k
        assert np.array_equal(ed.cpu().numpy(), e), k
    ctx.release_field(hs)
    ctx.release_field(hu)
