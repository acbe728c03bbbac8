"""GPU accuracy against FP64 oracles (true RK4 with re-sampled stages, FTLE).

Bars (from the project's precision targets):
* end-point error of re-sampled RK4 streamlines <= 1e-3 cell widths after
  1000 steps, for every curve whose step count equals the FP64 oracle's;
  curves whose count differs must end within 1e-3 cells of the domain
  boundary (the termination test flips there);
* FTLE relative error <= 1e-4 against the FP64 evaluation of the same flow
  map, counted where |FTLE| >= 1e-2 * max|FTLE| (below that floor the
  absolute error is held to 1e-4 * 1e-2 * max|FTLE|);
* FTLE of a linear flow equals ln(sigma_max(e^{AT})) / T within 1e-4.
"""
import numpy as np
import pytest
import scipy.linalg

pytestmark = pytest.mark.gpu


def split_curves(vertices):
    """Pruned vertices [seed, x1..xk, TERM]* -> list of (k+1, 4) arrays."""
    term = np.all(vertices == np.array([-2, -2, -2, 0], np.float32), axis=1)
    ends = np.nonzero(term)[0]
    out, start = [], 0
    for e in ends:
        out.append(vertices[start:e])
        start = e + 1
    return out


def test_resampled_rk4_streamlines_within_1e3_cells(ctx, port):
    from pars_gb300 import workloads as W
    cfg = W.streamline_config()
    f = cfg["field"]
    seeds = port.seed_generate(f.offset, f.size, cfg["stride"], cfg["iterations"])
    h = ctx.upload_field(f)
    s = ctx.trace(h, seeds, 2, 1, cfg["step"])
    assert s["batches"] == 1
    curves = split_curves(ctx.curves(1)[0]["vertices"])
    assert len(curves) == len(seeds)
    end64, steps64, _ = port.advect_fp64(f, seeds["position"][:, :3].astype(np.float64), cfg["iterations"] - 2,
                                         integrator=2, mode=1, step=cfg["step"])
    cell = float(f.spacing[0])
    steps32 = np.array([len(c) - 1 for c in curves])
    same = steps32 == steps64
    end32 = np.array([c[-1, :3] for c in curves], np.float64)
    err = np.linalg.norm(end32[same] - end64[same], axis=1) / cell
    assert err.max() <= 1e-3, f"max end-point error {err.max()} cells"
    # curves whose step count differs end at the domain boundary
    lo = f.offset.astype(np.float64)
    hi = lo + (f.dims - 1) * f.spacing.astype(np.float64)
    for i in np.nonzero(~same)[0]:
        k = min(steps32[i], steps64[i])
        p = curves[i][k, :3].astype(np.float64)
        gap = np.minimum(np.abs(p - lo), np.abs(hi - p)).min() / cell
        assert gap <= 1e-3 + 2 * float(cfg["step"]) * 5 / cell, (i, gap)
    assert same.mean() > 0.99
    ctx.release_field(h)


def test_resampled_flow_map_within_1e3_cells(ctx, port):
    from pars_gb300 import workloads as W
    f = W.abc_field(40, noise_sigma=0.01, seed=0)
    h = ctx.upload_field(f)
    iterations = 501
    fm, steps = ctx.flow_map_generate(h, iterations, 1.0, 2, 1, 0.01)
    flow = ctx.download_field(fm)
    start = np.stack(np.meshgrid(*[np.arange(n) for n in f.dims], indexing="ij"), -1).reshape(-1, 3)
    start = (start.astype(np.float32) * f.spacing).astype(np.float32).astype(np.float64)
    end64, steps64, _ = port.advect_fp64(f, start, iterations - 1, integrator=2, mode=1, step=0.01)
    assert steps == int(steps64.sum()) or abs(steps - int(steps64.sum())) < 1e-3 * steps
    err = np.linalg.norm(flow.reshape(-1, 3) - end64, axis=1) / float(f.spacing[0])
    # particles that exit at a different step stop at different places; all
    # others are held to the bar
    inside = np.all((end64 >= 0) & (end64 <= 2 * np.pi), axis=1)
    finished = steps64 == iterations - 1
    assert np.max(err[finished & inside]) <= 1e-3
    ctx.release_field(fm)
    ctx.release_field(h)


def test_ftle_matches_fp64_on_the_same_flow_map(ctx, port):
    from pars_gb300 import workloads as W
    f = W.abc_field(48, noise_sigma=0.01, seed=0)
    h = ctx.upload_field(f)
    fm, _ = ctx.flow_map_generate(h, 301, 1.0, 2, 1, 0.01)
    flow = ctx.download_field(fm)
    T = 3.0
    got = ctx.ftle_generate(fm, T, 0, shape=tuple(f.dims))
    ref = port.ftle_fp64(flow, f.spacing, T)
    floor = 1e-2 * np.abs(ref).max()
    big = np.abs(ref) >= floor
    rel = np.abs(got[big] - ref[big]) / np.abs(ref[big])
    assert rel.max() <= 1e-4, rel.max()
    assert np.abs(got[~big] - ref[~big]).max() <= 1e-4 * floor
    ctx.release_field(fm)
    ctx.release_field(h)


def test_fractional_anisotropy_matches_fp64_on_the_same_flow_map(ctx, port):
    """FA mode (ftle_map_generator.cpp:51-54): FA lies in [0, 1]; the FP32
    kernel (from the invariants of C) within 1e-5 absolute of the FP64
    oracle's eigenvalue formula on the same flow map, and the isotropic case
    (a flow map equal to the identity, C = I up to the FP32 rounding of the
    lattice positions) gives the oracle's near-zero values."""
    from pars_gb300 import workloads as W
    f = W.abc_field(48, noise_sigma=0.01, seed=0)
    h = ctx.upload_field(f)
    fm, _ = ctx.flow_map_generate(h, 301, 1.0, 2, 1, 0.01)
    flow = ctx.download_field(fm)
    got = ctx.ftle_generate(fm, 3.0, 1, shape=tuple(f.dims))
    ref = port.ftle_fp64(flow, f.spacing, 3.0, mode=1)
    assert np.all((ref >= 0) & (ref <= 1 + 1e-12))
    assert np.abs(got - ref).max() <= 1e-5, np.abs(got - ref).max()
    # C = I: identity flow map on its own lattice (the seeds of one iteration)
    fm1, _ = ctx.flow_map_generate(h, 1, 1.0, 2, 1, 0.01)
    iso = ctx.ftle_generate(fm1, 3.0, 1, shape=tuple(f.dims))
    iso_ref = port.ftle_fp64(ctx.download_field(fm1), f.spacing, 3.0, mode=1)
    assert np.abs(iso_ref).max() <= 1e-5
    assert np.abs(iso - iso_ref).max() <= 1e-6
    ctx.release_field(fm1)
    ctx.release_field(fm)
    ctx.release_field(h)


def test_ftle_of_linear_flow_is_analytic(ctx):
    from pars_gb300 import workloads as W
    A = np.array([[0.30, 0.05, 0.00], [0.02, -0.10, 0.04], [0.00, 0.03, -0.20]])
    n = 41
    f = W.linear_field(n, A, spacing=0.05)
    h = ctx.upload_field(f)
    T = 2.0
    step = 0.01
    fm, _ = ctx.flow_map_generate(h, int(round(T / step)) + 1, 1.0, 2, 1, step)
    got = ctx.ftle_generate(fm, T, 0, shape=(n, n, n))
    expected = np.log(np.linalg.svd(scipy.linalg.expm(A * T), compute_uv=False).max()) / T
    # interior voxels whose particles and neighbours stay inside the grid
    core = got[14:27, 14:27, 14:27]
    assert np.abs(core - expected).max() <= 1e-4 * abs(expected)
    ctx.release_field(fm)
    ctx.release_field(h)


@pytest.mark.parametrize("integrator", [0, 1, 3, 4, 5, 6, 7])
def test_resampled_schemes_of_every_integrator_within_1e3_cells(ctx, port, integrator):
    """Re-sampled stages ("true form") of the other integrators: streamlines
    and flow maps against the FP64 oracle of the same scheme (1e-3 cells for
    curves with the oracle's step count, as for RK4)."""
    from pars_gb300 import native, workloads as W
    f = W.abc_field(40)
    seeds = port.seed_generate(f.offset, f.size, (f.spacing * np.float32(3)).astype(np.float32), 402)
    h = ctx.upload_field(f)
    s = ctx.trace(h, seeds, integrator, native.STAGES_RESAMPLED, 0.01)
    vertices = np.concatenate([b["vertices"] for b in ctx.curves(s["batches"])])
    curves = split_curves(vertices)
    assert len(curves) == len(seeds)
    end64, steps64, _ = port.advect_fp64(f, seeds["position"][:, :3].astype(np.float64), 400, integrator=integrator,
                                         mode=1, step=0.01)
    cell = float(f.spacing[0])
    steps32 = np.array([len(c) - 1 for c in curves])
    same = steps32 == steps64
    assert same.mean() > 0.98
    end32 = np.array([c[-1, :3] for c in curves], np.float64)
    err = np.linalg.norm(end32[same] - end64[same], axis=1) / cell
    assert err.max() <= 1e-3, f"max end-point error {err.max()} cells"
    # flow map (per-seed kernel) against the same oracle
    fm, _ = ctx.flow_map_generate(h, 201, 1.0, integrator, native.STAGES_RESAMPLED, 0.01)
    flow = ctx.download_field(fm).reshape(-1, 3).astype(np.float64)
    g = np.stack(np.meshgrid(*[np.arange(40, dtype=np.float32) * f.spacing[0]] * 3, indexing="ij"), -1).reshape(-1, 3)
    pick = np.arange(0, len(g), 97)
    e64, s64, _ = port.advect_fp64(f, g[pick].astype(np.float64), 200, integrator=integrator, mode=1, step=0.01)
    inside = s64 == 200
    assert inside.sum() >= 100
    ferr = np.linalg.norm(flow[pick][inside] - e64[inside], axis=1) / cell
    # (the flow map has no per-seed step count: a seed whose path grazes the
    # boundary may stop on one side only)
    assert (ferr <= 1e-3).mean() >= 0.99, np.quantile(ferr, 0.99)
    ctx.release_field(fm)
    ctx.release_field(h)
