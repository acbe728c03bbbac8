"""The CPU restatement (oracle/pars_oracle.cpp) against golden fixtures written
by the reference's own code (tests/golden/make_golden.py).  Bit-exact."""
import numpy as np
import pytest

from conftest import golden, golden_curves, golden_field, particles_from, assert_colors_equal


def test_field_sampling_matches_reference(port):
    g = golden("sample_abc24.npz")
    f = golden_field(g)
    inside, vel = port.field_sample(f, g["positions"])
    assert np.array_equal(inside, g["inside"].astype(bool))
    assert np.array_equal(vel, g["velocity"])


def test_seed_generator_matches_reference(port):
    g = golden("seeds.npz")
    f = golden_field(golden("sample_abc24.npz"))
    lattice = port.seed_generate(f.offset, f.size, g["lattice_stride"], 102, rank=3)
    assert lattice.view(np.uint8).tobytes() == g["lattice"].tobytes()
    odd = port.seed_generate(np.array([0.25, -1.0, 2.0], np.float32), np.array([1.0, 2.5, 0.7], np.float32),
                             np.array([0.1, 0.3, 0.07], np.float32), 7, rank=1)
    assert odd.view(np.uint8).tobytes() == g["odd"].tobytes()


def test_partitioner_matches_reference(port):
    table = golden("partition.npz")["table"]
    for row in table:
        ranks, rank = int(row[0]), int(row[1])
        domain = row[2:5]
        info = port.partition(ranks, rank, domain)
        got = np.concatenate([info["grid"], info["block"], info["multi_rank"], info["offset"], info["ghosted"], info["neighbors"]])
        assert np.array_equal(got, row[5:]), (ranks, rank, domain)


def _compare_curves(got, expected, colors=True, colors_only=False):
    """Batches compared in (rank, round) order; within one rank and round the
    batch order is the reference's."""
    assert len(got.batches) == len(expected)
    key = lambda b: (b["rank"], b["round"])
    for a, e in zip(sorted(got.batches, key=key), sorted(expected, key=key)):
        assert (a["rank"], a["round"]) == (e["rank"], e["round"])
        if not colors_only:
            assert np.array_equal(a["vertices"], e["vertices"])
            assert np.array_equal(a["indices"], e["indices"])
        if colors and e["colors"] is not None:
            assert_colors_equal(a["colors"], e["colors"])


@pytest.mark.parametrize("integrator,name,color", [
    (2, "rk4", "rgb"), (2, "rk4", "hsv_constant_s"), (2, "rk4", "hsl_constant_l"), (0, "euler", "rgb")])
def test_streamlines_match_reference(port, integrator, name, color):
    g = golden("trace_abc24.npz")
    f = golden_field(g)
    seeds = particles_from(g, "seeds")
    got = port.trace_single(f, seeds, integrator, 0.01, color, 0.75)
    expected = golden_curves(g, f"{name}_{color}_")
    if color != "rgb":
        base = golden_curves(g, f"{name}_rgb_")
        for e, b in zip(expected, base):
            e["vertices"], e["indices"] = b["vertices"], b["indices"]
    _compare_curves(got, expected)


def test_streamline_edge_cases_match_reference(port):
    g = golden("trace_abc24.npz")
    f = golden_field(g)
    got = port.trace_single(f, particles_from(g, "edge_seeds"), 2, 0.05, "rgb", 0.5)
    _compare_curves(got, golden_curves(g, "edge_"))


def test_zero_velocity_termination_matches_reference(port):
    g = golden("trace_abc24.npz")
    f = golden_field(g, "zero_field_")
    got = port.trace_single(f, particles_from(g, "zero_seeds"), 2, 0.02, "hsv_constant_v", 0.6)
    _compare_curves(got, golden_curves(g, "zero_"))


def test_partitioned_domain_matches_reference(port):
    g = golden("multi_abc17.npz")
    f = golden_field(g)
    got = port.trace_multi(f, int(g["ranks"]), g["seed_offsets"], particles_from(g, "seeds"), 2, 0.01, "rgb", 0.5)
    _compare_curves(got, golden_curves(g, "multi_"))
    assert got.steps > 0


@pytest.mark.parametrize("key,iterations,scale,integrator,step", [
    ("rk4_s1", 61, 1.0, 2, 0.01), ("euler_s1", 31, 1.0, 0, 0.02), ("rk4_s05", 41, 0.5, 2, 0.01)])
def test_flow_map_matches_reference(port, key, iterations, scale, integrator, step):
    g = golden("flow_abc16.npz")
    f = golden_field(g)
    flow, steps = port.flow_map(f, iterations, scale, integrator, step)
    assert np.array_equal(flow, g[key])
    assert steps > 0


def test_index_and_color_buffers_match_reference(port):
    g = golden("index_color.npz")
    v = g["vertices"]
    idx = port.index_generate(v)
    assert np.array_equal(idx, g["indices"])
    for mode in ("rgb", "hsv_constant_s", "hsl_constant_l", "hsl_constant_s", "hsv_constant_v"):
        assert_colors_equal(port.color_generate(v, idx, mode, 0.3), g["colors_" + mode])
    assert len(port.index_generate(np.tile(np.array([-2, -2, -2, 0], np.float32), (5, 1)))) == 0
    assert np.array_equal(port.index_generate(v[:2]), g["two_indices"])


def test_reference_build_agrees_when_present(port):
    """Where the reference checkout exists, also run it live on a fresh case."""
    import oracle
    from pars_gb300 import workloads as W
    ref = oracle.reference()
    if ref is None:
        pytest.skip("reference build not available on this machine")
    f = W.abc_field(20)
    seeds = ref.seed_generate(f.offset, f.size, (f.spacing * np.float32(2)).astype(np.float32), 77)
    a = ref.trace_single(f, seeds, 2, 0.03, "hsv_constant_s", 0.4)
    b = port.trace_single(f, seeds, 2, 0.03, "hsv_constant_s", 0.4)
    for x, y in zip(a.batches, b.batches):
        assert np.array_equal(x["vertices"], y["vertices"])
        assert_colors_equal(y["colors"], x["colors"])


INTEGRATORS = ["euler", "modified_midpoint", "runge_kutta_4", "runge_kutta_cash_karp_54", "runge_kutta_dormand_prince_5",
               "runge_kutta_fehlberg_78", "adams_bashforth_2", "adams_bashforth_moulton_2"]


@pytest.mark.parametrize("k,name", list(enumerate(INTEGRATORS)))
def test_every_integrator_matches_reference(port, k, name):
    """The eight steppers of integrators.hpp:16-23 with the reference's frozen
    velocity: streamlines (particle_tracer) and flow maps (particle_advector),
    bit for bit against the reference build (odeint stand-in of oracle/ref_shim)."""
    g = golden("integrators_abc24.npz")
    f = golden_field(g)
    seeds = particles_from(g, "seeds")
    curves = port.trace_single(f, seeds, k, 0.02, None, 0.5)
    assert len(curves.batches) == int(g[f"{name}_batches"])
    for b, batch in enumerate(curves.batches):
        assert np.array_equal(batch["vertices"], g[f"{name}_{b}_vertices"])
    flow, _ = port.flow_map(golden_field(g, "flow_field_"), 41, 1.0, k, 0.02)
    assert np.array_equal(flow, g[f"{name}_flow"])
