"""Writes the golden fixtures in this directory from the REFERENCE's own code.

The reference's hot-path sources, compiled unmodified against oracle/ref_shim
(oracle/build_ref.sh -> oracle/_ref/libpars_ref.so), are run on small seeded
inputs; the inputs and outputs are saved as compressed .npz files.  The
fixtures pin the CPU restatement (oracle/pars_oracle.cpp) and, through it, the
GPU kernels.  Needs the reference checkout, so it runs only where that exists:

    oracle/build_ref.sh && python tests/golden/make_golden.py [integrators]

("integrators" writes only integrators_abc24.npz.)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from pars_gb300 import workloads as W  # noqa: E402

COLORS = ["rgb", "hsv_constant_s", "hsl_constant_l", "hsl_constant_s", "hsv_constant_v"]


def field_arrays(prefix, f):
    return {prefix + "xyz": f.xyz, prefix + "offset": f.offset, prefix + "size": f.size, prefix + "spacing": f.spacing}


def curves_arrays(prefix, curves, colors_only=False):
    out = {prefix + "batches": np.array(len(curves.batches))}
    for b, batch in enumerate(curves.batches):
        if not colors_only:
            out[f"{prefix}{b}_vertices"] = batch["vertices"]
            out[f"{prefix}{b}_indices"] = batch["indices"]
        if batch["colors"] is not None:
            out[f"{prefix}{b}_colors"] = batch["colors"]
        out[f"{prefix}{b}_rank"] = np.array(batch["rank"])
        out[f"{prefix}{b}_round"] = np.array(batch["round"])
    return out


def edge_particles(f):
    """Seeds that exercise the termination rules: remaining_iterations 0..3, seeds
    outside the block, on its last vertex, exactly on cell faces, and one at
    the invalid-vertex position."""
    h = float(f.spacing[0])
    n = int(f.dims[0])
    pos = [
        (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), (1.0, 1.0, 1.0),
        (-0.5, 1.0, 1.0), (1.0, 1.0, (n - 1) * h), (1.0, (n - 2) * h, 1.0),
        (2 * h, 3 * h, 4 * h), (0.0, 0.0, 0.0), (-1.0, -1.0, -1.0), (-0.0, 0.5, 0.5),
        ((n - 1) * h - 1e-6, 0.5, 0.5),
    ]
    remaining = [0, 1, 2, 3, 50, 50, 50, 50, 50, 50, 50, 50]
    p = np.zeros(len(pos), oracle.PARTICLE_DTYPE)
    p["position"][:, :3] = np.array(pos, np.float32)
    p["remaining_iterations"] = remaining
    p["vector_field_index"] = -1
    return p


def main():
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libpars_ref.so is missing: run oracle/build_ref.sh first")

    # -- field sampling ------------------------------------------------------
    f = W.abc_field(24)
    rng = np.random.default_rng(11)
    pos = np.zeros((4000, 4), np.float32)
    pos[:, :3] = rng.uniform(-0.3, 6.6, (4000, 3)).astype(np.float32)
    h = f.spacing[0]
    # positions on cell faces and at the grid's last vertex
    grid_pts = (np.arange(24, dtype=np.float32) * h).astype(np.float32)
    pos[:24, 0] = grid_pts
    pos[24:48, 1] = grid_pts
    pos[48:72, 2] = grid_pts
    inside, vel = ref.field_sample(f, pos)
    np.savez_compressed(os.path.join(HERE, "sample_abc24.npz"), positions=pos, inside=inside, velocity=vel,
                        **field_arrays("field_", f))

    # -- seeds ----------------------------------------------------------------
    stride = (f.spacing * np.float32(3)).astype(np.float32)
    seeds = ref.seed_generate(f.offset, f.size, stride, 102, rank=3)
    odd = ref.seed_generate(np.array([0.25, -1.0, 2.0], np.float32), np.array([1.0, 2.5, 0.7], np.float32),
                            np.array([0.1, 0.3, 0.07], np.float32), 7, rank=1)
    np.savez_compressed(os.path.join(HERE, "seeds.npz"), lattice=seeds.view(np.uint8), odd=odd.view(np.uint8),
                        lattice_stride=stride)

    # -- partitioner ------------------------------------------------------------
    rows = []
    for domain in ([64, 64, 64], [512, 512, 512], [100, 37, 64], [7, 300, 11]):
        for ranks in (1, 2, 6, 8, 12, 64, 97):
            for rank in range(ranks):
                info = ref.partition(ranks, rank, domain)
                rows.append(np.concatenate([[ranks, rank], domain, info["grid"], info["block"], info["multi_rank"],
                                            info["offset"], info["ghosted"], info["neighbors"]]))
    np.savez_compressed(os.path.join(HERE, "partition.npz"), table=np.array(rows, np.int32))

    # -- streamlines, one block ----------------------------------------------------
    out = {}
    out.update(field_arrays("field_", f))
    out["seeds"] = seeds.view(np.uint8)
    for integrator, name in ((2, "rk4"), (0, "euler")):
        for k, color in enumerate(COLORS[:3] if integrator == 2 else COLORS[:1]):
            curves = ref.trace_single(f, seeds, integrator, 0.01, color, 0.75)
            out.update(curves_arrays(f"{name}_{color}_", curves, colors_only=k > 0))
    edge = edge_particles(f)
    out["edge_seeds"] = edge.view(np.uint8)
    out.update(curves_arrays("edge_", ref.trace_single(f, edge, 2, 0.05, "rgb", 0.5)))
    # a field with a zero-velocity slab: curves stop where |v| <= 1e-5
    z = W.abc_field(16)
    z.xyz[:, :, 8:] *= np.float32(1e-6)
    out.update(field_arrays("zero_field_", z))
    zs = ref.seed_generate(z.offset, z.size, (z.spacing * np.float32(2)).astype(np.float32), 80)
    out["zero_seeds"] = zs.view(np.uint8)
    out.update(curves_arrays("zero_", ref.trace_single(z, zs, 2, 0.02, "hsv_constant_v", 0.6)))
    np.savez_compressed(os.path.join(HERE, "trace_abc24.npz"), **out)

    # -- streamlines over a partitioned domain -----------------------------------------
    d = W.abc_field(17)
    ranks = 8
    rng = np.random.default_rng(5)
    n = 400
    p = rng.uniform(0, 2 * np.pi, (n, 3)).astype(np.float32)
    info0 = ref.partition(ranks, 0, d.dims)
    extent = (d.spacing * info0["block"]).astype(np.float32)
    multi = np.minimum((p / extent).astype(np.int64), info0["grid"] - 1)
    owner = (multi[:, 0] * info0["grid"][1] + multi[:, 1]) * info0["grid"][2] + multi[:, 2]
    order = np.argsort(owner, kind="stable")
    seeds_m = np.zeros(n, oracle.PARTICLE_DTYPE)
    seeds_m["position"][:, :3] = p[order]
    seeds_m["remaining_iterations"] = 152
    seeds_m["vector_field_index"] = -1
    offsets = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=ranks))]).astype(np.int64)
    curves = ref.trace_multi(d, ranks, offsets, seeds_m, 2, 0.01, "rgb", 0.5)
    np.savez_compressed(os.path.join(HERE, "multi_abc17.npz"), seeds=seeds_m.view(np.uint8), seed_offsets=offsets,
                        ranks=np.array(ranks), **field_arrays("field_", d), **curves_arrays("multi_", curves))

    # -- flow maps -------------------------------------------------------------------
    g = W.abc_field(16, noise_sigma=0.01, seed=0)
    fm = {}
    fm.update(field_arrays("field_", g))
    fm["rk4_s1"] = ref.flow_map(g, 61, 1.0, 2, 0.01)
    fm["euler_s1"] = ref.flow_map(g, 31, 1.0, 0, 0.02)
    fm["rk4_s05"] = ref.flow_map(g, 41, 0.5, 2, 0.01)
    np.savez_compressed(os.path.join(HERE, "flow_abc16.npz"), **fm)

    # -- index / colour on hand-built buffers ----------------------------------------------
    T = np.array([-2, -2, -2, 0], np.float32)
    I = np.array([-1, -1, -1, 0], np.float32)
    rng = np.random.default_rng(7)
    v = rng.normal(size=(64, 4)).astype(np.float32)
    v[:, 3] = 0
    for k in (5, 6, 17, 30, 31, 63):
        v[k] = T
    v[40] = I
    v[41] = v[42]          # zero-length segment (tangent 0)
    v[50, :3] = v[49, :3] + np.float32(1e-30)
    ic = {"vertices": v, "indices": ref.index_generate(v)}
    for color in COLORS:
        ic["colors_" + color] = ref.color_generate(v, ic["indices"], color, 0.3)
    only_term = np.tile(T, (5, 1))
    ic["only_term_indices"] = ref.index_generate(only_term)
    ic["two_indices"] = ref.index_generate(v[:2])
    np.savez_compressed(os.path.join(HERE, "index_color.npz"), **ic)
    print("golden fixtures written to", HERE)


INTEGRATORS = ["euler", "modified_midpoint", "runge_kutta_4", "runge_kutta_cash_karp_54", "runge_kutta_dormand_prince_5",
               "runge_kutta_fehlberg_78", "adams_bashforth_2", "adams_bashforth_moulton_2"]


def integrators():
    """Streamlines and flow maps with each of the eight steppers of
    pa/include/pa/math/integrators.hpp:16-23 (frozen velocity, as the reference
    integrates), through the reference's tracer and advector."""
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libpars_ref.so is missing: run oracle/build_ref.sh first")
    f = W.abc_field(24)
    seeds = ref.seed_generate(f.offset, f.size, (f.spacing * np.float32(4)).astype(np.float32), 82)
    g = W.abc_field(16, noise_sigma=0.01, seed=0)
    out = {"seeds": seeds.view(np.uint8)}
    out.update(field_arrays("field_", f))
    out.update(field_arrays("flow_field_", g))
    for k, name in enumerate(INTEGRATORS):
        curves = ref.trace_single(f, seeds, k, 0.02, None, 0.5)
        out[f"{name}_batches"] = np.array(len(curves.batches))
        for b, batch in enumerate(curves.batches):
            out[f"{name}_{b}_vertices"] = batch["vertices"]
        out[f"{name}_flow"] = ref.flow_map(g, 41, 1.0, k, 0.02)
    np.savez_compressed(os.path.join(HERE, "integrators_abc24.npz"), **out)
    print("integrator fixtures written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:] == ["integrators"]:
        integrators()
    else:
        main()
