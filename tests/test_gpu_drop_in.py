"""The C++ drop-in (include/pa_gpu.hpp) driven the way pars::pipeline drives
the reference stages (tests/cpp/drop_in_pipeline.cpp), compiled with g++ and
checked against the oracle: bit-exact curves and indices, hsv colours within
2e-6, the ray tracer's `image` reply byte-identical to the CPU restatement's
render of the same curves, FTLE within 1e-4 of the FP64 evaluation of the
same flow map; and, with one thread per rank running pipeline.cpp's round
loop stage by stage (compute_round_info, allocate, initialize, trace,
out_of_bounds_distribute, check_completion; then prune, index, colour), a
64-block domain bit-exact per (rank, round) batch against the oracle's
round-by-round restatement of the reference's exchange."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, assert_colors_equal

pytestmark = pytest.mark.gpu


def _build(tmp):
    from pars_gb300 import native
    exe = os.path.join(tmp, "drop_in_pipeline")
    lib_dir = os.path.dirname(native.LIBRARY_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "drop_in_pipeline.cpp"), "-L" + lib_dir, "-lpars_gpu",
                    "-Wl,-rpath," + lib_dir, "-lpthread", "-o", exe], check=True)
    return exe


def test_cpp_drop_in_pipeline_matches_oracle(port):
    from pars_gb300 import workloads as W
    f = W.abc_field(32)
    with tempfile.TemporaryDirectory() as tmp:
        exe = _build(tmp)
        field_path = os.path.join(tmp, "field.bin")
        f.xyz.tofile(field_path)
        iterations, step, stride = 302, 0.01, 2
        r = subprocess.run([exe, "single", field_path, *map(str, f.dims), repr(float(f.spacing[0])), str(stride), str(iterations),
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


def test_cpp_drop_in_round_loop_64_ranks_matches_oracle(port):
    """64 ranks as threads (4x4x4 blocks of a 49^3 ABC field), 6000 clustered
    seeds, frozen RK4: every rank's batches, tagged by the round that
    allocated them, equal the oracle's (rank, round) batches bit for bit,
    with indices and rgb colours."""
    from pars_gb300 import workloads as W
    f = W.abc_field(49)
    ranks = 64
    info = port.partition(ranks, 0, f.dims)
    rng = np.random.default_rng(2)
    n = 6000
    centres = rng.uniform(1.0, 5.3, (4, 3))
    p = (centres[rng.integers(0, 4, n)] + rng.normal(0, 0.05 * 2 * np.pi, (n, 3))).clip(0, 6.2).astype(np.float32)
    extent = (f.spacing * info["block"]).astype(np.float32)
    multi = np.minimum((p / extent).astype(np.int64), info["grid"] - 1)
    owner = (multi[:, 0] * info["grid"][1] + multi[:, 1]) * info["grid"][2] + multi[:, 2]
    order = np.argsort(owner, kind="stable")
    import oracle
    seeds = np.zeros(n, oracle.PARTICLE_DTYPE)
    seeds["position"][:, :3] = p[order]
    seeds["remaining_iterations"] = 402
    seeds["vector_field_index"] = -1
    offsets = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=ranks))]).astype(np.int64)
    expected = port.trace_multi(f, ranks, offsets, seeds, 2, 0.01, "rgb", 0.5)
    want = {(b["rank"], b["round"]): b for b in expected.batches}
    with tempfile.TemporaryDirectory() as tmp:
        exe = _build(tmp)
        domain_path, seeds_path, offsets_path = (os.path.join(tmp, x) for x in ("domain.bin", "seeds.bin", "offsets.bin"))
        f.xyz.tofile(domain_path)
        seeds.tofile(seeds_path)
        offsets.tofile(offsets_path)
        r = subprocess.run([exe, "multi", domain_path, *map(str, f.dims), repr(float(f.spacing[0])), str(ranks), seeds_path,
                            offsets_path, "0.01", tmp], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        seen = set()
        for rank in range(ranks):
            lines = open(os.path.join(tmp, f"rank_{rank}.txt")).read().split("\n")
            per_round = {}
            for k, line in enumerate(x for x in lines if x):
                rnd, nv, ni = map(int, line.split())
                name = os.path.join(tmp, f"rank_{rank}_batch_{k}")
                v = np.fromfile(name + "_vertices.bin", np.float32).reshape(-1, 4)
                c = np.fromfile(name + "_colors.bin", np.float32).reshape(-1, 4)
                i = np.fromfile(name + "_indices.bin", np.int32)
                assert len(v) == nv and len(i) == ni
                per_round.setdefault(rnd, []).append(k)
                e = want[(rank, rnd)]
                assert np.array_equal(v, e["vertices"]), (rank, rnd)
                assert np.array_equal(i, e["indices"]), (rank, rnd)
                assert_colors_equal(c, e["colors"])
                seen.add((rank, rnd))
            for rnd, ks in per_round.items():
                assert len(ks) == 1, "the 6000-seed rounds fit one batch per rank"
        assert seen == set(want), "every (rank, round) batch of the oracle was produced"
