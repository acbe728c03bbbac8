"""Seeded synthetic inputs with the shapes of the five tracing workloads.

The reference's benchmarks ran on a private dataset; these fields stand in for
it.  A field follows ``pa::vector_field`` (pa/include/pa/math/vector_field.hpp:
14-24): ``xyz`` is ``[X][Y][Z][3]`` FP32 in C order (z fastest), ``offset``,
``size`` and ``spacing`` are FP32 3-vectors, and ``size = shape * spacing`` as
data_io.cpp:113 sets it (it counts one cell more than can be interpolated).
"""
import ctypes

import numpy as np

ABC_A = np.sqrt(3.0)
ABC_B = np.sqrt(2.0)
ABC_C = 1.0


class Field:
    """A steady vector field on a regular grid (host copy)."""

    def __init__(self, xyz, offset, spacing, size=None):
        self.xyz = np.ascontiguousarray(xyz, np.float32)
        assert self.xyz.ndim == 4 and self.xyz.shape[3] == 3
        self.dims = np.array(self.xyz.shape[:3], np.int32)
        self.offset = np.ascontiguousarray(offset, np.float32)
        self.spacing = np.ascontiguousarray(spacing, np.float32)
        if size is None:
            size = (self.dims.astype(np.float32) * self.spacing).astype(np.float32)
        self.size = np.ascontiguousarray(size, np.float32)

    def ctypes_args(self):
        return (self.xyz.ctypes.data, self.dims.ctypes.data, self.offset.ctypes.data,
                self.size.ctypes.data, self.spacing.ctypes.data)

    @property
    def nbytes(self):
        return self.xyz.nbytes


def abc_velocity(x, y, z, A=ABC_A, B=ABC_B, C=ABC_C):
    """Arnold-Beltrami-Childress flow (u, v, w) in FP64."""
    return (A * np.sin(z) + C * np.cos(y),
            B * np.sin(x) + A * np.cos(z),
            C * np.sin(y) + B * np.cos(x))


def abc_field(n, noise_sigma=0.0, seed=None, A=ABC_A, B=ABC_B, C=ABC_C):
    """ABC flow sampled at the n^3 vertices of [0, 2pi]^3 (spacing 2pi/(n-1),
    offset 0), optionally plus N(0, noise_sigma) per component from
    numpy's PCG64 generator with the given seed.  Built slab by slab to keep
    the FP64 temporaries small at 256^3 and above."""
    h = 2.0 * np.pi / (n - 1)
    coords = np.arange(n) * h
    xyz = np.empty((n, n, n, 3), np.float32)
    Y, Z = np.meshgrid(coords, coords, indexing="ij")
    rng = np.random.default_rng(seed) if noise_sigma else None
    for i in range(n):
        u, v, w = abc_velocity(coords[i], Y, Z, A, B, C)
        slab = np.stack([np.broadcast_to(u, Y.shape), v, np.broadcast_to(w, Y.shape)], -1)
        if rng is not None:
            slab = slab + rng.standard_normal(slab.shape) * noise_sigma
        xyz[i] = slab
    spacing = np.full(3, np.float32(h), np.float32)
    return Field(xyz, np.zeros(3, np.float32), spacing)


def linear_field(n, matrix, spacing=0.1, offset=(0.0, 0.0, 0.0)):
    """v(x) = M (x - centre) sampled on an n^3 grid; trilinear interpolation
    reproduces it exactly (up to FP32 rounding of the samples)."""
    h = np.float32(spacing)
    coords = np.arange(n, dtype=np.float64) * float(h)
    X, Y, Z = np.meshgrid(coords, coords, coords, indexing="ij")
    c = float(h) * (n - 1) / 2.0
    P = np.stack([X - c, Y - c, Z - c], -1)
    xyz = (P @ np.asarray(matrix, np.float64).T).astype(np.float32)
    return Field(xyz, np.asarray(offset, np.float32) + 0, np.full(3, h, np.float32))


def uniform_field(n, velocity, spacing=0.25):
    xyz = np.empty((n, n, n, 3), np.float32)
    xyz[...] = np.asarray(velocity, np.float32)
    return Field(xyz, np.zeros(3, np.float32), np.full(3, np.float32(spacing), np.float32))


def double_gyre_slices(n, slices, period=10.0, A=0.1, eps=0.25):
    """Unsteady 3-D double gyre on [0,2] x [0,1] x [0,1] sampled at n^3
    vertices and `slices` times spanning one period (t_k = k * period /
    (slices - 1)); omega = 2 pi / period, w = 0:
        f(x,t) = eps sin(wt) x^2 + (1 - 2 eps sin(wt)) x
        u = -pi A sin(pi f) cos(pi y),  v = pi A cos(pi f) sin(pi y) df/dx.
    Returns (xyz [slices, n, n, n, 3] FP32, offset, spacing, t0, slice_dt)."""
    omega = 2.0 * np.pi / period
    x = np.linspace(0.0, 2.0, n)
    y = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(x, y, indexing="ij")
    out = np.zeros((slices, n, n, n, 3), np.float32)
    dt = period / (slices - 1)
    for k in range(slices):
        t = k * dt
        a = eps * np.sin(omega * t)
        b = 1.0 - 2.0 * a
        f = a * X * X + b * X
        dfdx = 2.0 * a * X + b
        u = -np.pi * A * np.sin(np.pi * f) * np.cos(np.pi * Y)
        v = np.pi * A * np.cos(np.pi * f) * np.sin(np.pi * Y) * dfdx
        out[k, :, :, :, 0] = u[:, :, None]
        out[k, :, :, :, 1] = v[:, :, None]
    spacing = np.array([2.0 / (n - 1), 1.0 / (n - 1), 1.0 / (n - 1)], np.float32)
    return out, np.zeros(3, np.float32), spacing, 0.0, dt


def pathline_batch_config(seed=3, fields=32):
    """The batched-pathline workload: `fields` double-gyre fields with edge
    log-uniform in [32, 256], 16-64 slices, seed counts log-uniform in
    [1k, 512k], drawn with numpy's PCG64 from `seed`."""
    rng = np.random.default_rng(seed)
    edges = np.exp(rng.uniform(np.log(32), np.log(256), fields)).astype(int)
    slices = rng.integers(16, 65, fields)
    seeds = np.exp(rng.uniform(np.log(1000), np.log(512 * 1024), fields)).astype(int)
    return [{"edge": int(e), "slices": int(s), "seeds": int(c)} for e, s, c in zip(edges, slices, seeds)]


def double_gyre_device(torch, n, slices, period=10.0, A=0.1, eps=0.25):
    """double_gyre_slices computed on the GPU with torch (the 32-field
    workload holds ~48 GB of slices; building them on the host would dominate
    the run).  Returns (xyz device tensor [slices, n, n, n, 3] FP32, offset,
    spacing, t0, slice_dt)."""
    omega = 2.0 * np.pi / period
    x = torch.linspace(0.0, 2.0, n, dtype=torch.float64, device="cuda")
    y = torch.linspace(0.0, 1.0, n, dtype=torch.float64, device="cuda")
    X, Y = torch.meshgrid(x, y, indexing="ij")
    out = torch.zeros((slices, n, n, n, 3), dtype=torch.float32, device="cuda")
    dt = period / (slices - 1)
    for k in range(slices):
        t = k * dt
        a = eps * np.sin(omega * t)
        b = 1.0 - 2.0 * a
        f = a * X * X + b * X
        dfdx = 2.0 * a * X + b
        u = -np.pi * A * torch.sin(np.pi * f) * torch.cos(np.pi * Y)
        v = np.pi * A * torch.cos(np.pi * f) * torch.sin(np.pi * Y) * dfdx
        out[k, :, :, :, 0] = u.float()[:, :, None]
        out[k, :, :, :, 1] = v.float()[:, :, None]
    spacing = np.array([2.0 / (n - 1), 1.0 / (n - 1), 1.0 / (n - 1)], np.float32)
    return out, np.zeros(3, np.float32), spacing, 0.0, dt


def fourier_modes(seed=1, modes=8, amplitude=0.1):
    """Random Fourier perturbation: integer wave vectors in [-4, 4]^3 (non-zero),
    random unit directions and phases; each mode has amplitude
    amplitude / sqrt(modes), so the sum has RMS amplitude about amplitude/sqrt(2)."""
    rng = np.random.default_rng(seed)
    k = rng.integers(-4, 5, (modes, 3))
    k[np.all(k == 0, axis=1)] = (1, 0, 0)
    d = rng.normal(size=(modes, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    phase = rng.uniform(0.0, 2.0 * np.pi, modes)
    return k.astype(np.float64), d, phase, amplitude / np.sqrt(modes)


def beltrami_fourier_device(torch, n, seed=1):
    """ABC (Arnold-Beltrami) flow on the n^3 vertices of [0, 2pi]^3 plus
    fourier_modes(seed), computed slab by slab on the GPU.  Returns (xyz device
    tensor [n, n, n, 3] FP32, spacing)."""
    h = 2.0 * np.pi / (n - 1)
    c = torch.arange(n, dtype=torch.float64, device="cuda") * h
    Y, Z = torch.meshgrid(c, c, indexing="ij")
    k, d, phase, amp = fourier_modes(seed)
    out = torch.empty((n, n, n, 3), dtype=torch.float32, device="cuda")
    for i in range(n):
        x = float(c[i])
        u = ABC_A * torch.sin(Z) + ABC_C * torch.cos(Y)
        v = ABC_B * np.sin(x) + ABC_A * torch.cos(Z)
        w = ABC_C * torch.sin(Y) + ABC_B * np.cos(x)
        for m in range(len(k)):
            s = amp * torch.sin(k[m, 0] * x + k[m, 1] * Y + k[m, 2] * Z + phase[m])
            u = u + d[m, 0] * s
            v = v + d[m, 1] * s
            w = w + d[m, 2] * s
        out[i, :, :, 0] = u.float()
        out[i, :, :, 1] = v.float()
        out[i, :, :, 2] = w.float()
    return out, np.full(3, np.float32(h), np.float32)


def gaussian_mixture_seeds(count, n, spacing, partition, remaining, seed=2, centres=4, sigma_fraction=0.05):
    """`count` seeds from a `centres`-centre Gaussian mixture in [0, L)^3,
    L = (n - 1) * spacing, sigma = sigma_fraction * L, clipped into the
    domain; grouped by owning block of `partition` (the partitioner's grid).
    Returns (particles sorted by owner, seed_offsets per block)."""
    from .native import PARTICLE_DTYPE
    rng = np.random.default_rng(seed)
    L = float((n - 1) * spacing[0])
    centre = rng.uniform(0.2 * L, 0.8 * L, (centres, 3))
    which = rng.integers(0, centres, count)
    p = centre[which] + rng.normal(0.0, sigma_fraction * L, (count, 3))
    p = np.clip(p, 0.0, np.nextafter(L, 0.0)).astype(np.float32)
    grid = partition["grid"]
    extent = (spacing * partition["block"]).astype(np.float32)
    multi = np.minimum((p / extent).astype(np.int64), grid - 1)
    owner = (multi[:, 0] * grid[1] + multi[:, 1]) * grid[2] + multi[:, 2]
    order = np.argsort(owner, kind="stable")
    particles = np.zeros(count, PARTICLE_DTYPE)
    particles["position"][:, :3] = p[order]
    particles["remaining_iterations"] = remaining
    particles["vector_field_index"] = -1
    ranks = int(np.prod(grid))
    offsets = np.concatenate([[0], np.cumsum(np.bincount(owner, minlength=ranks))]).astype(np.int64)
    return particles, offsets


def abc_device(torch, n):
    """abc_field(n) computed on the GPU; returns (xyz device tensor, offset, size, spacing)."""
    h = 2.0 * np.pi / (n - 1)
    c = torch.arange(n, dtype=torch.float64, device="cuda") * h
    Y, Z = torch.meshgrid(c, c, indexing="ij")
    out = torch.empty((n, n, n, 3), dtype=torch.float32, device="cuda")
    for i in range(n):
        x = float(c[i])
        out[i, :, :, 0] = (ABC_A * torch.sin(Z) + ABC_C * torch.cos(Y)).float()
        out[i, :, :, 1] = (ABC_B * np.sin(x) + ABC_A * torch.cos(Z)).float()
        out[i, :, :, 2] = (ABC_C * torch.sin(Y) + ABC_B * np.cos(x)).float()
    spacing = np.full(3, np.float32(h), np.float32)
    return out, np.zeros(3, np.float32), (spacing * np.float32(n)).astype(np.float32), spacing


def gyre_snapshot_device(torch, n, t=2.5):
    """One time slice (time t) of the double gyre on n^3 vertices of
    [0,2] x [0,1] x [0,1], as a steady field."""
    xyz, offset, spacing, t0, dt = double_gyre_device(torch, n, 2, period=10.0)
    # double_gyre_device gives slices at t = 0 and t = period; rebuild at t
    omega = 2.0 * np.pi / 10.0
    x = torch.linspace(0.0, 2.0, n, dtype=torch.float64, device="cuda")
    y = torch.linspace(0.0, 1.0, n, dtype=torch.float64, device="cuda")
    X, Y = torch.meshgrid(x, y, indexing="ij")
    a = 0.25 * np.sin(omega * t)
    b = 1.0 - 2.0 * a
    f = a * X * X + b * X
    out = xyz[0]
    out[:, :, :, 0] = (-np.pi * 0.1 * torch.sin(np.pi * f) * torch.cos(np.pi * Y)).float()[:, :, None]
    out[:, :, :, 1] = (np.pi * 0.1 * torch.cos(np.pi * f) * torch.sin(np.pi * Y) * (2.0 * a * X + b)).float()[:, :, None]
    out = out.contiguous()
    return out, offset, (spacing * np.float32(n)).astype(np.float32), spacing


def served_stream_config(seed=4, requests=1000, datasets=8, streamline_seed_cap=16384):
    """The served mixed stream: `datasets` resident fields (ABC or a
    double-gyre snapshot, edge log-uniform in [64, 512]) and `requests`
    requests, 70 % streamline / 30 % FTLE, seed counts log-uniform in
    [1k, 2M] (streamline requests capped at streamline_seed_cap, since every
    step of every curve is returned to the host), step counts uniform in
    [200, 2000], Poisson arrivals (unit-rate exponential gaps, scaled by the
    offered rate).  The seed count is met with the smallest lattice stride
    that does not exceed it.  PCG64 from `seed`."""
    rng = np.random.default_rng(seed)
    ds = [{"name": f"field{k}", "kind": "abc" if rng.random() < 0.5 else "gyre",
           "edge": int(np.exp(rng.uniform(np.log(64), np.log(512))))} for k in range(datasets)]
    reqs = []
    for _ in range(requests):
        kind = "streamlines" if rng.random() < 0.7 else "ftle"
        d = int(rng.integers(0, datasets))
        seeds = float(np.exp(rng.uniform(np.log(1000), np.log(2_000_000))))
        if kind == "streamlines":
            seeds = min(seeds, streamline_seed_cap)
        steps = int(rng.integers(200, 2001))
        stride = max(1, int(np.ceil(ds[d]["edge"] / seeds ** (1.0 / 3.0))))
        reqs.append({"kind": kind, "dataset": d, "stride": stride, "steps": steps, "gap": float(rng.exponential())})
    return ds, reqs


def streamline_config():
    """The plain streamline workload: 64^3 ABC, seeds on a stride-4 lattice
    (16^3), RK4 h = 0.01, 1000 steps (remaining_iterations = 1002: seed, at most
    1000 steps, termination vertex; particle_tracer.cpp:266-278)."""
    field = abc_field(64)
    stride = (field.spacing * np.float32(4)).astype(np.float32)
    return {"field": field, "stride": stride, "iterations": 1002, "step": 0.01}


def ftle_config(n=256, noise_sigma=0.01, seed=0):
    """The FTLE workload: n^3 ABC + N(0, 0.01) noise (seed 0), one seed per
    vertex, RK4 h = 0.01 integrated to T = 5 (iterations = 501: at most 500
    steps; particle_advector.cpp:74,132)."""
    field = abc_field(n, noise_sigma=noise_sigma, seed=seed)
    return {"field": field, "iterations": 501, "step": 0.01, "time": 5.0}
