"""ctypes bindings for the oracles (test infrastructure only).

* ``port()`` -> the CPU restatement in ``oracle/pars_oracle.cpp`` (``liboracle.so``),
  built on every machine by ``__graft_entry__.build()``.
* ``reference()`` -> the reference's own hot-path sources compiled against
  ``oracle/ref_shim`` (``oracle/_ref/libpars_ref.so``), available only where the
  reference checkout exists (``oracle/build_ref.sh``); ``None`` elsewhere.

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
module.  The product path never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpars_ref.so")

_P = ctypes.c_void_p
_LL = ctypes.c_longlong
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double

PARTICLE_DTYPE = np.dtype([
    ("position", np.float32, 4),
    ("remaining_iterations", np.int32),
    ("vector_field_index", np.int32),
    ("original_rank", np.int32),
    ("original_voxel", np.int32, 3),
    ("padding", np.int32, 2),
])
assert PARTICLE_DTYPE.itemsize == 48

COLOR_MODES = {"hsl_constant_s": 0, "hsl_constant_l": 1, "hsv_constant_s": 2, "hsv_constant_v": 3, "rgb": 4}


def _ptr(a):
    return None if a is None else a.ctypes.data


class Curves:
    """Batches of integral curves as numpy arrays: list of dicts with
    vertices (n,4) f32, indices (m,) i32, colors (n,4) f32 (NaN = never written),
    rank, round."""

    def __init__(self, batches, steps=None):
        self.batches = batches
        self.steps = steps


class _Lib:
    def __init__(self, path, prefix):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        L = self.lib
        fn = lambda name: getattr(L, prefix + name)
        for name in ("curves_batches",):
            fn(name).restype = _LL
            fn(name).argtypes = [_P]
        for name in ("curves_vertex_count", "curves_index_count"):
            fn(name).restype = _LL
            fn(name).argtypes = [_P, _LL]
        for name in ("curves_vertices", "curves_colors", "curves_indices"):
            fn(name).restype = _P
            fn(name).argtypes = [_P, _LL]
        for name in ("curves_batch_rank", "curves_batch_round"):
            fn(name).restype = _I
            fn(name).argtypes = [_P, _LL]
        fn("curves_free").restype = None
        fn("curves_free").argtypes = [_P]
        fn("field_sample").restype = None
        fn("field_sample").argtypes = [_P] * 5 + [_P, _LL, _P, _P]
        fn("seed_generate").restype = _LL
        fn("seed_generate").argtypes = [_P, _P, _P, _I, _I, _P]
        fn("partition").restype = None
        fn("partition").argtypes = [_I, _I, _P, _P]
        fn("trace_single").restype = _P
        fn("trace_single").argtypes = [_P] * 5 + [_P, _LL, _I, _F, _I, _F]
        fn("trace_multi").restype = _P
        fn("trace_multi").argtypes = [_P, _P, _P, _I, _P, _P, _I, _F, _I, _F]
        fn("index_generate").restype = _LL
        fn("index_generate").argtypes = [_P, _LL, _P]
        fn("color_generate").restype = None
        fn("color_generate").argtypes = [_P, _LL, _P, _LL, _I, _F, _P]

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- curves ---------------------------------------------------------------
    def _collect(self, handle, with_steps=False):
        out = []
        nb = self._f("curves_batches")(handle)
        for b in range(nb):
            nv = self._f("curves_vertex_count")(handle, b)
            ni = self._f("curves_index_count")(handle, b)
            vp = self._f("curves_vertices")(handle, b)
            cp = self._f("curves_colors")(handle, b)
            ip = self._f("curves_indices")(handle, b)
            v = np.ctypeslib.as_array(ctypes.cast(vp, ctypes.POINTER(_F)), (nv * 4,)).reshape(-1, 4).copy() if nv else np.zeros((0, 4), np.float32)
            c = np.ctypeslib.as_array(ctypes.cast(cp, ctypes.POINTER(_F)), (nv * 4,)).reshape(-1, 4).copy() if (nv and cp) else None
            i = np.ctypeslib.as_array(ctypes.cast(ip, ctypes.POINTER(_I)), (ni,)).copy() if ni else np.zeros(0, np.int32)
            out.append({"vertices": v, "colors": c, "indices": i,
                        "rank": self._f("curves_batch_rank")(handle, b),
                        "round": self._f("curves_batch_round")(handle, b)})
        steps = None
        if with_steps:
            steps = int(self.lib.orc_curves_steps(ctypes.c_void_p(handle)))
        self._f("curves_free")(handle)
        return Curves(out, steps)

    # -- stages -----------------------------------------------------------------
    def field_sample(self, field, positions):
        positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        n = positions.shape[0]
        inside = np.zeros(n, np.uint8)
        vel = np.zeros((n, 3), np.float32)
        self._f("field_sample")(*field.ctypes_args(), _ptr(positions), n, _ptr(inside), _ptr(vel))
        return inside.astype(bool), vel

    def seed_generate(self, offset, size, stride, iterations, rank=0):
        o, s, st = (np.ascontiguousarray(a, np.float32) for a in (offset, size, stride))
        n = self._f("seed_generate")(_ptr(o), _ptr(s), _ptr(st), iterations, rank, None)
        out = np.zeros(n, PARTICLE_DTYPE)
        self._f("seed_generate")(_ptr(o), _ptr(s), _ptr(st), iterations, rank, _ptr(out))
        return out

    def partition(self, ranks, rank, domain):
        d = np.ascontiguousarray(domain, np.int32)
        info = np.zeros(21, np.int32)
        self._f("partition")(ranks, rank, _ptr(d), _ptr(info))
        return {"grid": info[0:3].copy(), "block": info[3:6].copy(), "multi_rank": info[6:9].copy(),
                "offset": info[9:12].copy(), "ghosted": info[12:15].copy(), "neighbors": info[15:21].copy()}

    def trace_single(self, field, particles, integrator=2, step=0.01, color="rgb", parameter=0.5):
        particles = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        cm = -1 if color is None else COLOR_MODES[color]
        h = self._f("trace_single")(*field.ctypes_args(), _ptr(particles), len(particles), integrator, step, cm, parameter)
        return self._collect(h, with_steps=(self.prefix == "orc_"))

    def trace_multi(self, domain_field, ranks, seed_offsets, seeds, integrator=2, step=0.01, color="rgb", parameter=0.5):
        seeds = np.ascontiguousarray(seeds, PARTICLE_DTYPE)
        offs = np.ascontiguousarray(seed_offsets, np.int64)
        dims = np.ascontiguousarray(domain_field.dims, np.int32)
        sp = np.ascontiguousarray(domain_field.spacing, np.float32)
        cm = -1 if color is None else COLOR_MODES[color]
        h = self._f("trace_multi")(_ptr(domain_field.xyz), _ptr(dims), _ptr(sp), ranks, _ptr(offs), _ptr(seeds),
                                   integrator, step, cm, parameter)
        return self._collect(h, with_steps=(self.prefix == "orc_"))

    def index_generate(self, vertices):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        out = np.zeros(max(len(v), 1), np.int32)
        n = self._f("index_generate")(_ptr(v), len(v), _ptr(out))
        return out[:n].copy()

    def color_generate(self, vertices, indices, mode="rgb", parameter=0.5):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        i = np.ascontiguousarray(indices, np.int32)
        out = np.zeros_like(v)
        self._f("color_generate")(_ptr(v), len(v), _ptr(i), len(i), COLOR_MODES[mode], parameter, _ptr(out))
        return out


class Port(_Lib):
    """The CPU restatement (liboracle.so)."""

    def __init__(self, path=PORT_PATH):
        super().__init__(path, "orc_")
        L = self.lib
        L.orc_curves_steps.restype = _LL
        L.orc_curves_steps.argtypes = [_P]
        L.orc_max_threads.restype = _I
        L.orc_set_threads.argtypes = [_I]
        L.orc_set_correctly_rounded_trig.argtypes = [_I]
        L.orc_set_correctly_rounded_trig.restype = None
        L.orc_flow_map.restype = _LL
        L.orc_flow_map.argtypes = [_P] * 5 + [_I, _F, _I, _F, _LL, _LL, _LL, _P]
        L.orc_advect_fp64.restype = None
        L.orc_advect_fp64.argtypes = [_P] * 5 + [_P, _LL, _I, _I, _D, _LL, _P, _P, _P, _D, ctypes.c_ulonglong]
        L.orc_ftle_fp64.restype = None
        L.orc_ftle_fp64.argtypes = [_P, _P, _P, _D, _I, _P]
        L.orc_largest_eigenvalue.restype = None
        L.orc_largest_eigenvalue.argtypes = [_P, _LL, _P]
        L.orc_largest_eigenvalue_closed_form.restype = None
        L.orc_largest_eigenvalue_closed_form.argtypes = [_P, _LL, _P]
        L.orc_advect_unsteady_fp64.restype = None
        L.orc_advect_unsteady_fp64.argtypes = [_P, _P, _I, _P, _P, _D, _D, _P, _LL, _D, _D, _LL, _P, _P]
        L.orc_render.restype = _I
        L.orc_render.argtypes = [_P, _P, _P, _LL, _F, _P, _P, _P, _P, _P, _P, _P, _I, _I, _LL, _I, _P, _P]

    def render(self, batches, radius, camera, size, frames=1, volume=None, accum=None, first_frame=0):
        """The ray tracer's image: batches = [(vertices (n,4), colours (n,4) or
        None, indices (m,))], camera = (position, forward, up), size = (width,
        height), volume = (values [X,Y,Z], offset, spacing) or None.  Adds
        `frames` frames to `accum` ([h, w, 4] float32 sums, new when None) and
        returns (rgba [h, w, 4] uint8, accum)."""
        width, height = size
        verts, cols, prims, offset = [], [], [], 0
        for v, c, i in batches:
            v = np.ascontiguousarray(v, np.float32).reshape(-1, 4)
            if len(i) == 0:
                continue
            verts.append(v)
            cols.append(None if c is None else np.ascontiguousarray(c, np.float32).reshape(-1, 4))
            prims.append(offset + np.asarray(i, np.int64))
            offset += len(v)
        vertices = np.concatenate(verts) if verts else np.zeros((1, 4), np.float32)
        colors = np.concatenate(cols) if cols and all(c is not None for c in cols) else None
        prim = np.concatenate(prims) if prims else np.zeros(1, np.int64)
        n = sum(len(p) for p in prims)
        if accum is None:
            accum = np.zeros((height, width, 4), np.float32)
        rgba = np.zeros((height, width, 4), np.uint8)
        vol = vs = vo = vh = None
        if volume is not None:
            vol = np.ascontiguousarray(volume[0], np.float32)
            vs = np.array(vol.shape, np.int32)
            vo = np.ascontiguousarray(volume[1], np.float32)
            vh = np.ascontiguousarray(volume[2], np.float32)
        pos, fwd, up = (np.ascontiguousarray(x, np.float32) for x in camera)
        self.lib.orc_render(_ptr(vertices), _ptr(colors), _ptr(prim), n, radius, _ptr(vol), _ptr(vs), _ptr(vo), _ptr(vh),
                            _ptr(pos), _ptr(fwd), _ptr(up), width, height, first_frame, frames, _ptr(accum), _ptr(rgba))
        return rgba, accum

    def advect_unsteady_fp64(self, xyz, offset, spacing, t0, slice_dt, start, time_begin, step, max_steps):
        """FP64 pathlines (classical RK4 in space-time) on an unsteady field
        xyz [slices, X, Y, Z, 3]."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        dims = np.array(xyz.shape[1:4], np.int32)
        o = np.ascontiguousarray(offset, np.float32)
        sp = np.ascontiguousarray(spacing, np.float32)
        start = np.ascontiguousarray(start, np.float64).reshape(-1, 3)
        end = np.zeros_like(start)
        steps = np.zeros(len(start), np.int64)
        self.lib.orc_advect_unsteady_fp64(_ptr(xyz), _ptr(dims), xyz.shape[0], _ptr(o), _ptr(sp), t0, slice_dt, _ptr(start),
                                          len(start), time_begin, step, max_steps, _ptr(end), _ptr(steps))
        return end, steps

    def max_threads(self):
        return self.lib.orc_max_threads()

    def set_threads(self, n):
        self.lib.orc_set_threads(n)

    def color_generate_correctly_rounded(self, vertices, indices, mode="rgb", parameter=0.5):
        """color_generate with to_spherical's atan2 / acos correctly rounded
        (FP64 rounded to FP32) instead of the host libm's FP32 functions."""
        self.lib.orc_set_correctly_rounded_trig(1)
        try:
            return self.color_generate(vertices, indices, mode, parameter)
        finally:
            self.lib.orc_set_correctly_rounded_trig(0)

    def flow_map(self, field, iterations, scale=1.0, integrator=2, step=0.01, first=0, count=None, stride=1):
        """Frozen-velocity FP32 flow map (reference semantics) of the seeds
        first + k * stride, k < count (default: all from `first`).  Returns
        (flow [X',Y',Z',3] f32 with NaN where no particle landed, steps)."""
        fm = [int(np.float32(d) * np.float32(scale)) for d in field.dims]
        flow = np.full(fm + [3], np.nan, np.float32)
        total = int(np.prod(fm))
        if count is None:
            count = (total - first + stride - 1) // stride
        steps = self.lib.orc_flow_map(*field.ctypes_args(), iterations, scale, integrator, step, first, count, stride,
                                      _ptr(flow))
        return flow, steps

    def advect_fp64(self, field, start, max_steps, integrator=2, mode=1, step=0.01, keep_vertices=False, noise=0.0, seed=0):
        """FP64 advection on the FP32 grid values (mode 1: classical RK4 with
        re-sampled stages).  noise > 0: per-step relative perturbation of that
        size (conditioning ensembles)."""
        start = np.ascontiguousarray(start, np.float64).reshape(-1, 3)
        n = len(start)
        end = np.zeros_like(start)
        steps = np.zeros(n, np.int64)
        verts = np.full((n, max_steps + 1, 3), np.nan) if keep_vertices else None
        self.lib.orc_advect_fp64(*field.ctypes_args(), _ptr(start), n, integrator, mode, step, max_steps,
                                 _ptr(end), _ptr(steps), _ptr(verts), noise, seed)
        return end, steps, verts

    def conditioning(self, field, start, max_steps, integrator=2, step=0.01, noise=6e-8, members=4):
        """Per-particle spread of FP64 end points under per-step relative noise
        `noise` (the size of FP32 rounding): max over `members` runs of the
        distance to the unperturbed FP64 end point, and whether every member
        took the unperturbed step count."""
        clean, steps, _ = self.advect_fp64(field, start, max_steps, integrator, 1, step)
        spread = np.zeros(len(clean))
        same = np.ones(len(clean), bool)
        for m in range(members):
            e, s, _ = self.advect_fp64(field, start, max_steps, integrator, 1, step, noise=noise, seed=m + 1)
            spread = np.maximum(spread, np.linalg.norm(e - clean, axis=1))
            same &= s == steps
        return clean, steps, spread, same

    def ftle_fp64(self, flow, spacing, time, mode=0):
        """mode 0: FTLE; mode 1: fractional anisotropy of C's eigenvalues."""
        flow = np.ascontiguousarray(flow, np.float32)
        dims = np.array(flow.shape[:3], np.int32)
        sp = np.ascontiguousarray(spacing, np.float32)
        out = np.zeros(flow.shape[:3], np.float64)
        self.lib.orc_ftle_fp64(_ptr(flow), _ptr(dims), _ptr(sp), time, mode, _ptr(out))
        return out

    def largest_eigenvalue(self, matrices, closed_form=False):
        m = np.ascontiguousarray(matrices, np.float64).reshape(-1, 9)
        out = np.zeros(len(m))
        fn = self.lib.orc_largest_eigenvalue_closed_form if closed_form else self.lib.orc_largest_eigenvalue
        fn(_ptr(m), len(m), _ptr(out))
        return out


class Reference(_Lib):
    """The reference's own sources built against oracle/ref_shim (libpars_ref.so)."""

    def __init__(self, path=REF_PATH):
        super().__init__(path, "ref_")
        L = self.lib
        L.ref_flow_map.restype = _LL
        L.ref_flow_map.argtypes = [_P] * 5 + [_I, _F, _I, _F, _P, _P]
        L.ref_ftle.restype = None
        L.ref_ftle.argtypes = [_P] * 5 + [_F, _I, _P]

    def flow_map(self, field, iterations, scale=1.0, integrator=2, step=0.01):
        dims = np.zeros(3, np.int32)
        n = self.lib.ref_flow_map(*field.ctypes_args(), iterations, scale, integrator, step, None, _ptr(dims))
        flow = np.zeros(list(dims) + [3], np.float32)
        self.lib.ref_flow_map(*field.ctypes_args(), iterations, scale, integrator, step, _ptr(flow), _ptr(dims))
        return flow


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            raise RuntimeError("oracle/liboracle.so is not built; run __graft_entry__.build()")
        _port = Port()
    return _port


def reference():
    """The reference build, or None where the reference sources were not available."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = Reference()
    return _ref
