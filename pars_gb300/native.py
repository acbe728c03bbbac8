"""ctypes binding of libpars_gpu.so (include/pars_gpu.h).

The product path: every call goes to the sm_103a library.  There is no CPU
fallback — importing works without a GPU, but using a Context requires the
built library and a CUDA device, and fails loudly otherwise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(HERE, "libpars_gpu.so")

PARTICLE_DTYPE = np.dtype([
    ("position", np.float32, 4),
    ("remaining_iterations", np.int32),
    ("vector_field_index", np.int32),
    ("original_rank", np.int32),
    ("original_voxel", np.int32, 3),
    ("padding", np.int32, 2),
])
assert PARTICLE_DTYPE.itemsize == 48

# enum values of include/pars_gpu.h
EULER, MODIFIED_MIDPOINT, RUNGE_KUTTA_4 = 0, 1, 2
INTEGRATORS = {"euler": 0, "modified_midpoint": 1, "runge_kutta_4": 2, "runge_kutta_cash_karp_54": 3,
               "runge_kutta_dormand_prince_5": 4, "runge_kutta_fehlberg_78": 5, "adams_bashforth_2": 6,
               "adams_bashforth_moulton_2": 7}
STAGES_FROZEN, STAGES_RESAMPLED = 0, 1
COLOR_MODES = {"hsl_constant_s": 0, "hsl_constant_l": 1, "hsv_constant_s": 2, "hsv_constant_v": 3, "rgb": 4}
FTLE_REGULAR, FTLE_FRACTIONAL_ANISOTROPY = 0, 1
STATUS = {0: "ok", -1: "invalid argument", -2: "cuda error", -3: "out of memory", -4: "unsupported",
          -5: "not found", -6: "over budget", -7: "cancelled", -8: "timeout", -9: "bad state"}


class PartitionInfo(ctypes.Structure):
    _fields_ = [("grid_size", ctypes.c_int32 * 3), ("block_size", ctypes.c_int32 * 3),
                ("multi_rank", ctypes.c_int32 * 3), ("offset", ctypes.c_int32 * 3),
                ("ghosted_block_size", ctypes.c_int32 * 3), ("neighbor_rank", ctypes.c_int32 * 6)]


class TraceSummary(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_int64), ("vertices", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("rounds", ctypes.c_int32), ("padding", ctypes.c_int32)]


class BatchJob(ctypes.Structure):
    """pars_gpu_batch_job (include/pars_gpu.h)."""
    _fields_ = [("field", ctypes.c_int32), ("integrator", ctypes.c_int32), ("stage_mode", ctypes.c_int32),
                ("max_steps", ctypes.c_int32), ("step_size", ctypes.c_float), ("padding0", ctypes.c_int32),
                ("time_begin", ctypes.c_double), ("seeds", ctypes.c_void_p), ("seed_count", ctypes.c_int64),
                ("lattice_offset", ctypes.c_float * 3), ("lattice_stride", ctypes.c_float * 3),
                ("lattice_count", ctypes.c_int32 * 3), ("padding1", ctypes.c_int32),
                ("end_positions", ctypes.c_void_p), ("end_steps", ctypes.c_void_p), ("steps", ctypes.c_int64)]


class EngineDone(ctypes.Structure):
    """pars_gpu_engine_done (include/pars_gpu.h)."""
    _fields_ = [("ticket", ctypes.c_int64), ("steps", ctypes.c_int64)]


class SettingsSummary(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_char * 64), ("dataset_filepath", ctypes.c_char * 256),
                ("particle_tracing_integrator", ctypes.c_char * 64), ("color_generation_mode", ctypes.c_char * 64),
                ("seed_generation_stride", ctypes.c_int32 * 3), ("seed_generation_iterations", ctypes.c_int32),
                ("particle_tracing_step_size", ctypes.c_float), ("particle_tracing_load_balance", ctypes.c_int32),
                ("color_generation_free_parameter", ctypes.c_float), ("raytracing_camera_position", ctypes.c_float * 3),
                ("raytracing_image_size", ctypes.c_int32 * 2), ("raytracing_streamline_radius", ctypes.c_float),
                ("raytracing_iterations", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("ftle_shape", ctypes.c_int32 * 3), ("batches", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("image_size", ctypes.c_int32 * 2)]


class ParsGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)} ({status}): {message}")
        self.status = status


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F = ctypes.c_float

# name -> argtypes (all return int32 status unless listed in _RESTYPES)
SIGNATURES = {
    "pars_gpu_create": [ctypes.POINTER(_P), _I32],
    "pars_gpu_destroy": [_P],
    "pars_gpu_last_error": [_P],
    "pars_gpu_abi_version": [],
    "pars_gpu_set_stream": [_P, _P],
    "pars_gpu_synchronize": [_P],
    "pars_gpu_memory_in_use": [_P, ctypes.POINTER(_I64)],
    "pars_gpu_field_upload": [_P, _P, _P, _P, _P, _P, ctypes.POINTER(_I32)],
    "pars_gpu_field_upload_device": [_P, _P, _P, _P, _P, _P, ctypes.POINTER(_I32)],
    "pars_gpu_field_release": [_P, _I32],
    "pars_gpu_field_info": [_P, _I32, _P, _P, _P, _P],
    "pars_gpu_field_download": [_P, _I32, _P],
    "pars_gpu_field_sample": [_P, _I32, _P, _I64, _P, _P],
    "pars_gpu_seed_generate": [_P, _P, _P, _P, _I32, _I32, _P, _I64, ctypes.POINTER(_I64)],
    "pars_gpu_partition": [_I32, _I32, _P, ctypes.POINTER(PartitionInfo)],
    "pars_gpu_trace": [_P, _I32, _P, _I64, _I32, _I32, _F, ctypes.POINTER(TraceSummary)],
    "pars_gpu_trace_device": [_P, _I32, _P, _I64, _I32, _I32, _F, ctypes.POINTER(TraceSummary)],
    "pars_gpu_domain_create": [_P, _P, _P, _P, _I32, ctypes.POINTER(_I32)],
    "pars_gpu_domain_release": [_P, _I32],
    "pars_gpu_domain_create_device": [_P, _P, _P, _P, _I32, ctypes.POINTER(_I32)],
    "pars_gpu_trace_domain": [_P, _I32, _P, _P, _I32, _I32, _F, ctypes.POINTER(TraceSummary)],
    "pars_gpu_domain_assemble": [_P, _I32, _P, _P, ctypes.POINTER(_I32)],
    "pars_gpu_round_trace": [_P, _I32, _I32, _P, _P, _I32, _I32, _F, _P, ctypes.POINTER(TraceSummary)],
    "pars_gpu_round_particles": [_P, _P],
    "pars_gpu_curves_index": [_P],
    "pars_gpu_curves_color": [_P, _I32, _F],
    "pars_gpu_curves_batch_info": [_P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I32), ctypes.POINTER(_I32)],
    "pars_gpu_curves_download": [_P, _I64, _P, _P, _P],
    "pars_gpu_index_generate": [_P, _P, _I64, _P, ctypes.POINTER(_I64)],
    "pars_gpu_color_generate": [_P, _P, _I64, _P, _I64, _I32, _F, _P],
    "pars_gpu_flow_map_generate": [_P, _I32, _I32, _F, _I32, _I32, _F, ctypes.POINTER(_I32), ctypes.POINTER(_I64)],
    "pars_gpu_ftle_generate": [_P, _I32, _F, _I32, _P],
    "pars_gpu_ftle_device_pointer": [_P, ctypes.POINTER(_P), ctypes.POINTER(_I64)],
    "pars_gpu_ftle_no_alloc": [_P, _P, _P, _P, _P, _I32, _I32, _I32, _F, _F, _I32, _P, _P, _P],
    "pars_gpu_unsteady_field_upload": [_P, _P, _P, _I32, _P, _P, _P, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_I32)],
    "pars_gpu_unsteady_field_upload_device": [_P, _P, _P, _I32, _P, _P, _P, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_I32)],
    "pars_gpu_batch_advect": [_P, _P, _I32, _I32],
    "pars_gpu_batch_variants": [_P, ctypes.POINTER(_I32)],
    "pars_gpu_batch_tuned": [_P, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)],
    "pars_gpu_engine_submit": [_P, ctypes.POINTER(BatchJob), ctypes.POINTER(_I64)],
    "pars_gpu_engine_advance": [_P, _I32, ctypes.POINTER(EngineDone), _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I64)],
    "pars_gpu_settings_decode": [_P, _I64, ctypes.POINTER(SettingsSummary)],
    "pars_gpu_settings_from_json": [ctypes.c_char_p, _I64, _P, _I64, ctypes.POINTER(_I64)],
    "pars_gpu_service_create": [ctypes.POINTER(_P), _I32, _I64, _I32, _I32],
    "pars_gpu_service_destroy": [_P],
    "pars_gpu_service_set_horizon": [_P, _I32],
    "pars_gpu_service_add_dataset": [_P, ctypes.c_char_p, _P, _P, _P, _P, _P],
    "pars_gpu_service_add_dataset_device": [_P, ctypes.c_char_p, _P, _P, _P, _P, _P],
    "pars_gpu_service_submit": [_P, _P, _I64, ctypes.POINTER(_I64)],
    "pars_gpu_service_wait": [_P, _I64, _I32, ctypes.POINTER(_I32)],
    "pars_gpu_service_result_info": [_P, _I64, ctypes.POINTER(RequestInfo)],
    "pars_gpu_service_result_batch": [_P, _I64, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_I64), _P, _P, _P],
    "pars_gpu_service_result_ftle": [_P, _I64, _P],
    "pars_gpu_service_release": [_P, _I64],
    "pars_gpu_service_add_volume": [_P, ctypes.c_char_p, _P, _P, _P, _P],
    "pars_gpu_service_add_volume_device": [_P, ctypes.c_char_p, _P, _P, _P, _P],
    "pars_gpu_service_result_image": [_P, _I64, _P, _P],
    "pars_gpu_service_profile_enable": [_P, _I32],
    "pars_gpu_service_profile_get": [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64)],
    "pars_gpu_raw_info": [ctypes.c_char_p, ctypes.POINTER(_I32), _P, _P],
    "pars_gpu_raw_write": [ctypes.c_char_p, _I32, _P, _P, _P],
    "pars_gpu_field_load": [_P, ctypes.c_char_p, _I32, _I32, ctypes.POINTER(_I32), ctypes.POINTER(PartitionInfo)],
    "pars_gpu_scalar_load": [ctypes.c_char_p, _I32, _I32, _P, _P, _P, _P, _P],
    "pars_gpu_ftle_save": [ctypes.c_char_p, _P, _P, _P, _P, _P],
    "pars_gpu_export_vtk": [ctypes.c_char_p, _I64, _P, _P, _P],
    "pars_gpu_curves_export_vtk": [_P, ctypes.c_char_p],
    "pars_gpu_ray_tracer_set_volume": [_P, _P, _P, _P, _P],
    "pars_gpu_ray_tracer_set_volume_device": [_P, _P, _P, _P, _P],
    "pars_gpu_ray_tracer_clear_volume": [_P],
    "pars_gpu_ray_tracer_set_integral_curves": [_P, _F],
    "pars_gpu_ray_tracer_set_integral_curves_host": [_P, _I64, _P, _P, _P, _P, _P, _F],
    "pars_gpu_ray_tracer_set_camera": [_P, _P, _P, _P],
    "pars_gpu_ray_tracer_set_image_size": [_P, _I32, _I32],
    "pars_gpu_ray_tracer_trace": [_P, _I32],
    "pars_gpu_ray_tracer_serialize": [_P, _P, _P],
    "pars_gpu_ray_tracer_frames": [_P, ctypes.POINTER(_I64)],
    "pars_gpu_image_encode": [_P, _P, _I64, _P, _I64, ctypes.POINTER(_I64)],
    "pars_gpu_profile_enable": [_P, _I32],
    "pars_gpu_profile_reset": [_P],
    "pars_gpu_profile_get": [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64)],
    "pars_gpu_launch_count": [_P, ctypes.POINTER(_I64)],
    "pars_gpu_gather_peak": [_P, _I64, _I32, ctypes.POINTER(ctypes.c_double)],
    "pars_gpu_transport_listen": [ctypes.c_char_p, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I64)],
    "pars_gpu_transport_close": [_I64],
    "pars_gpu_service_serve": [_P, _I64, _I64, ctypes.POINTER(_I64)],
}
_RESTYPES = {"pars_gpu_last_error": ctypes.c_char_p}

_lib = None


def library():
    """Loads libpars_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBRARY_PATH):
            raise RuntimeError(f"{LIBRARY_PATH} is missing: build it with pars_gb300.build.build()")
        lib = ctypes.CDLL(LIBRARY_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, _I32)
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))


def _i3(v):
    return np.ascontiguousarray(np.asarray(v, np.int32).reshape(3))


def partition(ranks, rank, domain_size):
    """partitioner::set_domain_size as seen from `rank` (no context needed)."""
    info = PartitionInfo()
    d = _i3(domain_size)
    status = library().pars_gpu_partition(ranks, rank, _ptr(d), ctypes.byref(info))
    if status:
        raise ParsGpuError(status, "pars_gpu_partition")
    return {"grid": np.array(info.grid_size), "block": np.array(info.block_size),
            "multi_rank": np.array(info.multi_rank), "offset": np.array(info.offset),
            "ghosted": np.array(info.ghosted_block_size), "neighbors": np.array(info.neighbor_rank)}


class Context:
    """One pars_gpu context (device memory, stream, resident fields/curves)."""

    def __init__(self, device=0):
        self.lib = library()
        handle = _P()
        self._check(self.lib.pars_gpu_create(ctypes.byref(handle), device), "pars_gpu_create", use_context=False)
        self.handle = handle

    # -- plumbing -------------------------------------------------------------
    def _check(self, status, what, use_context=True):
        if status:
            message = what
            if use_context and getattr(self, "handle", None):
                message += ": " + self.lib.pars_gpu_last_error(self.handle).decode()
            raise ParsGpuError(status, message)

    def _call(self, name, *args):
        self._check(getattr(self.lib, name)(self.handle, *args), name)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pars_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr):
        self._call("pars_gpu_set_stream", stream_ptr)

    def synchronize(self):
        self._call("pars_gpu_synchronize")

    def memory_in_use(self):
        v = _I64()
        self._call("pars_gpu_memory_in_use", ctypes.byref(v))
        return v.value

    # -- fields ------------------------------------------------------------------
    def upload_field(self, field):
        h = _I32()
        self._call("pars_gpu_field_upload", _ptr(field.xyz), _ptr(field.dims), _ptr(field.offset), _ptr(field.size),
                   _ptr(field.spacing), ctypes.byref(h))
        return h.value

    def upload_field_host(self, host_xyz_ptr, dims, offset, size, spacing):
        """pars_gpu_field_upload from a host address (e.g. a pinned buffer)."""
        h = _I32()
        d, o, s, sp = _i3(dims), _f3(offset), _f3(size), _f3(spacing)
        self._call("pars_gpu_field_upload", host_xyz_ptr, _ptr(d), _ptr(o), _ptr(s), _ptr(sp), ctypes.byref(h))
        return h.value

    def upload_field_device(self, device_xyz_ptr, dims, offset, size, spacing):
        h = _I32()
        d, o, s, sp = _i3(dims), _f3(offset), _f3(size), _f3(spacing)
        self._call("pars_gpu_field_upload_device", device_xyz_ptr, _ptr(d), _ptr(o), _ptr(s), _ptr(sp), ctypes.byref(h))
        return h.value

    def release_field(self, handle):
        self._call("pars_gpu_field_release", handle)

    def field_info(self, handle):
        shape = np.zeros(3, np.int32)
        offset, size, spacing = (np.zeros(3, np.float32) for _ in range(3))
        self._call("pars_gpu_field_info", handle, _ptr(shape), _ptr(offset), _ptr(size), _ptr(spacing))
        return {"shape": shape, "offset": offset, "size": size, "spacing": spacing}

    def download_field(self, handle):
        shape = self.field_info(handle)["shape"]
        out = np.zeros(list(shape) + [3], np.float32)
        self._call("pars_gpu_field_download", handle, _ptr(out))
        return out

    def sample(self, field, positions):
        p = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        inside = np.zeros(len(p), np.uint8)
        vel = np.zeros((len(p), 3), np.float32)
        self._call("pars_gpu_field_sample", field, _ptr(p), len(p), _ptr(inside), _ptr(vel))
        return inside.astype(bool), vel

    # -- seeds -----------------------------------------------------------------------
    def seed_generate(self, offset, size, stride, iterations, rank=0):
        o, s, st = _f3(offset), _f3(size), _f3(stride)
        n = _I64()
        self._call("pars_gpu_seed_generate", _ptr(o), _ptr(s), _ptr(st), iterations, rank, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, PARTICLE_DTYPE)
        if n.value:
            self._call("pars_gpu_seed_generate", _ptr(o), _ptr(s), _ptr(st), iterations, rank, _ptr(out), n.value, ctypes.byref(n))
        return out

    # -- tracing ---------------------------------------------------------------------
    def trace(self, field, particles, integrator=RUNGE_KUTTA_4, stage_mode=STAGES_FROZEN, step=0.01):
        particles = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        s = TraceSummary()
        self._call("pars_gpu_trace", field, _ptr(particles), len(particles), integrator, stage_mode, step, ctypes.byref(s))
        return {"batches": s.batches, "vertices": s.vertices, "steps": s.steps, "rounds": s.rounds}

    def trace_device(self, field, device_ptr, count, integrator=RUNGE_KUTTA_4, stage_mode=STAGES_FROZEN, step=0.01):
        s = TraceSummary()
        self._call("pars_gpu_trace_device", field, device_ptr, count, integrator, stage_mode, step, ctypes.byref(s))
        return {"batches": s.batches, "vertices": s.vertices, "steps": s.steps, "rounds": s.rounds}

    def domain_create(self, field, ranks):
        h = _I32()
        self._call("pars_gpu_domain_create", _ptr(field.xyz), _ptr(field.dims), _ptr(field.spacing), ranks, ctypes.byref(h))
        return h.value

    def domain_create_device(self, device_ptr, dims, spacing, ranks):
        h = _I32()
        d, sp = _i3(dims), _f3(spacing)
        self._call("pars_gpu_domain_create_device", device_ptr, _ptr(d), _ptr(sp), ranks, ctypes.byref(h))
        return h.value

    def domain_release(self, handle):
        self._call("pars_gpu_domain_release", handle)

    def trace_domain(self, domain, particles, seed_offsets, integrator=RUNGE_KUTTA_4, stage_mode=STAGES_FROZEN, step=0.01):
        particles = np.ascontiguousarray(particles, PARTICLE_DTYPE)
        offs = np.ascontiguousarray(seed_offsets, np.int64)
        s = TraceSummary()
        self._call("pars_gpu_trace_domain", domain, _ptr(particles), _ptr(offs), integrator, stage_mode, step, ctypes.byref(s))
        return {"batches": s.batches, "vertices": s.vertices, "steps": s.steps, "rounds": s.rounds}

    def domain_assemble(self, ranks, domain_size, fields):
        """A domain from per-rank block fields (pars_gpu_domain_assemble)."""
        h = _I32()
        d = _i3(domain_size)
        f = np.ascontiguousarray(fields, np.int32)
        self._call("pars_gpu_domain_assemble", ranks, _ptr(d), _ptr(f), ctypes.byref(h))
        return h.value

    def round_trace(self, domain, round_index, particles, offsets, ranks, integrator=RUNGE_KUTTA_4, stage_mode=STAGES_FROZEN,
                    step=0.01):
        """One round of every rank (pars_gpu_round_trace).  particles None: the
        device-resident particles of the previous round.  Returns (summary,
        next_offsets)."""
        s = TraceSummary()
        nxt = np.zeros(ranks + 1, np.int64)
        if particles is None:
            p, o = None, None
        else:
            particles = np.ascontiguousarray(particles, PARTICLE_DTYPE)
            offsets = np.ascontiguousarray(offsets, np.int64)
            p, o = _ptr(particles), _ptr(offsets)
        self._call("pars_gpu_round_trace", domain, round_index, p, o, integrator, stage_mode, step, _ptr(nxt), ctypes.byref(s))
        return {"batches": s.batches, "vertices": s.vertices, "steps": s.steps, "rounds": s.rounds}, nxt

    def round_particles(self, count):
        out = np.zeros(max(count, 1), PARTICLE_DTYPE)
        self._call("pars_gpu_round_particles", _ptr(out))
        return out[:count]

    def curves_index(self):
        self._call("pars_gpu_curves_index")

    def curves_color(self, mode="rgb", parameter=0.5):
        self._call("pars_gpu_curves_color", COLOR_MODES[mode] if isinstance(mode, str) else mode, parameter)

    def batch_info(self, b):
        nv, ni, r, rd = _I64(), _I64(), _I32(), _I32()
        self._call("pars_gpu_curves_batch_info", b, ctypes.byref(nv), ctypes.byref(ni), ctypes.byref(r), ctypes.byref(rd))
        return nv.value, ni.value, r.value, rd.value

    def curves(self, batches, vertices=True, colors=False, indices=False):
        """Downloads `batches` batches as dicts of numpy arrays."""
        out = []
        for b in range(batches):
            nv, ni, rank, rnd = self.batch_info(b)
            v = np.zeros((nv, 4), np.float32) if vertices else None
            c = np.zeros((nv, 4), np.float32) if colors else None
            i = np.zeros(ni, np.int32) if indices else None
            self._call("pars_gpu_curves_download", b, _ptr(v), _ptr(c), _ptr(i))
            out.append({"vertices": v, "colors": c, "indices": i, "rank": rank, "round": rnd})
        return out

    def index_generate(self, vertices):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        out = np.zeros(max(len(v), 1), np.int32)
        n = _I64()
        self._call("pars_gpu_index_generate", _ptr(v), len(v), _ptr(out), ctypes.byref(n))
        return out[: n.value].copy()

    def color_generate(self, vertices, indices, mode="rgb", parameter=0.5, colors=None):
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 4)
        i = np.ascontiguousarray(indices, np.int32)
        c = np.zeros_like(v) if colors is None else np.ascontiguousarray(colors, np.float32).reshape(-1, 4).copy()
        self._call("pars_gpu_color_generate", _ptr(v), len(v), _ptr(i), len(i),
                   COLOR_MODES[mode] if isinstance(mode, str) else mode, parameter, _ptr(c))
        return c

    # -- flow map / FTLE ------------------------------------------------------------------
    def flow_map_generate(self, field, iterations, scale=1.0, integrator=RUNGE_KUTTA_4, stage_mode=STAGES_RESAMPLED, step=0.01):
        h, steps = _I32(), _I64()
        self._call("pars_gpu_flow_map_generate", field, iterations, scale, integrator, stage_mode, step, ctypes.byref(h), ctypes.byref(steps))
        return h.value, steps.value

    def ftle_generate(self, flow_map, time, mode=FTLE_REGULAR, shape=None, download=True, out=None):
        """FTLE of a resident flow map; downloads into `out` (or a new array of
        `shape`) unless download is False."""
        if download and out is None:
            out = np.zeros(shape, np.float32)
        if not download:
            out = None
        self._call("pars_gpu_ftle_generate", flow_map, time, mode, _ptr(out))
        return out

    def ftle_device_pointer(self):
        p, n = _P(), _I64()
        self._call("pars_gpu_ftle_device_pointer", ctypes.byref(p), ctypes.byref(n))
        return p.value, n.value

    # -- unsteady fields / batched advection -------------------------------------------
    def upload_unsteady_field(self, xyz, offset, spacing, t0, slice_dt, size=None):
        """xyz: [slices, X, Y, Z, 3] FP32 host array."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        dims = np.array(xyz.shape[1:4], np.int32)
        o, sp = _f3(offset), _f3(spacing)
        s = _f3(size) if size is not None else (dims.astype(np.float32) * sp).astype(np.float32)
        h = _I32()
        self._call("pars_gpu_unsteady_field_upload", _ptr(xyz), _ptr(dims), xyz.shape[0], _ptr(o), _ptr(s), _ptr(sp),
                   t0, slice_dt, ctypes.byref(h))
        return h.value

    def upload_unsteady_field_device(self, device_ptr, dims, slices, offset, size, spacing, t0, slice_dt):
        h = _I32()
        d, o, s, sp = _i3(dims), _f3(offset), _f3(size), _f3(spacing)
        self._call("pars_gpu_unsteady_field_upload_device", device_ptr, _ptr(d), slices, _ptr(o), _ptr(s), _ptr(sp),
                   t0, slice_dt, ctypes.byref(h))
        return h.value

    def batch_advect(self, jobs, variant=-1):
        """jobs: list of BatchJob; returns the per-job step counts."""
        arr = (BatchJob * len(jobs))(*jobs)
        self._call("pars_gpu_batch_advect", ctypes.cast(arr, ctypes.c_void_p), len(jobs), variant)
        return [arr[i].steps for i in range(len(jobs))]

    def engine_submit(self, job):
        """Appends a BatchJob to the continuous engine; returns its ticket."""
        t = _I64()
        self._call("pars_gpu_engine_submit", ctypes.byref(job), ctypes.byref(t))
        return t.value

    def engine_advance(self, iterations, capacity=1024):
        """One horizon launch per job class with work (iterations 0: chosen by
        the engine for launches of about 2 ms); returns ([(ticket, steps) of the
        jobs completed], jobs still open)."""
        done = (EngineDone * max(1, capacity))()
        n, left = _I32(), _I64()
        self._call("pars_gpu_engine_advance", iterations, done, capacity, ctypes.byref(n), ctypes.byref(left))
        return [(done[i].ticket, done[i].steps) for i in range(n.value)], left.value

    def batch_tuned(self, job_class):
        v, t = _I32(), _I32()
        self._call("pars_gpu_batch_tuned", job_class, ctypes.byref(v), ctypes.byref(t))
        return v.value, t.value

    def curves_export_vtk(self, path):
        """The context's curves as VTK XML PolyData (data_io::save_integral_curves)."""
        self._call("pars_gpu_curves_export_vtk", os.fsencode(path))

    # -- field files -----------------------------------------------------------------
    def field_load(self, path, ranks=1, rank=0):
        """Loads a rank's ghosted block of a vector field file; returns (handle, partition dict)."""
        h, info = _I32(), PartitionInfo()
        self._call("pars_gpu_field_load", os.fsencode(path), ranks, rank, ctypes.byref(h), ctypes.byref(info))
        return h.value, {"grid": np.array(info.grid_size), "block": np.array(info.block_size), "offset": np.array(info.offset),
                         "ghosted": np.array(info.ghosted_block_size), "neighbors": np.array(info.neighbor_rank)}

    # -- ray tracer (pars::ray_tracer) -------------------------------------------------
    def ray_tracer_set_volume(self, values, offset, spacing):
        """values: [X, Y, Z] FP32 host array."""
        v = np.ascontiguousarray(values, np.float32)
        s, o, sp = _i3(v.shape), _f3(offset), _f3(spacing)     # kept alive across the call
        self._call("pars_gpu_ray_tracer_set_volume", _ptr(v), _ptr(s), _ptr(o), _ptr(sp))

    def ray_tracer_set_volume_device(self, device_ptr, shape, offset, spacing):
        s, o, sp = _i3(shape), _f3(offset), _f3(spacing)
        self._call("pars_gpu_ray_tracer_set_volume_device", device_ptr, _ptr(s), _ptr(o), _ptr(sp))

    def ray_tracer_clear_volume(self):
        self._call("pars_gpu_ray_tracer_clear_volume")

    def ray_tracer_set_integral_curves(self, radius):
        """The context's device-resident curves (indexed, optionally coloured)."""
        self._call("pars_gpu_ray_tracer_set_integral_curves", radius)

    def ray_tracer_set_integral_curves_host(self, batches, radius):
        """batches: list of (vertices (n,4), colours (n,4) or None, indices (m,))."""
        keep = [(np.ascontiguousarray(v, np.float32).reshape(-1, 4),
                 None if c is None else np.ascontiguousarray(c, np.float32).reshape(-1, 4),
                 np.ascontiguousarray(i, np.int32)) for v, c, i in batches]
        n = len(keep)
        vc = np.array([len(v) for v, _, _ in keep] or [0], np.int64)
        ic = np.array([len(i) for _, _, i in keep] or [0], np.int64)
        vp = (_P * max(n, 1))(*[v.ctypes.data for v, _, _ in keep])
        with_colors = n > 0 and all(c is not None for _, c, _ in keep)
        cp = (_P * max(n, 1))(*[c.ctypes.data for _, c, _ in keep]) if with_colors else None
        ip = (_P * max(n, 1))(*[i.ctypes.data if len(i) else None for _, _, i in keep])
        self._call("pars_gpu_ray_tracer_set_integral_curves_host", n, _ptr(vc), ctypes.cast(vp, _P),
                   ctypes.cast(cp, _P) if cp is not None else None, _ptr(ic), ctypes.cast(ip, _P), radius)

    def ray_tracer_set_camera(self, position, forward, up):
        p, f, u = _f3(position), _f3(forward), _f3(up)          # kept alive across the call
        self._call("pars_gpu_ray_tracer_set_camera", _ptr(p), _ptr(f), _ptr(u))

    def ray_tracer_set_image_size(self, width, height):
        self._call("pars_gpu_ray_tracer_set_image_size", width, height)

    def ray_tracer_trace(self, iterations=1):
        self._call("pars_gpu_ray_tracer_trace", iterations)

    def ray_tracer_serialize(self, out=None):
        """The image as a [height, width, 4] uint8 array (sRGB RGBA8, rows from
        the top), into `out` when given (a C-contiguous array of that shape)."""
        size = np.zeros(2, np.int32)
        self._call("pars_gpu_ray_tracer_serialize", None, _ptr(size))
        if out is None:
            out = np.zeros((size[1], size[0], 4), np.uint8)
        if out.shape != (size[1], size[0], 4) or out.dtype != np.uint8 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous uint8 array of shape (height, width, 4)")
        self._call("pars_gpu_ray_tracer_serialize", _ptr(out), _ptr(size))
        return out

    def ray_tracer_frames(self):
        n = _I64()
        self._call("pars_gpu_ray_tracer_frames", ctypes.byref(n))
        return n.value

    # -- instrumentation ----------------------------------------------------------------
    def profile_enable(self, on=True):
        self._call("pars_gpu_profile_enable", 1 if on else 0)

    def profile_reset(self):
        self._call("pars_gpu_profile_reset")

    def profile_get(self, name):
        ms, n = ctypes.c_double(), _I64()
        self._call("pars_gpu_profile_get", name.encode(), ctypes.byref(ms), ctypes.byref(n))
        return ms.value, n.value

    def launch_count(self):
        n = _I64()
        self._call("pars_gpu_launch_count", ctypes.byref(n))
        return n.value

    GATHER_PATTERNS = {"coalesced": 0, "random": 1, "cells": 2}

    def gather_peak(self, buffer_bytes, pattern):
        """Measured gather bandwidth (bytes/s) of 16-byte loads into a buffer
        of buffer_bytes; pattern "coalesced", "random" or "cells"."""
        out = ctypes.c_double()
        self._call("pars_gpu_gather_peak", int(buffer_bytes), self.GATHER_PATTERNS[pattern], ctypes.byref(out))
        return out.value


# -- the service's transport -----------------------------------------------------------
def transport_listen(address="127.0.0.1", port=0):
    """A TCP listener for pars_gpu_service_serve; returns (listener, port)."""
    lib = library()
    bound, handle = _I32(), _I64()
    status = lib.pars_gpu_transport_listen(address.encode(), port, ctypes.byref(bound), ctypes.byref(handle))
    if status:
        raise ParsGpuError(status, "pars_gpu_transport_listen")
    return handle.value, bound.value


def transport_close(listener):
    status = library().pars_gpu_transport_close(listener)
    if status:
        raise ParsGpuError(status, "pars_gpu_transport_close")


# -- field files (pa::data_io) ----------------------------------------------------------
def raw_write(path, data, spacing):
    """Writes a dataset: data [X, Y, Z, 3] (vector field) or [X, Y, Z] (scalar)."""
    data = np.ascontiguousarray(data, np.float32)
    components = 3 if data.ndim == 4 else 1
    shape = np.array(data.shape[:3], np.int64)
    sp = _f3(spacing)
    status = library().pars_gpu_raw_write(os.fsencode(path), components, _ptr(shape), _ptr(sp), _ptr(data))
    if status:
        raise ParsGpuError(status, "pars_gpu_raw_write")


def raw_info(path):
    """(components, shape, raw spacing) of a field file."""
    c, shape, sp = _I32(), np.zeros(3, np.int64), np.zeros(3, np.float32)
    status = library().pars_gpu_raw_info(os.fsencode(path), ctypes.byref(c), _ptr(shape), _ptr(sp))
    if status:
        raise ParsGpuError(status, "pars_gpu_raw_info")
    return c.value, tuple(int(x) for x in shape), sp


def scalar_load(path, ranks=1, rank=0):
    """A rank's ghosted block of a scalar field file: (values [X, Y, Z], offset, spacing, size)."""
    lib = library()
    shape, o, sp, sz = np.zeros(3, np.int32), np.zeros(3, np.float32), np.zeros(3, np.float32), np.zeros(3, np.float32)
    status = lib.pars_gpu_scalar_load(os.fsencode(path), ranks, rank, None, _ptr(shape), _ptr(o), _ptr(sp), _ptr(sz))
    if status:
        raise ParsGpuError(status, "pars_gpu_scalar_load")
    values = np.zeros(tuple(shape), np.float32)
    status = lib.pars_gpu_scalar_load(os.fsencode(path), ranks, rank, _ptr(values), _ptr(shape), _ptr(o), _ptr(sp), _ptr(sz))
    if status:
        raise ParsGpuError(status, "pars_gpu_scalar_load")
    return values, o, sp, sz


def ftle_save(path, domain, offset, values, spacing=(1.0, 1.0, 1.0)):
    """Writes a block of FTLE values at voxel `offset` into the file of the whole `domain`."""
    values = np.ascontiguousarray(values, np.float32)
    d, o, s, sp = _i3(domain), _i3(offset), _i3(values.shape), _f3(spacing)
    status = library().pars_gpu_ftle_save(os.fsencode(path), _ptr(d), _ptr(o), _ptr(s), _ptr(values), _ptr(sp))
    if status:
        raise ParsGpuError(status, "pars_gpu_ftle_save")


def export_vtk(path, batches):
    """Writes curves (a list of (vertices (n,4), colours (n,4) or None)) as VTK
    XML PolyData, as data_io::save_integral_curves assembles them."""
    keep = [(np.ascontiguousarray(v, np.float32).reshape(-1, 4),
             None if c is None else np.ascontiguousarray(c, np.float32).reshape(-1, 4)) for v, c in batches]
    n = len(keep)
    counts = np.array([len(v) for v, _ in keep] or [0], np.int64)
    vp = (_P * max(n, 1))(*[v.ctypes.data for v, _ in keep])
    cp = (_P * max(n, 1))(*[None if c is None else c.ctypes.data for _, c in keep])
    status = library().pars_gpu_export_vtk(os.fsencode(path), n, _ptr(counts), ctypes.cast(vp, _P), ctypes.cast(cp, _P))
    if status:
        raise ParsGpuError(status, "pars_gpu_export_vtk")


def image_encode(rgba):
    """The `image` message (pars/proto/image.proto) of a [height, width, 4] uint8 image."""
    lib = library()
    rgba = np.ascontiguousarray(rgba, np.uint8)
    size = np.array([rgba.shape[1], rgba.shape[0]], np.int32)
    n = _I64()
    status = lib.pars_gpu_image_encode(_ptr(size), _ptr(rgba), rgba.size, None, 0, ctypes.byref(n))
    if status:
        raise ParsGpuError(status, "pars_gpu_image_encode")
    out = np.zeros(n.value, np.uint8)
    status = lib.pars_gpu_image_encode(_ptr(size), _ptr(rgba), rgba.size, _ptr(out), n.value, ctypes.byref(n))
    if status:
        raise ParsGpuError(status, "pars_gpu_image_encode")
    return out.tobytes()


def settings_from_json(text):
    """The binary `settings` message of its JSON form (the benchmark's settings files)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    lib = library()
    n = _I64()
    status = lib.pars_gpu_settings_from_json(data, len(data), None, 0, ctypes.byref(n))
    if status:
        raise ParsGpuError(status, "pars_gpu_settings_from_json")
    out = np.zeros(max(n.value, 1), np.uint8)
    status = lib.pars_gpu_settings_from_json(data, len(data), _ptr(out), n.value, ctypes.byref(n))
    if status:
        raise ParsGpuError(status, "pars_gpu_settings_from_json")
    return out[: n.value].tobytes()


def decode_settings(message):
    """pars_gpu_settings_decode: the scalar fields of a `settings` message."""
    data = np.frombuffer(bytes(message), np.uint8)
    out = SettingsSummary()
    status = library().pars_gpu_settings_decode(data.ctypes.data if len(data) else None, len(data), ctypes.byref(out))
    if status:
        raise ParsGpuError(status, "pars_gpu_settings_decode")
    return out


class Service:
    """The request service (pars_gpu_service_*): submit `settings` messages,
    wait, collect results."""

    def __init__(self, device=0, budget_bytes=64 << 30, lanes=2, max_batch=64):
        self.lib = library()
        handle = _P()
        status = self.lib.pars_gpu_service_create(ctypes.byref(handle), device, budget_bytes, lanes, max_batch)
        if status:
            raise ParsGpuError(status, "pars_gpu_service_create")
        self.handle = handle

    def _check(self, status, what):
        if status:
            raise ParsGpuError(status, what)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pars_gpu_service_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_horizon(self, iterations):
        """Steps per warp of each continuous-engine launch for FTLE requests
        (0: each FTLE batch in one launch; -1, the default: chosen by the engine
        for launches of about 2 ms)."""
        self._check(self.lib.pars_gpu_service_set_horizon(self.handle, iterations), "pars_gpu_service_set_horizon")

    def add_dataset(self, name, field):
        self._check(self.lib.pars_gpu_service_add_dataset(self.handle, name.encode(), _ptr(field.xyz), _ptr(field.dims),
                                                          _ptr(field.offset), _ptr(field.size), _ptr(field.spacing)),
                    "pars_gpu_service_add_dataset")

    def add_dataset_device(self, name, device_ptr, dims, offset, size, spacing):
        d, o, s, sp = _i3(dims), _f3(offset), _f3(size), _f3(spacing)
        self._check(self.lib.pars_gpu_service_add_dataset_device(self.handle, name.encode(), device_ptr, _ptr(d), _ptr(o),
                                                                 _ptr(s), _ptr(sp)), "pars_gpu_service_add_dataset_device")

    def submit(self, message):
        data = np.frombuffer(bytes(message), np.uint8)
        t = _I64()
        self._check(self.lib.pars_gpu_service_submit(self.handle, data.ctypes.data, len(data), ctypes.byref(t)),
                    "pars_gpu_service_submit")
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        s = _I32()
        self._check(self.lib.pars_gpu_service_wait(self.handle, ticket, timeout_ms, ctypes.byref(s)), "pars_gpu_service_wait")
        return s.value

    def info(self, ticket):
        i = RequestInfo()
        self._check(self.lib.pars_gpu_service_result_info(self.handle, ticket, ctypes.byref(i)), "pars_gpu_service_result_info")
        return i

    def streamlines(self, ticket):
        """List of (vertices, colors, indices) per batch."""
        out = []
        for b in range(self.info(ticket).batches):
            nv, ni = _I64(), _I64()
            self._check(self.lib.pars_gpu_service_result_batch(self.handle, ticket, b, ctypes.byref(nv), ctypes.byref(ni),
                                                               None, None, None), "pars_gpu_service_result_batch")
            v = np.zeros((nv.value, 4), np.float32)
            c = np.zeros((nv.value, 4), np.float32)
            i = np.zeros(ni.value, np.int32)
            self._check(self.lib.pars_gpu_service_result_batch(self.handle, ticket, b, ctypes.byref(nv), ctypes.byref(ni),
                                                               _ptr(v), _ptr(c), _ptr(i)), "pars_gpu_service_result_batch")
            out.append((v, c, i))
        return out

    def ftle(self, ticket):
        shape = tuple(self.info(ticket).ftle_shape)
        out = np.zeros(shape, np.float32)
        self._check(self.lib.pars_gpu_service_result_ftle(self.handle, ticket, _ptr(out)), "pars_gpu_service_result_ftle")
        return out

    def batch_counts(self, ticket, batch):
        """(vertices, indices) of one streamline batch."""
        nv, ni = _I64(), _I64()
        self._check(self.lib.pars_gpu_service_result_batch(self.handle, ticket, batch, ctypes.byref(nv), ctypes.byref(ni),
                                                           None, None, None), "pars_gpu_service_result_batch")
        return nv.value, ni.value

    def batch_into(self, ticket, batch, vertices_ptr, colors_ptr, indices_ptr):
        """Copies one streamline batch to host addresses (e.g. pinned
        buffers); returns (vertices, indices)."""
        nv, ni = _I64(), _I64()
        self._check(self.lib.pars_gpu_service_result_batch(self.handle, ticket, batch, ctypes.byref(nv), ctypes.byref(ni),
                                                           vertices_ptr, colors_ptr, indices_ptr),
                    "pars_gpu_service_result_batch")
        return nv.value, ni.value

    def ftle_into(self, ticket, values_ptr):
        """Copies an FTLE result to a host address."""
        self._check(self.lib.pars_gpu_service_result_ftle(self.handle, ticket, values_ptr), "pars_gpu_service_result_ftle")

    def add_volume(self, name, values, offset, spacing):
        """A scalar volume [X, Y, Z] for requests whose mode contains "volume"."""
        v = np.ascontiguousarray(values, np.float32)
        s, o, sp = _i3(v.shape), _f3(offset), _f3(spacing)
        self._check(self.lib.pars_gpu_service_add_volume(self.handle, name.encode(), _ptr(v), _ptr(s), _ptr(o), _ptr(sp)),
                    "pars_gpu_service_add_volume")

    def serve(self, listener, max_requests=0):
        """Answers one ZMTP PAIR peer on `listener` (pars_gpu_service_serve);
        returns the number of requests answered."""
        n = _I64()
        self._check(self.lib.pars_gpu_service_serve(self.handle, listener, max_requests, ctypes.byref(n)), "pars_gpu_service_serve")
        return n.value

    def image_into(self, ticket, rgba_ptr):
        """Copies the request's image to a host address (width * height * 4
        bytes); returns (width, height), (0, 0) without an image."""
        size = np.zeros(2, np.int32)
        self._check(self.lib.pars_gpu_service_result_image(self.handle, ticket, rgba_ptr, _ptr(size)),
                    "pars_gpu_service_result_image")
        return int(size[0]), int(size[1])

    def image(self, ticket):
        """The request's image, [height, width, 4] uint8 (None without one)."""
        size = np.zeros(2, np.int32)
        self._check(self.lib.pars_gpu_service_result_image(self.handle, ticket, None, _ptr(size)), "pars_gpu_service_result_image")
        if size[0] == 0:
            return None
        out = np.zeros((size[1], size[0], 4), np.uint8)
        self._check(self.lib.pars_gpu_service_result_image(self.handle, ticket, _ptr(out), _ptr(size)),
                    "pars_gpu_service_result_image")
        return out

    def release(self, ticket):
        self._check(self.lib.pars_gpu_service_release(self.handle, ticket), "pars_gpu_service_release")

    def profile_enable(self, on=True):
        self._check(self.lib.pars_gpu_service_profile_enable(self.handle, 1 if on else 0), "pars_gpu_service_profile_enable")

    def profile_get(self, name):
        """(milliseconds, count) of a kernel or batch phase (see pars_gpu.h)."""
        ms, n = ctypes.c_double(), _I64()
        self._check(self.lib.pars_gpu_service_profile_get(self.handle, name.encode(), ctypes.byref(ms), ctypes.byref(n)),
                    "pars_gpu_service_profile_get")
        return ms.value, n.value
