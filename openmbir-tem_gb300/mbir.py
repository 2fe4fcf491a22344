"""ctypes binding of libmbir_gb300.so (the C ABI in include/mbir_gb300.h).

This is a thin host-side wrapper for Python callers, tests and the benchmark.  It loads the
in-tree CUDA library and raises if it is missing: there is no CPU fallback.

    import mbir
    p = mbir.default_params()
    p.sample_thickness = 32; p.diffuseness = 0.1; p.sigma_x = 0.2; p.num_resolutions = 1
    eng = mbir.Engine(p)
    eng.set_sinogram(counts, tilts_deg, delta_r=1.0, delta_t=1.0)   # counts[theta][r][t]
    eng.run()
    vol = eng.volume()                                              # [z][x][y]
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmbir_gb300.so")

MBIR_OK = 0
ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "EDEVICE", -4: "EIO", -5: "ESTATE", -6: "ETIMEOUT",
          -7: "ENOTSUP", -999: "ECANCELLED"}
HAADF, BF = 0, 1
ORDER_PARALLEL, ORDER_REFERENCE = 0, 1
FP32, FP64 = 0, 1
SEED_PER_CALL, SEED_FIXED = 0, 1
# observer aspects (mbir_set_observer), the reference's ObserverAspect order
(UPDATE_PROGRESS_VALUE, UPDATE_PROGRESS_MESSAGE, UPDATE_WARNING_MESSAGE, UPDATE_ERROR_MESSAGE,
 UPDATE_PROGRESS_VALUE_AND_MESSAGE, UPDATE_INTERMEDIATE_IMAGE) = range(6)
OBSERVER = C.CFUNCTYPE(None, C.c_char_p, C.c_int32, C.c_int32, C.c_void_p)


class MbirParams(C.Structure):
    """Mirror of struct mbir_params (include/mbir_gb300.h); field order and types must match."""
    _fields_ = [
        ("struct_size", C.c_int32),
        ("modality", C.c_int32),
        ("sample_thickness", C.c_double),
        ("diffuseness", C.c_double),
        ("sigma_x", C.c_double),
        ("stop_threshold", C.c_double),
        ("num_resolutions", C.c_int32),
        ("final_resolution", C.c_int32),
        ("level", C.c_int32),
        ("target_gain", C.c_double),
        ("outer_iterations", C.c_int32),
        ("inner_iterations", C.c_int32),
        ("default_offset", C.c_double),
        ("use_default_offset", C.c_int32),
        ("default_variance", C.c_double),
        ("default_recon_value", C.c_double),
        ("extend_object", C.c_int32),
        ("interpolate_initial_recon", C.c_int32),
        ("tilt_selection", C.c_int32),
        ("use_subvolume", C.c_int32),
        ("subvolume", C.c_int32 * 6),
        ("default_pixel_size", C.c_double),
        ("n_excluded_views", C.c_int32),
        ("excluded_views", C.c_int32 * 256),
        ("x_shrink_factor", C.c_double),
        ("z_stretch", C.c_int32),
        ("detector_response_bins", C.c_int32),
        ("profile_resolution", C.c_int32),
        ("beam_resolution", C.c_int32),
        ("joint_estimation", C.c_int32),
        ("zero_skipping", C.c_int32),
        ("noise_model", C.c_int32),
        ("noise_estimation", C.c_int32),
        ("estimate_prior", C.c_int32),
        ("threshold_reduction_factor", C.c_double),
        ("qggmrf_p", C.c_double),
        ("qggmrf_q", C.c_double),
        ("qggmrf_c", C.c_double),
        ("qggmrf_alpha", C.c_double),
        ("bragg_threshold", C.c_double),
        ("bragg_delta", C.c_double),
        ("bf_offset", C.c_double),
        ("default_dosage", C.c_double),
        ("order_mode", C.c_int32),
        ("precision", C.c_int32),
        ("seed", C.c_uint32),
        ("compat_double_angle", C.c_int32),
        ("cost_every_sweep", C.c_int32),
        ("device", C.c_int32),
        ("verbose", C.c_int32),
        ("slice_staging", C.c_int32),
        ("nhicd", C.c_int32),
        ("lane_shape", C.c_int32),
        ("call_schedule", C.c_int32),
        ("seed_mode", C.c_int32),
        ("float_params", C.c_int32),
    ]


class MbirStatus(C.Structure):
    _fields_ = [
        ("state", C.c_int32), ("outer_iter", C.c_int32), ("inner_iter", C.c_int32),
        ("sweeps_done", C.c_int32), ("last_cost", C.c_double), ("last_rel_update", C.c_double),
        ("icd_ms_total", C.c_double), ("total_ms", C.c_double), ("voxels_visited", C.c_int64),
        ("voxels_updated", C.c_int64), ("footprint_entries", C.c_int64), ("t_rows", C.c_int32),
        ("stride", C.c_int32), ("staged", C.c_int32), ("lane_shape", C.c_int32),
        ("sched_levels", C.c_int32), ("sched_ms_total", C.c_double),
        ("kernel_ms_total", C.c_double), ("colour_ms_total", C.c_double),
    ]


class MbirServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
        ("active", C.c_int32), ("queued", C.c_int32), ("p50_ms", C.c_double),
        ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("voxel_updates", C.c_double),
        ("busy_s", C.c_double), ("batched_sweep_ms", C.c_double), ("batched_sweeps", C.c_int64),
        ("budget_bytes", C.c_int64), ("peak_bytes", C.c_int64), ("peak_active", C.c_int32),
        ("reserved", C.c_int32), ("admitted", C.c_int64), ("admitted_out_of_order", C.c_int64),
    ]


_lib = None

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)

SIGNATURES = {
    "mbir_version": (C.c_char_p, []),
    "mbir_params_default": (None, [C.POINTER(MbirParams), C.c_int32]),
    "mbir_create": (C.c_void_p, [C.POINTER(MbirParams)]),
    "mbir_destroy": (None, [C.c_void_p]),
    "mbir_last_error": (C.c_char_p, [C.c_void_p]),
    "mbir_set_sinogram": (C.c_int32, [C.c_void_p, _F, _F, C.c_int32, C.c_int32, C.c_int32,
                                      C.c_double, C.c_double]),
    "mbir_load_sinogram_mrc": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "mbir_set_initial_volume_f64": (C.c_int32, [C.c_void_p, _D, C.c_int64]),
    "mbir_get_volume_f64": (C.c_int32, [C.c_void_p, _D, C.c_int64]),
    "mbir_set_bright_field": (C.c_int32, [C.c_void_p, _F, C.c_int32, C.c_int32, C.c_int32]),
    "mbir_load_bright_field_mrc": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "mbir_set_intermediate_dir": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "mbir_set_observer": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mbir_write_checkpoint": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "mbir_read_checkpoint": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "mbir_set_initial_volume": (C.c_int32, [C.c_void_p, _F, C.c_int64]),
    "mbir_set_initial_nuisance": (C.c_int32, [C.c_void_p, _D, _D, _D]),
    "mbir_get_dims": (C.c_int32, [C.c_void_p, _I]),
    "mbir_run": (C.c_int32, [C.c_void_p]),
    "mbir_prepare": (C.c_int32, [C.c_void_p]),
    "mbir_sweep": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, _D]),
    "mbir_joint_estimation": (C.c_int32, [C.c_void_p]),
    "mbir_update_weights": (C.c_int32, [C.c_void_p]),
    "mbir_compute_cost": (C.c_int32, [C.c_void_p, _D, _D]),
    "mbir_forward_project": (C.c_int32, [C.c_void_p]),
    "mbir_get_volume": (C.c_int32, [C.c_void_p, _F, C.c_int64]),
    "mbir_get_error_sinogram": (C.c_int32, [C.c_void_p, _F, C.c_int64]),
    "mbir_get_projection": (C.c_int32, [C.c_void_p, _F, C.c_int64]),
    "mbir_get_nuisance": (C.c_int32, [C.c_void_p, _D, _D, _D]),
    "mbir_get_tables": (C.c_int32, [C.c_void_p, _D, _D]),
    "mbir_get_schedule": (C.c_int32, [C.c_void_p, C.c_int32, _I, _I]),
    "mbir_get_call_lines": (C.c_int32, [C.c_void_p, _I, C.c_int32, _I]),
    "mbir_get_call_schedule": (C.c_int32, [C.c_void_p, _I, C.c_int32, _I, C.c_int32, _I, _I]),
    "mbir_get_footprint_bins": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int16),
                                            C.POINTER(C.c_uint16), C.POINTER(C.c_uint8)]),
    "mbir_error_view_sums_noalloc": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                                 C.c_void_p, C.c_void_p]),
    "mbir_get_bf_state": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint8), _F, _D, _D, _D]),
    "mbir_set_bragg_threshold": (C.c_int32, [C.c_void_p, C.c_double]),
    "mbir_set_slab": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "mbir_sweep_colour": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _D]),
    "mbir_get_planes": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, _F]),
    "mbir_set_planes": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, _F]),
    "mbir_view_sums": (C.c_int32, [C.c_void_p, C.c_int32, _D]),
    "mbir_bf_call_begin": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "mbir_bf_call_magnitudes": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "mbir_bf_call_end": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "mbir_bf_slab_sums": (C.c_int32, [C.c_void_p, C.c_int32, _D]),
    "mbir_bf_slab_apply": (C.c_int32, [C.c_void_p, C.c_int32, _D]),
    "mbir_roi_sums": (C.c_int32, [C.c_void_p, _D]),
    "mbir_apply_nuisance": (C.c_int32, [C.c_void_p, _D, _D, _D]),
    "mbir_status_get": (C.c_int32, [C.c_void_p, C.POINTER(MbirStatus)]),
    "mbir_cancel": (None, [C.c_void_p]),
    "mbir_write_outputs": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "mbir_estimate_sigma_x": (C.c_int32, [C.c_char_p, C.c_double, C.c_double, C.c_int32,
                                          C.c_double, _F, C.c_int32, _I, _I, _D]),
    "mbir_write_outputs_ex": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                          C.c_char_p]),
    "mbir_batch_create": (C.c_void_p, [C.c_int32]),
    "mbir_batch_destroy": (None, [C.c_void_p]),
    "mbir_batch_add": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mbir_batch_remove": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mbir_batch_size": (C.c_int32, [C.c_void_p]),
    "mbir_batch_set_threads": (C.c_int32, [C.c_void_p, C.c_int32]),
    "mbir_batch_get_threads": (C.c_int32, [C.c_void_p]),
    "mbir_batch_set_wait_limit": (C.c_int32, [C.c_void_p, C.c_double]),
    "mbir_batch_sweep": (C.c_int32, [C.c_void_p, C.c_int32, _D]),
    "mbir_batch_run": (C.c_int32, [C.c_void_p, C.c_int32, C.c_double, _I, _D]),
    "mbir_batch_last_ms": (C.c_double, [C.c_void_p]),
    "mbir_batch_total_ms": (C.c_double, [C.c_void_p]),
    "mbir_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "mbir_server_create": (C.c_void_p, [C.c_int32, C.c_int64, C.c_int32]),
    "mbir_server_destroy": (None, [C.c_void_p]),
    "mbir_server_submit": (C.c_int64, [C.c_void_p, C.POINTER(MbirParams), _F, _F, C.c_int32,
                                       C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32,
                                       C.c_double]),
    "mbir_server_poll": (C.c_int32, [C.c_void_p, C.c_int64, _I, _D, _I, _D]),
    "mbir_server_wait": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double]),
    "mbir_server_result": (C.c_int32, [C.c_void_p, C.c_int64, _F, C.c_int64, _I]),
    "mbir_server_release": (C.c_int32, [C.c_void_p, C.c_int64]),
    "mbir_server_get_stats": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "mbir_server_last_error": (C.c_char_p, [C.c_void_p]),
    "mbir_run_multires": (C.c_int32, [C.POINTER(MbirParams), _F, _F, C.c_int32, C.c_int32,
                                      C.c_int32, C.c_double, C.c_double, _F, C.c_int64, _I]),
    "mbir_colour_schedule": (C.c_int32, [C.c_int32] * 7 + [C.POINTER(C.c_uint8),
                                                           C.POINTER(C.c_uint8),
                                                           C.POINTER(C.c_int16),
                                                           C.POINTER(C.c_uint16), _I, C.c_int32,
                                                           _I, C.c_int32, _I, _I]),
    "mbir_level_schedule": (C.c_int32, [C.c_int32] * 6 + [_I, C.POINTER(C.c_uint8),
                                                          C.POINTER(C.c_uint8),
                                                          C.POINTER(C.c_int16),
                                                          C.POINTER(C.c_uint16), _I, C.c_int32,
                                                          _I, C.c_int32, _I, _I]),
}


def colour_schedule(lineok, lo, mask, nb, n_r, active=None, max_colours=1024, class_cap=0):
    """Colour schedule of a sparse ICD call (mbir_colour_schedule): returns (lines, lofs)."""
    lineok = np.ascontiguousarray(lineok, np.uint8)
    n_z, n_x = lineok.shape
    lo = np.ascontiguousarray(lo, np.int16)
    mask = np.ascontiguousarray(mask, np.uint16)
    act = None if active is None else np.ascontiguousarray(active, np.uint8)
    cap = n_z * n_x
    lines = np.zeros(cap, np.int32)
    lofs = np.zeros(cap + 1, np.int32)
    nl = C.c_int32()
    nc = C.c_int32()
    u8 = C.POINTER(C.c_uint8)
    rc = lib().mbir_colour_schedule(
        n_z, n_x, lo.shape[2], int(n_r), int(nb), int(max_colours), int(class_cap),
        lineok.ctypes.data_as(u8),
        None if act is None else act.ctypes.data_as(u8), lo.ctypes.data_as(C.POINTER(C.c_int16)),
        mask.ctypes.data_as(C.POINTER(C.c_uint16)), lines.ctypes.data_as(_I), cap,
        lofs.ctypes.data_as(_I), cap + 1, C.byref(nl), C.byref(nc))
    if rc != 0:
        raise MbirError(rc, "mbir_colour_schedule failed")
    return lines[:nl.value].copy(), lofs[:nc.value + 1].copy()


def level_schedule(rows, lineok, lo, mask, nb, stride, n_r, active=None):
    """Dependency levels of a sparse ICD call (mbir_level_schedule): returns (lines, lofs).
    lineok/active are [n_z, n_x] bytes, lo/mask [n_z, n_x, n_theta]."""
    lineok = np.ascontiguousarray(lineok, np.uint8)
    n_z, n_x = lineok.shape
    lo = np.ascontiguousarray(lo, np.int16)
    mask = np.ascontiguousarray(mask, np.uint16)
    n_theta = lo.shape[2]
    rows = np.ascontiguousarray(rows, np.int32)
    act = None if active is None else np.ascontiguousarray(active, np.uint8)
    cap = n_z * n_x
    lines = np.zeros(cap, np.int32)
    lofs = np.zeros(cap + 1, np.int32)
    nl = C.c_int32()
    nlev = C.c_int32()
    u8 = C.POINTER(C.c_uint8)
    rc = lib().mbir_level_schedule(
        n_z, n_x, n_theta, int(n_r), int(nb), int(stride), rows.ctypes.data_as(_I),
        lineok.ctypes.data_as(u8), None if act is None else act.ctypes.data_as(u8),
        lo.ctypes.data_as(C.POINTER(C.c_int16)), mask.ctypes.data_as(C.POINTER(C.c_uint16)),
        lines.ctypes.data_as(_I), cap, lofs.ctypes.data_as(_I), cap + 1, C.byref(nl),
        C.byref(nlev))
    if rc != 0:
        raise MbirError(rc, "mbir_level_schedule failed")
    return lines[:nl.value].copy(), lofs[:nlev.value + 1].copy()


def lib():
    """Load libmbir_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with openmbir-tem_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def default_params(modality=HAADF):
    p = MbirParams()
    lib().mbir_params_default(C.byref(p), modality)
    if p.struct_size != C.sizeof(MbirParams):
        raise RuntimeError("mbir_params layout mismatch between the binding and the library")
    return p


def _fp(a):
    return a.ctypes.data_as(_F)


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


class MbirError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Engine:
    """One reconstruction on one GPU (mbir_engine*)."""

    def __init__(self, params):
        self._h = lib().mbir_create(C.byref(params))
        if not self._h:
            raise MbirError(-1, lib().mbir_last_error(None).decode())
        self.params = params

    def close(self):
        if getattr(self, "_h", None):
            lib().mbir_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != MBIR_OK:
            raise MbirError(rc, lib().mbir_last_error(self._h).decode())
        return rc

    def set_sinogram(self, counts, tilts_deg, delta_r=1.0, delta_t=1.0):
        counts = np.ascontiguousarray(counts, dtype=np.float32)
        tilts = np.ascontiguousarray(tilts_deg, dtype=np.float32)
        nt, nr, ntt = counts.shape
        self._counts = counts
        return self._check(lib().mbir_set_sinogram(self._h, _fp(counts), _fp(tilts), nt, nr, ntt,
                                                   delta_r, delta_t))

    def load_mrc(self, path):
        return self._check(lib().mbir_load_sinogram_mrc(self._h, str(path).encode()))

    def set_bright_field(self, counts):
        """HAADF with bright-field data: counts[theta][r][t] of the sinogram's size."""
        c = np.ascontiguousarray(counts, np.float32)
        n_theta, n_r, n_t = c.shape
        return self._check(lib().mbir_set_bright_field(self._h, c.ctypes.data_as(_F), n_theta,
                                                        n_r, n_t))

    def set_intermediate_dir(self, directory):
        """HAADF: <dir>/<outer>_<inner>_ReconstructedVolume.rec after every inner iteration."""
        d = b"" if directory is None else str(directory).encode()
        return self._check(lib().mbir_set_intermediate_dir(self._h, d))

    def set_observer(self, fn):
        """fn(msg: str, progress: int, aspect: int) receives the engine's messages (aspects
        UPDATE_*, the reference's ObserverAspect order); None removes it."""
        if fn is None:
            self._observer = None
            return self._check(lib().mbir_set_observer(self._h, None, None))

        def forward(msg, progress, aspect, _user):
            fn(msg.decode(errors="replace") if msg else "", progress, aspect)

        self._observer = OBSERVER(forward)  # kept alive as long as the engine can call it
        return self._check(lib().mbir_set_observer(self._h, C.cast(self._observer, C.c_void_p),
                                                   None))

    def write_checkpoint(self, directory):
        """HAADF: the run's state in `directory` (the reference's .bin files + Checkpoint.bin)."""
        return self._check(lib().mbir_write_checkpoint(self._h, str(directory).encode()))

    def read_checkpoint(self, directory):
        """HAADF: start every later prepare from a checkpoint of the same configuration and
        series; run() continues at its outer iteration."""
        return self._check(lib().mbir_read_checkpoint(self._h, str(directory).encode()))

    def load_bright_field_mrc(self, path):
        return self._check(lib().mbir_load_bright_field_mrc(self._h, str(path).encode()))

    def dims(self):
        d = np.zeros(6, np.int32)
        self._check(lib().mbir_get_dims(self._h, d.ctypes.data_as(_I)))
        return tuple(int(v) for v in d)

    def set_initial_volume(self, vol):
        """[z][x][y]; float64 arrays go through the FP64 entry point (exact for FP64 engines)."""
        if np.asarray(vol).dtype == np.float64:
            v = np.ascontiguousarray(vol, dtype=np.float64)
            return self._check(lib().mbir_set_initial_volume_f64(self._h, v.ctypes.data_as(_D),
                                                                 v.size))
        vol = np.ascontiguousarray(vol, dtype=np.float32)
        return self._check(lib().mbir_set_initial_volume(self._h, _fp(vol), vol.size))

    def set_initial_nuisance(self, gains=None, offsets=None, variances=None):
        g = None if gains is None else np.ascontiguousarray(gains, np.float64)
        o = None if offsets is None else np.ascontiguousarray(offsets, np.float64)
        v = None if variances is None else np.ascontiguousarray(variances, np.float64)
        return self._check(lib().mbir_set_initial_nuisance(self._h, _dp(g), _dp(o), _dp(v)))

    def prepare(self):
        return self._check(lib().mbir_prepare(self._h))

    def run(self):
        return self._check(lib().mbir_run(self._h))

    def sweep(self, outer=0, inner=0):
        st = np.zeros(4, np.float64)
        self._check(lib().mbir_sweep(self._h, outer, inner, _dp(st)))
        return st

    def joint_estimation(self):
        return self._check(lib().mbir_joint_estimation(self._h))

    def update_weights(self):
        return self._check(lib().mbir_update_weights(self._h))

    def cost(self):
        parts = np.zeros(3, np.float64)
        tot = C.c_double()
        self._check(lib().mbir_compute_cost(self._h, _dp(parts), C.byref(tot)))
        return tot.value, parts

    def forward_project(self):
        return self._check(lib().mbir_forward_project(self._h))

    def volume(self):
        nz, nx, ny = self.dims()[:3]
        out = np.empty((nz, nx, ny), np.float32)
        self._check(lib().mbir_get_volume(self._h, _fp(out), out.size))
        return out

    def volume64(self):
        """The volume as doubles (an FP64 engine's values exactly)."""
        nz, nx, ny = self.dims()[:3]
        out = np.empty((nz, nx, ny), np.float64)
        self._check(lib().mbir_get_volume_f64(self._h, out.ctypes.data_as(_D), out.size))
        return out

    def _sino(self, fn):
        _, _, _, nt, nr, ntt = self.dims()
        out = np.empty((nt, nr, ntt), np.float32)
        self._check(fn(self._h, _fp(out), out.size))
        return out

    def error_sinogram(self):
        return self._sino(lib().mbir_get_error_sinogram)

    def projection(self):
        return self._sino(lib().mbir_get_projection)

    def nuisance(self):
        nt = self.dims()[3]
        g, o, v = (np.zeros(nt) for _ in range(3))
        self._check(lib().mbir_get_nuisance(self._h, _dp(g), _dp(o), _dp(v)))
        return g, o, v

    def tables(self):
        nt = self.dims()[3]
        bins = self.params.detector_response_bins
        H = np.zeros((nt, bins))
        Ht = np.zeros(bins)
        self._check(lib().mbir_get_tables(self._h, _dp(H), _dp(Ht)))
        return H, Ht

    def schedule(self, sweep=0):
        nz = self.dims()[0]
        rows = np.zeros(nz, np.int32)
        stride = C.c_int32()
        self._check(lib().mbir_get_schedule(self._h, sweep, rows.ctypes.data_as(_I),
                                            C.byref(stride)))
        return rows, stride.value

    def call_lines(self):
        n = C.c_int32()
        self._check(lib().mbir_get_call_lines(self._h, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1), np.int32)
        self._check(lib().mbir_get_call_lines(self._h, out.ctypes.data_as(_I), n.value, C.byref(n)))
        return out[:n.value]

    def call_schedule(self):
        """(lines level by level, level offsets) of the last scheduled call."""
        n = C.c_int32()
        nl = C.c_int32()
        self._check(lib().mbir_get_call_schedule(self._h, None, 0, None, 0, C.byref(n),
                                                 C.byref(nl)))
        lines = np.zeros(max(n.value, 1), np.int32)
        lofs = np.zeros(nl.value + 1, np.int32)
        self._check(lib().mbir_get_call_schedule(self._h, lines.ctypes.data_as(_I), n.value,
                                                 lofs.ctypes.data_as(_I), nl.value + 1,
                                                 C.byref(n), C.byref(nl)))
        return lines[:n.value], lofs[:nl.value + 1]

    def footprint_bins(self):
        """(lo [z][x][theta] int16, mask uint16, lineok [z][x] uint8) of the schedules."""
        nz, nx, ny, nt, nr, ntt = self.dims()
        lo = np.zeros((nz, nx, nt), np.int16)
        mask = np.zeros((nz, nx, nt), np.uint16)
        ok = np.zeros((nz, nx), np.uint8)
        self._check(lib().mbir_get_footprint_bins(
            self._h, lo.ctypes.data_as(C.POINTER(C.c_int16)),
            mask.ctypes.data_as(C.POINTER(C.c_uint16)), ok.ctypes.data_as(C.POINTER(C.c_uint8))))
        return lo, mask, ok

    def bf_state(self):
        """(selector [theta][r][t] uint8, weights float32, mag [z][x], filtered mag, T)"""
        nz, nx, ny, nt, nr, ntt = self.dims()
        sel = np.zeros((nt, nr, ntt), np.uint8)
        w = np.zeros((nt, nr, ntt), np.float32)
        mag = np.zeros((nz, nx))
        filt = np.zeros((nz, nx))
        t = C.c_double()
        self._check(lib().mbir_get_bf_state(self._h, sel.ctypes.data_as(C.POINTER(C.c_uint8)),
                                            w.ctypes.data_as(_F), mag.ctypes.data_as(_D),
                                            filt.ctypes.data_as(_D), C.byref(t)))
        return sel, w, mag, filt, t.value

    # ---- y-slab sharding -----------------------------------------------------------------
    def set_slab(self, y0, y1):
        self._check(lib().mbir_set_slab(self._h, y0, y1))

    def sweep_colour(self, colour, outer=0, inner=0):
        st = np.zeros(4)
        self._check(lib().mbir_sweep_colour(self._h, colour, outer, inner, st.ctypes.data_as(_D)))
        return st

    def get_planes(self, y, n):
        nz, nx = self.dims()[:2]
        out = np.zeros((n, nz, nx), np.float32)
        self._check(lib().mbir_get_planes(self._h, y, n, out.ctypes.data_as(_F)))
        return out

    def set_planes(self, y, planes):
        planes = np.ascontiguousarray(planes, np.float32)
        self._check(lib().mbir_set_planes(self._h, y, planes.shape[0], planes.ctypes.data_as(_F)))

    def view_sums(self, kind):
        nt = self.dims()[3]
        out = np.zeros(nt * (6 if kind == 0 else 1))
        self._check(lib().mbir_view_sums(self._h, kind, out.ctypes.data_as(_D)))
        return out

    def bf_call_begin(self, outer=0, inner=0):
        """Bright-field slabs: open one NHICD call (its lines, schedule and row order); the
        slab's colours follow with sweep_colour, and bf_call_end closes it."""
        self._check(lib().mbir_bf_call_begin(self._h, outer, inner))

    def bf_call_magnitudes(self):
        """The open call's update magnitude per line [z][x] over the slab's slices (uint64,
        fixed point 2^-32), to add over slabs."""
        nz, nx = self.dims()[:2]
        out = np.zeros(nz * nx, np.uint64)
        self._check(lib().mbir_bf_call_magnitudes(
            self._h, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def bf_call_end(self, magnitudes=None):
        """Close the call; the magnitude map takes `magnitudes` (summed over slabs; None: the
        slab's own)."""
        m = None if magnitudes is None else np.ascontiguousarray(magnitudes, np.uint64)
        self._check(lib().mbir_bf_call_end(
            self._h, m.ctypes.data_as(C.POINTER(C.c_uint64)) if m is not None else None))

    def bf_slab_sums(self, kind):
        """kind 2: offset-step numerator and denominator per view [theta][2]; kind 3: the two
        variance sums and the number of entries they cover (scales the slab's weights first:
        once per update)."""
        nt = self.dims()[3]
        out = np.zeros(2 * nt if kind == 2 else 3)
        self._check(lib().mbir_bf_slab_sums(self._h, kind, out.ctypes.data_as(_D)))
        return out

    def bf_slab_apply(self, kind, sums):
        s = np.ascontiguousarray(sums, np.float64)
        self._check(lib().mbir_bf_slab_apply(self._h, kind, s.ctypes.data_as(_D)))

    def roi_sums(self):
        """The stop rule's ROI sums: magnitude map, and the slab's volume."""
        out = np.zeros(2)
        self._check(lib().mbir_roi_sums(self._h, out.ctypes.data_as(_D)))
        return out

    def apply_nuisance(self, gain=None, offset=None, variance=None):
        def ptr(a):
            return None if a is None else np.ascontiguousarray(a, np.float64).ctypes.data_as(_D)
        g = None if gain is None else np.ascontiguousarray(gain, np.float64)
        o = None if offset is None else np.ascontiguousarray(offset, np.float64)
        v = None if variance is None else np.ascontiguousarray(variance, np.float64)
        self._check(lib().mbir_apply_nuisance(
            self._h, g.ctypes.data_as(_D) if g is not None else None,
            o.ctypes.data_as(_D) if o is not None else None,
            v.ctypes.data_as(_D) if v is not None else None))

    def set_bragg(self, t):
        self._check(lib().mbir_set_bragg_threshold(self._h, float(t)))

    def status(self):
        st = MbirStatus()
        self._check(lib().mbir_status_get(self._h, C.byref(st)))
        return st

    def cancel(self):
        lib().mbir_cancel(self._h)

    def write_outputs(self, directory, mrc_path=""):
        return self._check(lib().mbir_write_outputs(self._h, str(directory).encode(),
                                                    str(mrc_path).encode()))


class Batch:
    """Many prepared FP32 engines advanced together (mbir_batch*)."""

    def __init__(self, device=0):
        self._h = lib().mbir_batch_create(device)
        if not self._h:
            raise MbirError(-2, "mbir_batch_create failed")
        self.engines = []

    def close(self):
        if getattr(self, "_h", None):
            lib().mbir_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != MBIR_OK:
            raise MbirError(rc, lib().mbir_batch_last_error(self._h).decode())
        return rc

    def add(self, engine):
        self._check(lib().mbir_batch_add(self._h, engine._h))
        self.engines.append(engine)

    def remove(self, engine):
        self._check(lib().mbir_batch_remove(self._h, engine._h))
        self.engines.remove(engine)

    def sweep(self, outer=0):
        st = np.zeros((len(self.engines), 4))
        self._check(lib().mbir_batch_sweep(self._h, outer, _dp(st)))
        return st

    def run(self, max_outer, tol):
        n = len(self.engines)
        od = np.zeros(n, np.int32)
        fc = np.zeros(n)
        self._check(lib().mbir_batch_run(self._h, max_outer, tol, od.ctypes.data_as(_I), _dp(fc)))
        return od, fc

    def last_ms(self):
        return lib().mbir_batch_last_ms(self._h)

    def total_ms(self):
        return lib().mbir_batch_total_ms(self._h)

    def set_threads(self, threads):
        """CTA size of the persistent batched sweep: 512, 256 (two slices per SM) or 0 (tuned
        online over the second to fifth sweeps, the default)."""
        self._check(lib().mbir_batch_set_threads(self._h, int(threads)))

    def threads(self):
        """The CTA size in use (0 while the online tuning runs)."""
        return int(lib().mbir_batch_get_threads(self._h))

    def set_wait_limit(self, seconds):
        """Limit of the device-side wait of a colour-1 slice (mbir_batch_set_wait_limit)."""
        self._check(lib().mbir_batch_set_wait_limit(self._h, float(seconds)))


class Server:
    """Continuous-batching reconstruction server on one device (mbir_server*)."""

    def __init__(self, device=0, mem_budget=0, max_active=0):
        self._h = lib().mbir_server_create(device, mem_budget, max_active)
        if not self._h:
            raise MbirError(-2, "mbir_server_create failed")

    def close(self):
        if getattr(self, "_h", None):
            lib().mbir_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params, counts, tilts_deg, delta_r=1.0, delta_t=1.0, max_outer=20,
               tol=1e-4):
        counts = np.ascontiguousarray(counts, np.float32)
        tilts = np.ascontiguousarray(tilts_deg, np.float32)
        nt, nr, ntt = counts.shape
        rid = lib().mbir_server_submit(self._h, C.byref(params), _fp(counts), _fp(tilts), nt, nr,
                                       ntt, delta_r, delta_t, max_outer, tol)
        if rid <= 0:
            raise MbirError(int(rid), lib().mbir_server_last_error(self._h).decode())
        return rid

    def poll(self, rid):
        st, od = C.c_int32(), C.c_int32()
        lat, cost = C.c_double(), C.c_double()
        rc = lib().mbir_server_poll(self._h, rid, C.byref(st), C.byref(lat), C.byref(od),
                                    C.byref(cost))
        if rc != MBIR_OK:
            raise MbirError(rc, "poll")
        return st.value, lat.value, od.value, cost.value

    def wait(self, rid, timeout=600.0):
        rc = lib().mbir_server_wait(self._h, rid, timeout)
        if rc != MBIR_OK:
            raise MbirError(rc, lib().mbir_server_last_error(self._h).decode())

    def result(self, rid):
        dims = np.zeros(3, np.int32)
        rc = lib().mbir_server_result(self._h, rid, None, 0, dims.ctypes.data_as(_I))
        if rc != MBIR_OK:
            raise MbirError(rc, "result")
        out = np.empty(tuple(int(d) for d in dims), np.float32)
        rc = lib().mbir_server_result(self._h, rid, _fp(out), out.size, dims.ctypes.data_as(_I))
        if rc != MBIR_OK:
            raise MbirError(rc, "result")
        return out

    def release(self, rid):
        return lib().mbir_server_release(self._h, rid)

    def stats(self):
        st = MbirServerStats()
        lib().mbir_server_get_stats(self._h, C.byref(st))
        return st


def run_multires(params, counts, tilts_deg, delta_r=1.0, delta_t=1.0):
    counts = np.ascontiguousarray(counts, np.float32)
    tilts = np.ascontiguousarray(tilts_deg, np.float32)
    nt, nr, ntt = counts.shape
    finest = MbirParams.from_buffer_copy(params)
    finest.level = -1
    with Engine(finest) as probe:
        probe.set_sinogram(counts, tilts, delta_r, delta_t)
        nz, nx, ny = probe.dims()[:3]
    dims = np.zeros(3, np.int32)
    out = np.empty((nz, nx, ny), np.float32)
    rc = lib().mbir_run_multires(C.byref(params), _fp(counts), _fp(tilts), nt, nr, ntt, delta_r,
                                 delta_t, _fp(out), out.size, dims.ctypes.data_as(_I))
    if rc != MBIR_OK:
        raise MbirError(rc, "multires")
    return out


def estimate_sigma_x(mrc_path, sample_thickness, target_gain=1.0, bf_offset=None, tilts=None,
                     x_range=None, y_range=None):
    """sigma_x estimate of an MRC tilt series (mbir_estimate_sigma_x); bf_offset not None uses
    the bright-field log form."""
    t = None if tilts is None else np.ascontiguousarray(tilts, np.float32)
    xr = None if x_range is None else np.ascontiguousarray(x_range, np.int32)
    yr = None if y_range is None else np.ascontiguousarray(y_range, np.int32)
    out = C.c_double()
    rc = lib().mbir_estimate_sigma_x(str(mrc_path).encode(), float(sample_thickness),
                                     float(target_gain), 0 if bf_offset is None else 1,
                                     0.0 if bf_offset is None else float(bf_offset),
                                     None if t is None else _fp(t), 0 if t is None else len(t),
                                     None if xr is None else xr.ctypes.data_as(_I),
                                     None if yr is None else yr.ctypes.data_as(_I),
                                     C.byref(out))
    if rc != MBIR_OK:
        raise MbirError(rc, "mbir_estimate_sigma_x failed")
    return out.value
