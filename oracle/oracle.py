"""ctypes binding of the FP64 CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by the
cpu_baseline / reference leg of bench.py, always as the checker or the timed CPU baseline,
never as a product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "mbir_oracle.c")


class OrcParams(C.Structure):
    _fields_ = [
        ("delta_xz_factor", C.c_double), ("interpolate_factor", C.c_double),
        ("length_z", C.c_double), ("extend_object", C.c_int32), ("x_shrink_factor", C.c_double),
        ("z_stretch", C.c_int32), ("response_bins", C.c_int32),
        ("profile_resolution", C.c_int32), ("beam_resolution", C.c_int32),
        ("compat_double_angle", C.c_int32), ("sigma_x", C.c_double), ("mrf_p", C.c_double),
        ("mrf_q", C.c_double), ("mrf_c", C.c_double), ("mrf_alpha", C.c_double),
        ("target_gain", C.c_double), ("default_offset", C.c_double),
        ("default_variance", C.c_double), ("default_recon_value", C.c_double),
        ("use_default_offset", C.c_int32), ("joint_estimation", C.c_int32),
        ("noise_model", C.c_int32), ("zero_skipping", C.c_int32), ("stop_threshold", C.c_double),
        ("outer_iterations", C.c_int32), ("inner_iterations", C.c_int32),
        ("threshold_reduction_factor", C.c_double),
        ("pinned_pow", C.c_int32),
        ("modality", C.c_int32), ("noise_estimation", C.c_int32),
        ("bragg_threshold", C.c_double), ("bragg_delta", C.c_double), ("bf_offset", C.c_double),
        ("nhicd", C.c_int32),
    ]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)
_lib = None


def build(force=False):
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", LIB,
                               SRC, "-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        sig = {
            "orc_create": (C.c_void_p, [C.POINTER(OrcParams), _D, _D, C.c_int, C.c_int, C.c_int,
                                        C.c_double, C.c_double]),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_pinned_pow": (C.c_double, [C.c_double, C.c_double]),
            "orc_dims": (None, [C.c_void_p, _I, _D]),
            "orc_offsets": (None, [C.c_void_p, _D]),
            "orc_volume": (_D, [C.c_void_p]), "orc_error": (_D, [C.c_void_p]),
            "orc_weight": (_D, [C.c_void_p]), "orc_yest": (_D, [C.c_void_p]), "orc_counts": (_D, [C.c_void_p]),
            "orc_gain": (_D, [C.c_void_p]), "orc_offset": (_D, [C.c_void_p]),
            "orc_variance": (_D, [C.c_void_p]),
            "orc_detector_response": (_D, [C.c_void_p]), "orc_ht": (_D, [C.c_void_p]),
            "orc_voxel_profile": (_D, [C.c_void_p]), "orc_mag_map": (_D, [C.c_void_p]),
            "orc_amatrix_column": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _I, _D, C.c_int]),
            "orc_voxel_line_response": (C.c_int, [C.c_void_p, C.c_int, _I, _D, C.c_int]),
            "orc_init_volume": (None, [C.c_void_p, _D]),
            "orc_init_nuisance": (C.c_int, [C.c_void_p]),
            "orc_forward_project": (None, [C.c_void_p]),
            "orc_measurement_weight": (None, [C.c_void_p]),
            "orc_icd_sweep_reference": (None, [C.c_void_p, C.c_uint32, C.c_int, C.c_int, _D]),
            "orc_icd_sweep_reference_mt": (None, [C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_int,
                                                   _D]),
            "orc_icd_sweep_slices": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, _D]),
            "orc_icd_sweep_lines": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, _D]),
            "orc_joint_estimation": (C.c_int, [C.c_void_p]),
            "orc_set_bf_assist": (None, [C.c_void_p, _D]),
            "orc_update_weights": (None, [C.c_void_p]),
            "orc_cost": (C.c_double, [C.c_void_p, _D]),
            "orc_visit_order": (None, [C.c_uint32, C.c_int, C.c_int, _I]),
            "orc_run": (C.c_int, [C.c_void_p, C.c_uint32, _D, C.c_int]),
            "orc_run_seeded": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, _D, C.c_int]),
            "orc_selector": (_U8, [C.c_void_p]), "orc_filt_map": (_D, [C.c_void_p]),
            "orc_set_bragg": (None, [C.c_void_p, C.c_double]),
            "orc_get_bragg": (C.c_double, [C.c_void_p]),
            "orc_rand_list_perm": (None, [C.c_uint32, C.c_int, _I]),
            "orc_bf_sweep_lines": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, _D]),
            "orc_bf_sweep_slices": (None, [C.c_void_p, _U8, _I, C.c_int, C.c_int, C.c_int, _D]),
            "orc_bf_sweep_slices_order": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, _D]),
            "orc_bf_vsc": (None, [C.c_void_p]),
            "orc_bf_nh_threshold": (C.c_double, [C.c_void_p]),
            "orc_bf_nh_lines": (C.c_int, [C.c_void_p, C.c_double, _I]),
            "orc_roi_volume_sum": (C.c_double, [C.c_void_p]),
            "orc_roi_mag_sum": (C.c_double, [C.c_void_p]),
            "orc_bf_joint_estimation": (None, [C.c_void_p]),
            "orc_bf_update_weights": (None, [C.c_void_p]),
            "orc_bf_update_selector": (None, [C.c_void_p]),
            "orc_bf_cost": (C.c_double, [C.c_void_p, _D]),
            "orc_bf_run": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int]),
            "orc_bf_run_fixed_seed": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int]),
            "orc_icd_sweep_colour": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.c_int, C.c_int, _D]),
            "orc_view_sums": (None, [C.c_void_p, C.c_int, C.c_int, C.c_int, _D]),
            "orc_bf_reset_mag": (None, [C.c_void_p, _U8]),
            "orc_bf_sweep_colour": (None, [C.c_void_p, _U8, _I, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_int, C.c_int, _D]),
            "orc_bf_offset_sums": (None, [C.c_void_p, C.c_int, C.c_int, _D]),
            "orc_bf_apply_offsets": (None, [C.c_void_p, _D, C.c_int, C.c_int]),
            "orc_bf_variance_sums": (None, [C.c_void_p, C.c_int, C.c_int, _D]),
            "orc_bf_apply_variance": (None, [C.c_void_p, _D, C.c_int, C.c_int]),
            "orc_roi_volume_sum_range": (C.c_double, [C.c_void_p, C.c_int, C.c_int]),
            "orc_apply_nuisance": (None, [C.c_void_p, _D, _D, _D]),
            "orc_bf_sweep_lines_mt": (None, [C.c_void_p, _I, C.c_int, C.c_int, C.c_int, C.c_int,
                                             _D]),
        }
        for n, (r, a) in sig.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def params_from_mbir(p):
    """Map the engine's mbir_params (CLI-level) onto one oracle level."""
    o = OrcParams()
    levels = max(p.num_resolutions, 1)
    lvl = levels - 1 if (p.level < 0 or p.level >= levels) else p.level
    fres = max(p.final_resolution, 1)
    o.delta_xz_factor = 2.0 ** (levels - 1 - lvl) * fres
    o.interpolate_factor = 2.0 ** (levels - 1) * fres
    o.length_z = p.sample_thickness
    o.extend_object = p.extend_object
    o.x_shrink_factor = p.x_shrink_factor
    o.z_stretch = p.z_stretch
    o.response_bins = p.detector_response_bins
    o.profile_resolution = p.profile_resolution
    o.beam_resolution = p.beam_resolution
    o.compat_double_angle = p.compat_double_angle
    o.sigma_x = p.sigma_x
    o.mrf_p = p.qggmrf_p
    o.mrf_q = p.qggmrf_q if p.qggmrf_q != 0 else p.diffuseness + 1.0
    o.mrf_c = p.qggmrf_c
    o.mrf_alpha = p.qggmrf_alpha
    o.target_gain = p.target_gain
    o.default_offset = p.default_offset
    o.default_variance = p.default_variance
    o.default_recon_value = p.default_recon_value
    o.use_default_offset = p.use_default_offset
    o.joint_estimation = p.joint_estimation
    o.noise_model = p.noise_model
    o.zero_skipping = p.zero_skipping
    o.stop_threshold = p.stop_threshold
    o.outer_iterations = p.outer_iterations
    o.inner_iterations = p.inner_iterations
    o.threshold_reduction_factor = p.threshold_reduction_factor
    # the engine's reference-exact mode (FP64, reference order) evaluates powers by the
    # pinned method; the oracle does the same for that mode
    o.pinned_pow = 1 if (p.precision == 1 and p.order_mode == 1) else 0
    o.modality = p.modality
    o.noise_estimation = p.noise_estimation
    o.bragg_threshold = p.bragg_threshold
    o.bragg_delta = p.bragg_delta
    o.bf_offset = p.bf_offset
    o.nhicd = p.nhicd
    if p.modality == 1:
        # the BF command line turns the void dosage into the offset d = -log(dosage + bf_offset)
        # (BFReconstructionArgsParser.cpp:272-274)
        o.default_offset = -np.log(p.default_dosage + p.bf_offset) if p.use_default_offset else 0.0
    if getattr(p, "float_params", 0):
        # the pipeline's float members (HAADF_MultiResolutionReconstruction.h:76-89,
        # BFMultiResolutionReconstruction.h:76-107); p = diffuseness + 1 in float (:333)
        f32 = lambda v: float(np.float32(v))  # noqa: E731
        if p.qggmrf_q == 0:
            o.mrf_q = float(np.float32(np.float32(p.diffuseness) + np.float32(1.0)))
        for k in ("length_z", "sigma_x", "target_gain", "default_offset", "default_variance",
                  "default_recon_value", "stop_threshold", "bragg_threshold", "bragg_delta",
                  "bf_offset"):
            setattr(o, k, f32(getattr(o, k)))
    return o


class Oracle:
    def __init__(self, oparams, counts, tilts_deg, delta_r=1.0, delta_t=1.0):
        counts = np.ascontiguousarray(counts, np.float64)
        tilts = np.ascontiguousarray(tilts_deg, np.float64)
        self.shape = counts.shape
        self.params = oparams
        self._h = lib().orc_create(C.byref(oparams), counts.ctypes.data_as(_D),
                                   tilts.ctypes.data_as(_D), *counts.shape, delta_r, delta_t)
        d = np.zeros(3, np.int32)
        geo = np.zeros(8)
        lib().orc_dims(self._h, d.ctypes.data_as(_I), geo.ctypes.data_as(_D))
        self.nz, self.nx, self.ny = (int(v) for v in d)
        self.geo = geo

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def _view(self, fn, shape):
        p = fn(self._h)
        return np.ctypeslib.as_array(p, shape=shape)

    def volume(self):
        return self._view(lib().orc_volume, (self.nz, self.nx, self.ny))

    def error(self):
        return self._view(lib().orc_error, self.shape)

    def weight(self):
        return self._view(lib().orc_weight, self.shape)

    def yest(self):
        return self._view(lib().orc_yest, self.shape)

    def gain(self):
        return self._view(lib().orc_gain, (self.shape[0],))

    def offset(self):
        return self._view(lib().orc_offset, (self.shape[0],))

    def variance(self):
        return self._view(lib().orc_variance, (self.shape[0],))

    def detector_response(self):
        return self._view(lib().orc_detector_response, (self.shape[0], self.params.response_bins))

    def ht(self):
        return self._view(lib().orc_ht, (self.params.response_bins,))

    def offsets(self):
        o = np.zeros(2)
        lib().orc_offsets(self._h, o.ctypes.data_as(_D))
        return o

    def amatrix_column(self, z, x):
        cap = 64 * self.shape[0]
        idx = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        n = lib().orc_amatrix_column(self._h, z, x, idx.ctypes.data_as(_I),
                                     val.ctypes.data_as(_D), cap)
        return idx[:n].copy(), val[:n].copy()

    def voxel_line_response(self, y):
        val = np.zeros(16)
        t0 = C.c_int32()
        n = lib().orc_voxel_line_response(self._h, y, C.byref(t0), val.ctypes.data_as(_D), 16)
        return t0.value, val[:n].copy()

    def init_volume(self, vol=None):
        if vol is None:
            lib().orc_init_volume(self._h, None)
        else:
            v = np.ascontiguousarray(vol, np.float64)
            lib().orc_init_volume(self._h, v.ctypes.data_as(_D))

    def init_nuisance(self):
        return lib().orc_init_nuisance(self._h)

    def set_bf_assist(self, bf_counts):
        """HAADF with bright-field data: counts [theta][r][t] of the same size (None clears);
        before prepare."""
        if bf_counts is None:
            lib().orc_set_bf_assist(self._h, None)
            return
        b = np.ascontiguousarray(bf_counts, np.float64)
        assert b.shape == tuple(self.shape), (b.shape, self.shape)
        lib().orc_set_bf_assist(self._h, b.ctypes.data_as(_D))

    def prepare(self, vol=None):
        """volume init, nuisance init, forward projection, weights (execute() up to :691)."""
        self.init_volume(vol)
        self.init_nuisance()
        lib().orc_forward_project(self._h)
        lib().orc_measurement_weight(self._h)

    def forward_project(self):
        lib().orc_forward_project(self._h)

    def measurement_weight(self):
        lib().orc_measurement_weight(self._h)

    def sweep_reference(self, seed, outer=0, inner=0):
        st = np.zeros(4)
        lib().orc_icd_sweep_reference(self._h, seed, outer, inner, st.ctypes.data_as(_D))
        return st

    def sweep_reference_mt(self, seed, outer=0, inner=0, threads=None):
        st = np.zeros(4)
        n = threads or os.cpu_count() or 1
        lib().orc_icd_sweep_reference_mt(self._h, seed, outer, inner, n, st.ctypes.data_as(_D))
        return st

    def sweep_slices(self, row_order, stride, outer=0, inner=0):
        rows = np.ascontiguousarray(row_order, np.int32)
        st = np.zeros(4)
        lib().orc_icd_sweep_slices(self._h, rows.ctypes.data_as(_I), stride, outer, inner,
                                   st.ctypes.data_as(_D))
        return st

    def sweep_lines(self, lines, outer=0, inner=0):
        ln = np.ascontiguousarray(lines, np.int32)
        st = np.zeros(4)
        lib().orc_icd_sweep_lines(self._h, ln.ctypes.data_as(_I), len(ln), outer, inner,
                                  st.ctypes.data_as(_D))
        return st

    def joint_estimation(self):
        return lib().orc_joint_estimation(self._h)

    def update_weights(self):
        lib().orc_update_weights(self._h)

    def cost(self):
        parts = np.zeros(3)
        c = lib().orc_cost(self._h, parts.ctypes.data_as(_D))
        return c, parts

    # ---- y-slab sharding ---------------------------------------------------------------------
    def sweep_colour(self, row_order, stride, colour, y0, y1, outer=0, inner=0):
        rows = np.ascontiguousarray(row_order, np.int32)
        st = np.zeros(4)
        lib().orc_icd_sweep_colour(self._h, rows.ctypes.data_as(_I), stride, colour, y0, y1,
                                   outer, inner, st.ctypes.data_as(_D))
        return st

    def view_sums(self, kind, t0, t1):
        out = np.zeros(self.shape[0] * (6 if kind == 0 else 1))
        lib().orc_view_sums(self._h, kind, t0, t1, out.ctypes.data_as(_D))
        return out

    def apply_nuisance(self, gain, offset, variance=None):
        g = np.ascontiguousarray(gain, np.float64)
        o = np.ascontiguousarray(offset, np.float64)
        v = np.ascontiguousarray(variance, np.float64) if variance is not None else None
        lib().orc_apply_nuisance(self._h, g.ctypes.data_as(_D), o.ctypes.data_as(_D),
                                 v.ctypes.data_as(_D) if v is not None else None)

    # ---- bright field ---------------------------------------------------------------------
    def selector(self):
        return self._view(lib().orc_selector, self.shape)

    def mag_map(self):
        return self._view(lib().orc_mag_map, (self.nz, self.nx))

    def filt_map(self):
        return self._view(lib().orc_filt_map, (self.nz, self.nx))

    def set_bragg(self, t):
        lib().orc_set_bragg(self._h, t)

    def bragg(self):
        return lib().orc_get_bragg(self._h)

    def bf_sweep_lines(self, lines, outer=0, inner=0):
        lines = np.ascontiguousarray(lines, np.int32)
        st = np.zeros(4)
        lib().orc_bf_sweep_lines(self._h, lines.ctypes.data_as(_I), len(lines), outer, inner,
                                 st.ctypes.data_as(_D))
        return st

    def bf_sweep_slices(self, active, row_order, stride, outer=0, inner=0):
        active = np.ascontiguousarray(active, np.uint8)
        rows = np.ascontiguousarray(row_order, np.int32)
        st = np.zeros(4)
        lib().orc_bf_sweep_slices(self._h, active.ctypes.data_as(_U8), rows.ctypes.data_as(_I),
                                  stride, outer, inner, st.ctypes.data_as(_D))
        return st

    def bf_reset_mag(self, active):
        a = np.ascontiguousarray(active, np.uint8)
        lib().orc_bf_reset_mag(self._h, a.ctypes.data_as(_U8))

    def bf_sweep_colour(self, active, row_order, stride, colour, y0, y1, outer=0, inner=0):
        active = np.ascontiguousarray(active, np.uint8)
        rows = np.ascontiguousarray(row_order, np.int32)
        st = np.zeros(4)
        lib().orc_bf_sweep_colour(self._h, active.ctypes.data_as(_U8), rows.ctypes.data_as(_I),
                                  stride, colour, y0, y1, outer, inner, st.ctypes.data_as(_D))
        return st

    def bf_offset_sums(self, t0, t1):
        out = np.zeros(2 * self.shape[0])
        lib().orc_bf_offset_sums(self._h, t0, t1, out.ctypes.data_as(_D))
        return out

    def bf_apply_offsets(self, sums, t0, t1):
        s = np.ascontiguousarray(sums, np.float64)
        lib().orc_bf_apply_offsets(self._h, s.ctypes.data_as(_D), t0, t1)

    def bf_variance_sums(self, t0, t1):
        out = np.zeros(3)
        lib().orc_bf_variance_sums(self._h, t0, t1, out.ctypes.data_as(_D))
        return out

    def bf_apply_variance(self, sums, t0, t1):
        s = np.ascontiguousarray(sums, np.float64)
        lib().orc_bf_apply_variance(self._h, s.ctypes.data_as(_D), t0, t1)

    def roi_volume_sum_range(self, y0, y1):
        return lib().orc_roi_volume_sum_range(self._h, y0, y1)

    def bf_sweep_slices_order(self, lines, outer=0, inner=0):
        """The slice-parallel call with every slice visiting `lines` in the given order."""
        lines = np.ascontiguousarray(lines, np.int32)
        st = np.zeros(4)
        lib().orc_bf_sweep_slices_order(self._h, lines.ctypes.data_as(_I), len(lines), outer,
                                        inner, st.ctypes.data_as(_D))
        return st

    def bf_sweep_lines_mt(self, lines, outer=0, inner=0, threads=None):
        lines = np.ascontiguousarray(lines, np.int32)
        st = np.zeros(4)
        lib().orc_bf_sweep_lines_mt(self._h, lines.ctypes.data_as(_I), len(lines), outer, inner,
                                    threads or os.cpu_count() or 1, st.ctypes.data_as(_D))
        return st

    def bf_vsc(self):
        lib().orc_bf_vsc(self._h)

    def bf_nh_threshold(self):
        return lib().orc_bf_nh_threshold(self._h)

    def bf_nh_lines(self, threshold):
        out = np.zeros(self.nz * self.nx, np.int32)
        n = lib().orc_bf_nh_lines(self._h, threshold, out.ctypes.data_as(_I))
        return out[:n]

    def roi_volume_sum(self):
        return lib().orc_roi_volume_sum(self._h)

    def roi_mag_sum(self):
        return lib().orc_roi_mag_sum(self._h)

    def bf_joint_estimation(self):
        lib().orc_bf_joint_estimation(self._h)

    def bf_update_weights(self):
        lib().orc_bf_update_weights(self._h)

    def bf_update_selector(self):
        lib().orc_bf_update_selector(self._h)

    def bf_cost(self):
        parts = np.zeros(3)
        c = lib().orc_bf_cost(self._h, parts.ctypes.data_as(_D))
        return c, parts

    def bf_run(self, seed, max_calls=0):
        return lib().orc_bf_run(self._h, seed, max_calls)

    def bf_run_fixed_seed(self, seed, max_calls=0):
        """bf_run with every list drawn from `seed` (the reference with its clock seed frozen)."""
        return lib().orc_bf_run_fixed_seed(self._h, seed, max_calls)

    def measured(self):
        """The measurements the engine works on (BF: -log(counts + bf_offset) once prepared)."""
        return self._view(lib().orc_counts, self.shape)

    def run(self, seed, n_cost=0, seed_step=0):
        """execute()'s loops; sweep k visits in the order of seed + k * seed_step."""
        log = np.zeros(max(n_cost, 1))
        n = lib().orc_run_seeded(self._h, seed, seed_step,
                                 log.ctypes.data_as(_D) if n_cost else None, n_cost)
        return n, log[:min(n, n_cost)]


def visit_order(seed, nz, nx):
    out = np.zeros(nz * nx, np.int32)
    lib().orc_visit_order(seed, nz, nx, out.ctypes.data_as(_I))
    return out


def rand_list_perm(seed, n):
    """GenRandList's permutation: element i of a list goes to position out[i]."""
    out = np.zeros(max(n, 1), np.int32)
    lib().orc_rand_list_perm(seed, n, out.ctypes.data_as(_I))
    return out[:n]


def pinned_pow(x, y):
    """x**y by the oracle's pinned double-double method (see mbir_oracle.c)."""
    return lib().orc_pinned_pow(float(x), float(y))
