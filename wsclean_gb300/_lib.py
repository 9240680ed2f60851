"""ctypes binding of the C ABI declared in include/wgpu.h.

The shared library is the in-tree build wsclean_gb300/_build/libwgpu.so.  There
is no fallback: if the library is missing or cannot load, every entry point
raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwgpu.so")

WGPU_OK = 0
WGPU_ERR_INVALID = -1
WGPU_ERR_CUDA = -2
WGPU_ERR_NOMEM = -3
WGPU_ERR_STATE = -4
WGPU_ERR_TIMEOUT = -5

NOALLOC_MAX_VISIBILITIES = 1 << 20
NOALLOC_MAX_CHANNELS = 4096

GAIN_XX, GAIN_YY, GAIN_TRACE, GAIN_2VIS_DIAGONAL, GAIN_FULL = range(5)
(POL_I, POL_Q, POL_U, POL_V, POL_XX, POL_XY, POL_YX, POL_YY, POL_RR, POL_RL, POL_LR, POL_LL,
 POL_FULL_STOKES, POL_INSTRUMENTAL, POL_DIAGONAL_INSTRUMENTAL) = range(15)


class WgpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"wgpu status {status}: {message}")
        self.status = status


class Plan(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "width", "height", "nu", "nv", "support", "tile", "n_planes", "plane_batch",
        "fft_n1", "fft_n2")] + [(n, C.c_double) for n in (
        "sigma", "beta", "dl", "dm", "l_shift", "m_shift", "w0", "dw", "nm1_min",
        "nm1_max", "nm1_center", "est_error", "est_seconds")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PlanRequest(C.Structure):
    _fields_ = [("width", C.c_int64), ("height", C.c_int64), ("dl", C.c_double),
                ("dm", C.c_double), ("l_shift", C.c_double), ("m_shift", C.c_double),
                ("epsilon", C.c_double), ("w_min", C.c_double), ("w_max", C.c_double),
                ("n_vis", C.c_int64), ("sigma_min", C.c_double), ("sigma_max", C.c_double),
                ("force_support", C.c_int64), ("force_sigma", C.c_double),
                ("force_tile", C.c_int64), ("max_plane_batch", C.c_int64),
                ("memory_budget_bytes", C.c_double)]


class TuningTrial(C.Structure):
    """wgpu_tuning_trial_t: one candidate plan timed by a tuning gridder."""
    _fields_ = [("support", C.c_int64), ("sigma", C.c_double), ("nu", C.c_int64),
                ("nv", C.c_int64), ("n_planes", C.c_int64), ("est_seconds", C.c_double),
                ("measured_ms", C.c_double), ("chosen", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Request(C.Structure):
    """wgpu_request_t: one inversion or prediction request for the server."""
    _fields_ = [("kind", C.c_int), ("session", C.c_uint64),
                ("width", C.c_size_t), ("height", C.c_size_t),
                ("width_t", C.c_size_t), ("height_t", C.c_size_t),
                ("pixel_size_x", C.c_double), ("pixel_size_y", C.c_double),
                ("l_shift", C.c_double), ("m_shift", C.c_double), ("epsilon", C.c_double),
                ("n_rows", C.c_size_t), ("n_chan", C.c_size_t),
                ("uvw", C.c_void_p), ("freq", C.c_void_p), ("mask", C.c_void_p),
                ("vis", C.c_void_p), ("image_factor", C.c_double),
                ("image_out", C.c_void_p), ("model", C.c_void_p), ("vis_out", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("failed", C.c_uint64), ("queued", C.c_uint64),
                ("running", C.c_uint64), ("peak_running", C.c_uint64),
                ("device_bytes_in_use", C.c_double), ("peak_device_bytes", C.c_double),
                ("visibilities", C.c_double), ("elapsed_s", C.c_double),
                ("held_for_memory", C.c_uint64)]


class Facet(C.Structure):
    """wgpu_facet_t: one facet of a facet batch."""
    _fields_ = [("width", C.c_size_t), ("height", C.c_size_t),
                ("pixel_size_x", C.c_double), ("pixel_size_y", C.c_double),
                ("l_shift", C.c_double), ("m_shift", C.c_double)]


class FacetsInfo(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("n_jobs", "n_waves", "support", "graph_kernels",
                                           "image_elems")] + \
               [("job_visibilities", C.c_double), ("last_ms", C.c_double),
                ("bind_ms", C.c_double * 4)]


class RowWeighting(C.Structure):
    """wgpu_row_weighting_t: the settings CalculateWeightsImplementation reads."""
    _fields_ = [("psf_mode", C.c_int), ("psf_dl", C.c_double), ("psf_dm", C.c_double),
                ("subtract_model", C.c_int), ("visibility_weighting", C.c_int),
                ("polarization", C.c_int)]


class WeightSums(C.Structure):
    """wgpu_weight_sums_t: the sums ApplyWeights accumulates."""
    _fields_ = [("visibility_weight_sum", C.c_double), ("max_gridded_weight", C.c_double),
                ("total_weight", C.c_double), ("gridded_visibility_count", C.c_uint64)]


REQUEST_INVERT = 1
REQUEST_PREDICT = 2

WEIGHT_NATURAL, WEIGHT_UNIFORM, WEIGHT_BRIGGS = range(3)
VISW_NORMAL, VISW_SQUARED, VISW_UNIT = range(3)
PSF_NONE, PSF_SINGLE, PSF_DIRECTION_DEPENDENT = range(3)
(TAPER_MIN_UV, TAPER_MAX_UV, TAPER_TUKEY, TAPER_TUKEY_INNER, TAPER_EDGE, TAPER_EDGE_TUKEY,
 TAPER_GAUSSIAN, TAPER_RANK_FILTER) = range(8)

_lib = None

P = C.c_void_p
SZ = C.c_size_t
D = C.c_double
I = C.c_int

_PROTOS = {
    "wgpu_last_error": (C.c_char_p, []),
    "wgpu_version": (C.c_char_p, []),
    "wgpu_gain_mode_n_visibilities": (SZ, [I]),
    "wgpu_select_gain_mode": (I, [I, SZ, C.POINTER(I)]),
    "wgpu_plan_make": (I, [C.POINTER(PlanRequest), C.POINTER(Plan)]),
    "wgpu_plan_candidates": (I, [C.POINTER(PlanRequest), C.POINTER(Plan), I, C.POINTER(I)]),
    "wgpu_gridder_last_tuning": (I, [P, C.POINTER(TuningTrial), I, C.POINTER(I)]),
    "wgpu_tuning_cache_clear": (None, []),
    "wgpu_gridder_create": (I, [SZ, SZ, SZ, SZ, D, D, D, D, SZ, D, SZ, I, I, C.POINTER(P)]),
    "wgpu_gridder_destroy": (None, [P]),
    "wgpu_gridder_constant_memory": (SZ, [P]),
    "wgpu_gridder_per_visibility_memory": (SZ, [P]),
    "wgpu_gridder_initialize_inversion": (I, [P]),
    "wgpu_gridder_add_inversion_data": (I, [P, SZ, SZ, P, P, P]),
    "wgpu_gridder_add_inversion_data_device": (I, [P, SZ, SZ, P, P, P]),
    "wgpu_gridder_add_inversion_data_corrected": (
        I, [P, I, SZ, SZ, P, P, SZ, P, P, P, P, SZ, SZ, SZ, I]),
    "wgpu_gridder_predict_visibilities_corrected": (
        I, [P, I, SZ, SZ, P, P, SZ, P, P, P, SZ, SZ, SZ, I, P]),
    "wgpu_gridder_finalize_image": (I, [P, D]),
    "wgpu_gridder_real_image": (I, [P, P]),
    "wgpu_gridder_initialize_prediction": (I, [P, P]),
    "wgpu_gridder_predict_visibilities": (I, [P, SZ, SZ, P, P, P]),
    "wgpu_gridder_predict_visibilities_device": (I, [P, SZ, SZ, P, P, P]),
    "wgpu_gridder_predict_visibilities_masked": (I, [P, SZ, SZ, P, P, P, P]),
    "wgpu_gridder_predict_visibilities_masked_device": (I, [P, SZ, SZ, P, P, P, P]),
    "wgpu_gridder_last_plan": (I, [P, C.POINTER(Plan)]),
    "wgpu_gridder_last_timings": (I, [P, C.POINTER(C.c_double), C.POINTER(I), I, C.c_char_p,
                                      SZ, C.POINTER(I)]),
    "wgpu_gridder_pin_plan": (I, [P, C.POINTER(Plan)]),
    "wgpu_gridder_bind": (I, [P, SZ, SZ, P, P, P]),
    "wgpu_gridder_unbind": (I, [P]),
    "wgpu_gridder_invert_bound": (I, [P, P]),
    "wgpu_gridder_invert_bound_device": (I, [P, P]),
    "wgpu_gridder_predict_bound": (I, [P, P]),
    "wgpu_gridder_predict_bound_device": (I, [P, P]),
    "wgpu_gridder_set_plane_budget": (I, [P, D]),
    "wgpu_gridder_stream": (P, [P]),
    "wgpu_kernel_launch_count": (C.c_uint64, []),
    "wgpu_selftest_bounded_wait": (I, [D]),
    "wgpu_bucket_debug": (I, [C.POINTER(Plan), SZ, SZ, P, P, P, I, P, P, P, P, P, P, P, P,
                              C.POINTER(C.c_int64)]),
    "wgpu_bucket_debug_rows": (I, [C.POINTER(Plan), SZ, SZ, P, P, P, I, P, P, P]),
    "wgpu_bucket_noalloc": (I, [C.POINTER(Plan), SZ, SZ, P, P, P, I, P, P, P, P,
                                C.POINTER(C.c_int64)]),
    "wgpu_bucket_noalloc_scratch_bytes": (SZ, []),
    "wgpu_server_create": (I, [D, I, D, C.POINTER(P)]),
    "wgpu_server_submit": (I, [P, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "wgpu_server_wait": (I, [P, C.c_uint64, C.POINTER(D), C.POINTER(D)]),
    "wgpu_server_close_session": (I, [P, C.c_uint64]),
    "wgpu_server_stats": (I, [P, C.POINTER(ServerStats)]),
    "wgpu_server_destroy": (None, [P]),
    "wgpu_facets_create": (I, [C.POINTER(Facet), SZ, C.POINTER(SZ), SZ, D, D, C.POINTER(P)]),
    "wgpu_facets_bind": (I, [P, SZ, SZ, P, P]),
    "wgpu_facets_invert": (I, [P, P, P]),
    "wgpu_facets_invert_device": (I, [P, P, P]),
    "wgpu_facets_bind_corrected": (I, [P, SZ, SZ, P, P]),
    "wgpu_facets_invert_corrected": (I, [P, I, SZ, P, P, P, P, SZ, SZ, SZ, I, P]),
    "wgpu_facets_info": (I, [P, C.POINTER(FacetsInfo)]),
    "wgpu_facets_job_plan": (I, [P, SZ, C.POINTER(Plan)]),
    "wgpu_facets_stream": (P, [P]),
    "wgpu_facets_destroy": (None, [P]),
    "wgpu_imageweights_create": (I, [I, D, SZ, SZ, D, D, I, D, C.POINTER(P)]),
    "wgpu_imageweights_destroy": (None, [P]),
    "wgpu_imageweights_grid": (I, [P, SZ, SZ, SZ, P, P, P]),
    "wgpu_imageweights_grid_device": (I, [P, SZ, SZ, SZ, P, P, P]),
    "wgpu_imageweights_stream": (P, [P]),
    "wgpu_imageweights_finish": (I, [P]),
    "wgpu_imageweights_taper": (I, [P, I, D, D]),
    "wgpu_imageweights_set_all": (I, [P, D]),
    "wgpu_imageweights_get": (I, [P, I, P]),
    "wgpu_imageweights_info": (I, [P, C.POINTER(SZ), C.POINTER(SZ), C.POINTER(D)]),
    "wgpu_imageweights_sample": (I, [P, SZ, P, P, P]),
    "wgpu_prepare_rows": (I, [P, C.POINTER(RowWeighting), SZ, SZ, SZ, P, P, P, P, P, P, P, P,
                              P, C.POINTER(WeightSums)]),
    "wgpu_prepare_rows_device": (I, [P, C.POINTER(RowWeighting), SZ, SZ, SZ, P, P, P, P, P, P,
                                     P, P, P, C.POINTER(WeightSums)]),
    "wgpu_gridder_add_inversion_rows_corrected": (
        I, [P, P, C.POINTER(RowWeighting), I, SZ, SZ, SZ, P, P, P, P, P, P, P, P, P, SZ, SZ, SZ,
            C.POINTER(WeightSums), P]),
    "wgpu_calculate_fft_size": (I, [SZ, D, D, C.POINTER(SZ), C.POINTER(SZ)]),
    "wgpu_small_inversion_size": (I, [SZ, SZ, D, D, D, C.POINTER(SZ), C.POINTER(SZ),
                                      C.POINTER(D), C.POINTER(D)]),
    "wgpu_actual_trimmed_size": (I, [SZ, SZ, D, C.POINTER(SZ), C.POINTER(SZ)]),
    "wgpu_resample": (I, [P, SZ, SZ, P, SZ, SZ]),
    "wgpu_resample_device": (I, [P, SZ, SZ, P, SZ, SZ, P]),
    "wgpu_gridder_finish_inversion": (I, [P, SZ, SZ, SZ, SZ, P]),
    "wgpu_gridder_start_predict": (I, [P, SZ, SZ, SZ, SZ, P]),
    "wgpu_gridder_add_inversion_rows": (I, [P, P, C.POINTER(RowWeighting), SZ, SZ, SZ, P, P,
                                            P, P, P, P, C.POINTER(WeightSums)]),
}


def lib():
    """Loads libwgpu.so (building nothing); raises if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise WgpuError(WGPU_ERR_CUDA, f"{LIB_PATH} is missing; run "
                            "python -m wsclean_gb300.build")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def gain_mode_n_visibilities(mode):
    """GetNVisibilities (gridding/gainmode.h:33-46)."""
    return int(lib().wgpu_gain_mode_n_visibilities(mode))


def select_gain_mode(polarization, n_visibility_polarizations):
    """SelectGainMode (gridding/gainmode.h:52-95); raises WgpuError for the
    combinations the reference rejects."""
    m = C.c_int()
    check(lib().wgpu_select_gain_mode(polarization, n_visibility_polarizations, C.byref(m)))
    return m.value


def exported_symbols():
    return list(_PROTOS)


def check(status):
    if status != WGPU_OK:
        msg = lib().wgpu_last_error().decode(errors="replace")
        raise WgpuError(status, msg)


def ptr(a):
    """Address of a numpy array's data (None for None)."""
    return None if a is None else a.ctypes.data


def make_plan(**kw):
    r = PlanRequest()
    for k, v in kw.items():
        setattr(r, k, v)
    p = Plan()
    check(lib().wgpu_plan_make(C.byref(r), C.byref(p)))
    return p


def plan_candidates(max_plans=64, **kw):
    """The plans meeting the request's epsilon, lowest cost-model time first."""
    r = PlanRequest()
    for k, v in kw.items():
        setattr(r, k, v)
    out = (Plan * max_plans)()
    n = C.c_int()
    check(lib().wgpu_plan_candidates(C.byref(r), out, max_plans, C.byref(n)))
    return [out[i] for i in range(n.value)]


def tuning_cache_clear():
    lib().wgpu_tuning_cache_clear()
