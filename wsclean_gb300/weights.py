"""Imaging weights and raw-row weighting on the GPU.

``ImageWeights`` mirrors WSClean's ImageWeights (structures/imageweights.h):
the same constructor arguments and method names (Grid, FinishGridding, the
tapers, RankFilter, GetWeight, GetGrid), with the grid held on the device.
``prepare_rows`` and ``WGriddingGridder_Simple.AddInversionRows`` run
MsGridderData's CalculateWeights + ApplyWeights + CollapseData
(gridding/msgridderdata.h:36-52, 760-886) on raw measurement-set rows.  Every
call goes through the C ABI (include/wgpu.h) to the CUDA kernels.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib, ptr

NATURAL, UNIFORM, BRIGGS = _lib.WEIGHT_NATURAL, _lib.WEIGHT_UNIFORM, _lib.WEIGHT_BRIGGS


class ImageWeights:
    """ImageWeights(weightMode, imageWidth, imageHeight, pixelScaleX,
    pixelScaleY, weightsAsTaper, superWeight) (imageweights.cpp:34-49);
    ``mode`` is NATURAL, UNIFORM or BRIGGS and ``briggs_robustness`` the
    Briggs robustness."""

    def __init__(self, mode, image_width, image_height, pixel_scale_x, pixel_scale_y,
                 weights_as_taper=False, super_weight=1.0, briggs_robustness=0.0):
        h = C.c_void_p()
        check(lib().wgpu_imageweights_create(int(mode), float(briggs_robustness), image_width,
                                             image_height, float(pixel_scale_x),
                                             float(pixel_scale_y), int(bool(weights_as_taper)),
                                             float(super_weight), C.byref(h)))
        self._h = h
        w, hh = C.c_size_t(), C.c_size_t()
        check(lib().wgpu_imageweights_info(self._h, C.byref(w), C.byref(hh), None))
        self._width, self._height = w.value, hh.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().wgpu_imageweights_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def Width(self):
        return self._width

    def Height(self):
        return self._height

    def TotalSum(self):
        t = C.c_double()
        check(lib().wgpu_imageweights_info(self._h, None, None, C.byref(t)))
        return t.value

    def Grid(self, uvw, frequencies, weights):
        """Grid(MSProvider &, BandData) over one chunk of rows: uvw (rows, 3)
        metres, frequencies (chans,) Hz, weights (rows, chans, pols)."""
        uvw = np.ascontiguousarray(uvw, np.float64)
        freq = np.ascontiguousarray(frequencies, np.float64)
        wts = np.ascontiguousarray(weights, np.float32)
        n_rows, n_chan = uvw.shape[0], freq.size
        n_pol = wts.size // (n_rows * n_chan) if n_rows * n_chan else 1
        assert wts.size == n_rows * n_chan * n_pol
        check(lib().wgpu_imageweights_grid(self._h, n_rows, n_chan, n_pol, ptr(uvw), ptr(freq),
                                           ptr(wts)))

    def grid_device(self, n_rows, n_chan, n_pol, d_uvw, d_freq, d_weights):
        """Grid with device-resident inputs (integer device addresses, e.g.
        torch tensor data_ptr()), on this object's stream."""
        check(lib().wgpu_imageweights_grid_device(self._h, n_rows, n_chan, n_pol, d_uvw, d_freq,
                                                  d_weights))

    def stream(self):
        """The CUDA stream the weight kernels run on (an integer handle)."""
        return lib().wgpu_imageweights_stream(self._h)

    def FinishGridding(self):
        check(lib().wgpu_imageweights_finish(self._h))

    def _taper(self, kind, a, b=0.0):
        check(lib().wgpu_imageweights_taper(self._h, kind, float(a), float(b)))

    def SetMinUVRange(self, min_uv_in_lambda):
        self._taper(_lib.TAPER_MIN_UV, min_uv_in_lambda)

    def SetMaxUVRange(self, max_uv_in_lambda):
        self._taper(_lib.TAPER_MAX_UV, max_uv_in_lambda)

    def SetTukeyTaper(self, transition_size_in_lambda, max_uv_in_lambda):
        self._taper(_lib.TAPER_TUKEY, transition_size_in_lambda, max_uv_in_lambda)

    def SetTukeyInnerTaper(self, transition_size_in_lambda, min_uv_in_lambda):
        self._taper(_lib.TAPER_TUKEY_INNER, transition_size_in_lambda, min_uv_in_lambda)

    def SetEdgeTaper(self, size_in_lambda):
        self._taper(_lib.TAPER_EDGE, size_in_lambda)

    def SetEdgeTukeyTaper(self, transition_size_in_lambda, edge_size_in_lambda):
        self._taper(_lib.TAPER_EDGE_TUKEY, transition_size_in_lambda, edge_size_in_lambda)

    def SetGaussianTaper(self, beam_size):
        self._taper(_lib.TAPER_GAUSSIAN, beam_size)

    def RankFilter(self, rank_limit, window_size):
        self._taper(_lib.TAPER_RANK_FILTER, rank_limit, int(window_size))

    def SetAllValues(self, value):
        check(lib().wgpu_imageweights_set_all(self._h, float(value)))

    def GetWeight(self, u, v):
        """GetWeight for scalars or arrays of (u, v) in wavelengths."""
        scalar = np.ndim(u) == 0
        ua = np.ascontiguousarray(np.atleast_1d(u), np.float64).ravel()
        va = np.ascontiguousarray(np.atleast_1d(v), np.float64).ravel()
        out = np.empty(ua.size, np.float64)
        check(lib().wgpu_imageweights_sample(self._h, ua.size, ptr(ua), ptr(va), ptr(out)))
        return float(out[0]) if scalar else out

    def GetGrid(self):
        """The (height, width) image of GetGrid (imageweights.cpp:284-300)."""
        out = np.empty((self._height, self._width), np.float64)
        check(lib().wgpu_imageweights_get(self._h, 1, ptr(out)))
        return out

    def half_grid(self):
        """The stored (height / 2, width) half-plane."""
        out = np.empty((self._height // 2, self._width), np.float64)
        check(lib().wgpu_imageweights_get(self._h, 0, ptr(out)))
        return out


def row_weighting(psf_mode=_lib.PSF_NONE, psf_dl=0.0, psf_dm=0.0, subtract_model=False,
                  visibility_weighting=_lib.VISW_NORMAL, polarization=_lib.POL_I):
    return _lib.RowWeighting(int(psf_mode), float(psf_dl), float(psf_dm), int(bool(subtract_model)),
                             int(visibility_weighting), int(polarization))


def _row_inputs(uvw, frequencies, weights, vis, model, selected, rw):
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(frequencies, np.float64)
    wts = np.ascontiguousarray(weights, np.float32)
    n_rows, n_chan, n_pol = wts.shape
    assert uvw.shape == (n_rows, 3) and freq.size == n_chan
    vis_a = None if rw.psf_mode != _lib.PSF_NONE else np.ascontiguousarray(vis, np.complex64)
    mod_a = np.ascontiguousarray(model, np.complex64) if rw.subtract_model else None
    sel_a = None if selected is None else np.ascontiguousarray(selected, np.uint8)
    for a, shape in ((vis_a, wts.shape), (mod_a, wts.shape), (sel_a, (n_rows, n_chan))):
        assert a is None or a.shape == shape
    return uvw, freq, wts, vis_a, mod_a, sel_a, (n_rows, n_chan, n_pol)


def sums_dict(s):
    return {"visibility_weight_sum": s.visibility_weight_sum,
            "max_gridded_weight": s.max_gridded_weight, "total_weight": s.total_weight,
            "gridded_visibility_count": s.gridded_visibility_count}


def prepare_rows(image_weights, uvw, frequencies, weights, vis=None, model=None, selected=None,
                 **settings):
    """CalculateWeights + ApplyWeights + CollapseData on the GPU for rows
    without corrections.  weights / vis / model are (rows, chans, pols),
    selected (rows, chans).  ``settings`` are the fields of row_weighting().
    Returns (vis_out (rows, chans) complex64, cumulative weights (rows, chans,
    pols), imaging weights (rows, chans), sums dict)."""
    rw = row_weighting(**settings)
    uvw, freq, wts, vis_a, mod_a, sel_a, (n_rows, n_chan, n_pol) = _row_inputs(
        uvw, frequencies, weights, vis, model, selected, rw)
    vis_out = np.empty((n_rows, n_chan), np.complex64)
    w_out = np.empty((n_rows, n_chan, n_pol), np.float32)
    iw_out = np.empty((n_rows, n_chan), np.float32)
    sums = _lib.WeightSums()
    check(lib().wgpu_prepare_rows(image_weights.handle, C.byref(rw), n_pol, n_rows, n_chan,
                                  ptr(uvw), ptr(freq), ptr(vis_a), ptr(wts), ptr(mod_a),
                                  ptr(sel_a), ptr(vis_out), ptr(w_out), ptr(iw_out),
                                  C.byref(sums)))
    return vis_out, w_out, iw_out, sums_dict(sums)


def add_inversion_rows(gridder, image_weights, uvw, frequencies, weights, vis=None, model=None,
                       selected=None, sums=None, **settings):
    """GetCollapsedVisibilities + AddInversionData on the device for one
    chunk of raw rows; returns the accumulated sums (a WeightSums)."""
    rw = row_weighting(**settings)
    uvw, freq, wts, vis_a, mod_a, sel_a, (n_rows, n_chan, n_pol) = _row_inputs(
        uvw, frequencies, weights, vis, model, selected, rw)
    if sums is None:
        sums = _lib.WeightSums()
    check(lib().wgpu_gridder_add_inversion_rows(gridder._h, image_weights.handle, C.byref(rw),
                                                n_pol, n_rows, n_chan, ptr(uvw), ptr(freq),
                                                ptr(vis_a), ptr(wts), ptr(mod_a), ptr(sel_a),
                                                C.byref(sums)))
    return sums


def prepare_rows_device(image_weights, n_pol, n_rows, n_chan, d_uvw, d_freq, d_weights, d_vis_out,
                        d_vis=None, d_model=None, d_selected=None, d_weights_out=None,
                        d_imaging_out=None, **settings):
    """prepare_rows on device buffers (integer device addresses), on the image
    weights' stream; returns the sums dict."""
    rw = row_weighting(**settings)
    sums = _lib.WeightSums()
    check(lib().wgpu_prepare_rows_device(image_weights.handle, C.byref(rw), n_pol, n_rows, n_chan,
                                         d_uvw, d_freq, d_vis, d_weights, d_model, d_selected,
                                         d_vis_out, d_weights_out, d_imaging_out, C.byref(sums)))
    return sums_dict(sums)


def add_inversion_rows_corrected(gridder, image_weights, mode, uvw, frequencies, weights, vis,
                                 antennas, time_offsets, solutions, nparms, n_times, n_antenna,
                                 model=None, selected=None, sums=None, with_correction_sum=False,
                                 **settings):
    """GetCollapsedVisibilities with h5parm corrections + AddInversionData on
    the device (wgpu_gridder_add_inversion_rows_corrected).  Returns (sums,
    correction sum or None): with with_correction_sum a float for TRACE and a
    4 x 4 complex Hermitian matrix for the other modes."""
    rw = row_weighting(**settings)
    uvw, freq, wts, vis_a, mod_a, sel_a, (n_rows, n_chan, n_pol) = _row_inputs(
        uvw, frequencies, weights, vis, model, selected, rw)
    ant = np.ascontiguousarray(antennas, np.uint64)
    tof = np.ascontiguousarray(time_offsets, np.uint64)
    sol = np.ascontiguousarray(solutions, np.complex64)
    if sums is None:
        sums = _lib.WeightSums()
    corr = np.zeros(32, np.float64)
    check(lib().wgpu_gridder_add_inversion_rows_corrected(
        gridder._h, image_weights.handle, C.byref(rw), int(mode), n_pol, n_rows, n_chan, ptr(uvw),
        ptr(freq), ptr(vis_a), ptr(wts), ptr(mod_a), ptr(sel_a), ptr(ant), ptr(tof), ptr(sol),
        nparms, n_times, n_antenna, C.byref(sums), ptr(corr) if with_correction_sum else None))
    if not with_correction_sum:
        return sums, None
    if mode == _lib.GAIN_TRACE:
        return sums, float(corr[0])
    return sums, (corr[0::2] + 1j * corr[1::2]).reshape(4, 4)
