"""Python mirror of WSClean's WGriddingGridder_Simple<NumT> (wgridder/gridder_simple.h).

Method names, argument meaning and call order follow the reference class; every
call goes through the C ABI (include/wgpu.h) to the CUDA path.  numpy arrays are
used for the host buffers; device-pointer variants take raw integer addresses
(for example from torch tensors) and run on the gridder's stream.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib, ptr

GainMode = {"xx": _lib.GAIN_XX, "yy": _lib.GAIN_YY, "trace": _lib.GAIN_TRACE,
            "diagonal": _lib.GAIN_2VIS_DIAGONAL, "full": _lib.GAIN_FULL}


def _c64(a):
    a = np.ascontiguousarray(a, dtype=np.complex64)
    return a


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class WGriddingGridder_Simple:
    """GPU w-gridder with the reference's interface (gridder_simple.h:54-245).

    ``num_t`` is np.float32 or np.float64, the type of the accumulated image
    (WSClean picks double when epsilon <= 1.01e-5, wgriddingmsgridder.cpp:43-53).
    """

    sigma_min = 1.1
    sigma_max = 2.0

    def __init__(self, width, height, width_t, height_t, pixel_size_x, pixel_size_y,
                 l_shift, m_shift, nthreads, epsilon=1e-4, verbosity=0, tuning=False,
                 num_t=np.float32):
        self.width, self.height = int(width), int(height)
        self.width_t, self.height_t = int(width_t), int(height_t)
        prec = np.dtype(num_t).itemsize
        h = C.c_void_p()
        check(lib().wgpu_gridder_create(self.width, self.height, self.width_t, self.height_t,
                                        float(pixel_size_x), float(pixel_size_y),
                                        float(l_shift), float(m_shift), int(nthreads),
                                        float(epsilon), int(verbosity), 1 if tuning else 0,
                                        prec, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().wgpu_gridder_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # gridder_simple_implementation.h:53-68
    def ConstantMemoryUsage(self):
        return lib().wgpu_gridder_constant_memory(self._h)

    def PerVisibilityMemoryUsage(self):
        return lib().wgpu_gridder_per_visibility_memory(self._h)

    def InitializeInversion(self):
        check(lib().wgpu_gridder_initialize_inversion(self._h))

    def AddInversionData(self, n_rows, n_chan, uvw, freq, vis):
        uvw, freq, vis = _f64(uvw), _f64(freq), _c64(vis)
        assert uvw.size == 3 * n_rows and freq.size == n_chan and vis.size == n_rows * n_chan
        check(lib().wgpu_gridder_add_inversion_data(self._h, n_rows, n_chan, ptr(uvw),
                                                    ptr(freq), ptr(vis)))

    def AddInversionDataDevice(self, n_rows, n_chan, d_uvw, d_freq, d_vis):
        check(lib().wgpu_gridder_add_inversion_data_device(self._h, n_rows, n_chan, d_uvw,
                                                           d_freq, d_vis))

    def AddInversionDataWithCorrectionCallback(self, mode, n_polarizations, n_rows, uvws,
                                               frequencies, n_channels, antennas,
                                               visibilities, time_offsets, solutions,
                                               nparms, n_times, n_antenna,
                                               polarization=_lib.POL_I):
        """gridder_simple_implementation.h:92-110 with the correction data passed
        explicitly (solution table instead of an MsGridder callback)."""
        if isinstance(mode, str):
            mode = GainMode[mode]
        uvws, frequencies = _f64(uvws), _f64(frequencies)
        vis = _c64(visibilities)
        ant = np.ascontiguousarray(antennas, dtype=np.uint64)
        tof = np.ascontiguousarray(time_offsets, dtype=np.uint64)
        sol = _c64(solutions)
        check(lib().wgpu_gridder_add_inversion_data_corrected(
            self._h, int(mode), n_polarizations, n_rows, ptr(uvws), ptr(frequencies),
            n_channels, ptr(ant), ptr(vis), ptr(tof), ptr(sol), nparms, n_times, n_antenna,
            int(polarization)))

    def PredictVisibilitiesWithCorrection(self, mode, n_polarizations, n_rows, uvws,
                                          frequencies, n_channels, antennas, time_offsets,
                                          solutions, nparms, n_times, n_antenna,
                                          polarization=_lib.POL_I):
        """PredictVisibilities followed by the prediction write-back of
        msgridderdata.h:180-202, 943-1003 (expansion to the correlations and the
        forward gains of each row's antennas) on the device; returns
        [n_rows * n_channels * n_polarizations] complex64."""
        if isinstance(mode, str):
            mode = GainMode[mode]
        uvws, frequencies = _f64(uvws), _f64(frequencies)
        ant = np.ascontiguousarray(antennas, dtype=np.uint64)
        tof = np.ascontiguousarray(time_offsets, dtype=np.uint64)
        sol = _c64(solutions)
        out = np.empty(n_rows * n_channels * n_polarizations, dtype=np.complex64)
        check(lib().wgpu_gridder_predict_visibilities_corrected(
            self._h, int(mode), n_polarizations, n_rows, ptr(uvws), ptr(frequencies),
            n_channels, ptr(ant), ptr(tof), ptr(sol), nparms, n_times, n_antenna,
            int(polarization), ptr(out)))
        return out

    def AddInversionRows(self, image_weights, uvw, frequencies, weights, vis=None, model=None,
                         selected=None, sums=None, **settings):
        """Raw rows -> weighted, collapsed visibilities -> AddInversionData,
        all on the device (wgpu_gridder_add_inversion_rows); see
        wsclean_gb300.weights.prepare_rows for the arguments.  Returns the
        accumulated weight sums."""
        from . import weights as _weights
        return _weights.add_inversion_rows(self, image_weights, uvw, frequencies, weights, vis,
                                           model, selected, sums, **settings)

    def FinalizeImage(self, multiplication_factor):
        check(lib().wgpu_gridder_finalize_image(self._h, float(multiplication_factor)))

    def RealImage(self, out=None):
        """The image as float32 (width * height); `out` (contiguous float32 of
        that size, e.g. pinned host memory) receives it when given."""
        if out is None:
            out = np.empty(self.width * self.height, dtype=np.float32)
        else:
            assert out.dtype == np.float32 and out.flags.c_contiguous
            assert out.size == self.width * self.height
        check(lib().wgpu_gridder_real_image(self._h, ptr(out)))
        return out

    def FinishInversion(self, image_width, image_height, trim_width, trim_height):
        """After FinalizeImage: RealImage resampled from the gridder's size to
        image_width x image_height (when different) and trimmed to
        trim_width x trim_height, as WGriddingMSGridder::FinishInversion does
        (wgriddingmsgridder.cpp:273-309); returns (trim_height, trim_width)."""
        out = np.empty((trim_height, trim_width), np.float32)
        check(lib().wgpu_gridder_finish_inversion(self._h, image_width, image_height, trim_width,
                                                  trim_height, ptr(out)))
        return out

    def StartPredict(self, model, image_width, image_height):
        """The (trim_height, trim_width) model untrimmed to image_width x
        image_height, resampled to the gridder's size and set as the
        prediction image, as WGriddingMSGridder::StartPredict does
        (wgriddingmsgridder.cpp:311-340)."""
        m = np.ascontiguousarray(model, np.float32)
        th, tw = m.shape
        check(lib().wgpu_gridder_start_predict(self._h, tw, th, image_width, image_height,
                                               ptr(m)))

    def InitializePrediction(self, image_data):
        img = np.ascontiguousarray(image_data, dtype=np.float32).ravel()
        assert img.size == self.width * self.height
        check(lib().wgpu_gridder_initialize_prediction(self._h, ptr(img)))

    def PredictVisibilities(self, n_rows, n_chan, uvw, freq):
        uvw, freq = _f64(uvw), _f64(freq)
        out = np.empty(n_rows * n_chan, dtype=np.complex64)
        check(lib().wgpu_gridder_predict_visibilities(self._h, n_rows, n_chan, ptr(uvw),
                                                      ptr(freq), ptr(out)))
        return out

    def PredictVisibilitiesMasked(self, n_rows, n_chan, uvw, freq, mask, out=None):
        """PredictVisibilities for the samples with mask != 0 (others -> 0)."""
        uvw, freq = _f64(uvw), _f64(freq)
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        assert mask.size == n_rows * n_chan
        if out is None:
            out = np.empty(n_rows * n_chan, dtype=np.complex64)
        check(lib().wgpu_gridder_predict_visibilities_masked(
            self._h, n_rows, n_chan, ptr(uvw), ptr(freq), ptr(mask), ptr(out)))
        return out

    def PredictVisibilitiesMaskedDevice(self, n_rows, n_chan, d_uvw, d_freq, d_mask, d_vis):
        check(lib().wgpu_gridder_predict_visibilities_masked_device(
            self._h, n_rows, n_chan, d_uvw, d_freq, d_mask, d_vis))

    def PredictVisibilitiesDevice(self, n_rows, n_chan, d_uvw, d_freq, d_vis):
        check(lib().wgpu_gridder_predict_visibilities_device(self._h, n_rows, n_chan, d_uvw,
                                                             d_freq, d_vis))

    # device-resident state across major cycles
    def Bind(self, n_rows, n_chan, uvw, freq, mask=None):
        """Plan and bucket this visibility set once; later cycles replay graphs."""
        uvw, freq = _f64(uvw), _f64(freq)
        self._bound_n = n_rows * n_chan
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        check(lib().wgpu_gridder_bind(self._h, n_rows, n_chan, ptr(uvw), ptr(freq), ptr(m)))

    def Unbind(self):
        check(lib().wgpu_gridder_unbind(self._h))

    def InvertBound(self, vis):
        vis = _c64(vis)
        assert vis.size == self._bound_n
        check(lib().wgpu_gridder_invert_bound(self._h, ptr(vis)))

    def InvertBoundDevice(self, d_vis):
        check(lib().wgpu_gridder_invert_bound_device(self._h, d_vis))

    def PredictBound(self, out=None):
        if out is None:
            out = np.empty(self._bound_n, dtype=np.complex64)
        check(lib().wgpu_gridder_predict_bound(self._h, ptr(out)))
        return out

    def PredictBoundDevice(self, d_vis):
        check(lib().wgpu_gridder_predict_bound_device(self._h, d_vis))

    # diagnostics
    def last_plan(self):
        p = _lib.Plan()
        check(lib().wgpu_gridder_last_plan(self._h, C.byref(p)))
        return p

    def last_timings(self):
        """{stage: (milliseconds, launches)} of the last call."""
        ms = (C.c_double * 64)()
        cnt = (C.c_int * 64)()
        names = C.create_string_buffer(4096)
        n = C.c_int()
        check(lib().wgpu_gridder_last_timings(self._h, ms, cnt, 64, names, 4096, C.byref(n)))
        keys = names.value.decode().split(";") if n.value else []
        return {k: (ms[i], cnt[i]) for i, k in enumerate(keys)}

    def last_tuning(self):
        """Candidates timed by the last planning of a tuning gridder (an empty
        list when the plan came from a remembered choice, a pinned plan or a
        gridder without tuning)."""
        trials = (_lib.TuningTrial * 64)()
        n = C.c_int()
        check(lib().wgpu_gridder_last_tuning(self._h, trials, 64, C.byref(n)))
        return [trials[i].as_dict() for i in range(n.value)]

    def pin_plan(self, plan):
        """Use `plan` (a Plan from last_plan()) for following calls; None unpins."""
        check(lib().wgpu_gridder_pin_plan(self._h, None if plan is None else C.byref(plan)))

    def stream(self):
        return lib().wgpu_gridder_stream(self._h)


def bucket_debug(plan, n_rows, n_chan, uvw, freq, vis, skip_zero):
    """Runs the GPU bucketing pass alone and returns its outputs (test hook)."""
    uvw, freq = _f64(uvw), _f64(freq)
    vis = _c64(vis) if vis is not None else None
    n = n_rows * n_chan
    perm = np.zeros(n, np.uint32)
    iu = np.zeros(n, np.int32)
    iv = np.zeros(n, np.int32)
    ip = np.zeros(n, np.int32)
    fu = np.zeros(n, np.float32)
    fv = np.zeros(n, np.float32)
    fw = np.zeros(n, np.float32)
    n_keys = (plan.nu // plan.tile) * (plan.nv // plan.tile) * 4 * plan.n_planes
    off = np.zeros(n_keys + 1, np.uint32)
    n_out = C.c_int64()
    check(lib().wgpu_bucket_debug(C.byref(plan), n_rows, n_chan, ptr(uvw), ptr(freq), ptr(vis),
                                  1 if skip_zero else 0, ptr(perm), ptr(iu), ptr(iv), ptr(ip),
                                  ptr(fu), ptr(fv), ptr(fw), ptr(off), C.byref(n_out)))
    k = n_out.value
    return dict(perm=perm[:k], iu=iu[:k], iv=iv[:k], ip=ip[:k], fu=fu[:k], fv=fv[:k],
                fw=fw[:k], offsets=off)


def bucket_debug_rows(plan, n_rows, n_chan, uvw, freq, vis, skip_zero):
    """Row occupancy of the bucketing pass (wgpu_bucket_debug_rows): flags
    [n_planes, nv] uint8, start [n_planes + 1] and the row list."""
    uvw = _f64(uvw)
    freq = _f64(freq)
    if vis is not None:
        vis = _c64(vis)
    cells = int(plan.n_planes) * int(plan.nv)
    flags = np.zeros(cells, np.uint8)
    start = np.zeros(int(plan.n_planes) + 1, np.uint32)
    rows = np.zeros(cells, np.uint32)
    check(lib().wgpu_bucket_debug_rows(C.byref(plan), n_rows, n_chan, ptr(uvw), ptr(freq),
                                       ptr(vis), 1 if skip_zero else 0, ptr(flags), ptr(start),
                                       ptr(rows)))
    return dict(flags=flags.reshape(int(plan.n_planes), int(plan.nv)), start=start,
                list=rows[:int(start[-1])])
