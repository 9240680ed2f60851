"""Resampling and trimming around the gridder boundary.

Mirrors what WGriddingMSGridder::FinishInversion / StartPredict do around the
gridder (wgridder/wgriddingmsgridder.cpp:273-340) and the small-inversion
sizing (gridding/msgridder.cpp:42-75, math/calculatefftsize.h).  The sizing
functions run on the host; the FFT resampling, trimming and the gridder
helpers run on the GPU through the C ABI (include/wgpu.h).
"""
import ctypes as C

import numpy as np

from ._lib import check, lib, ptr


def calculate_fft_size(size, pixel_scale, beam_size):
    """CalculateFFTSize: (minimal, optimal) sizes."""
    mn, opt = C.c_size_t(), C.c_size_t()
    check(lib().wgpu_calculate_fft_size(int(size), float(pixel_scale), float(beam_size),
                                        C.byref(mn), C.byref(opt)))
    return mn.value, opt.value


def small_inversion_size(width, height, pixel_size_x, pixel_size_y, beam_size):
    """(inversion width, height, pixel size x, y) of the small inversion."""
    w, h, px, py = C.c_size_t(), C.c_size_t(), C.c_double(), C.c_double()
    check(lib().wgpu_small_inversion_size(int(width), int(height), float(pixel_size_x),
                                          float(pixel_size_y), float(beam_size), C.byref(w),
                                          C.byref(h), C.byref(px), C.byref(py)))
    return w.value, h.value, px.value, py.value


def actual_trimmed_size(inversion_width, inversion_height, image_padding):
    """getActualTrimmedSize: the gridder's trimmed (width, height)."""
    w, h = C.c_size_t(), C.c_size_t()
    check(lib().wgpu_actual_trimmed_size(int(inversion_width), int(inversion_height),
                                         float(image_padding), C.byref(w), C.byref(h)))
    return w.value, h.value


def resample(image, out_width, out_height):
    """FFT resampling of a (height, width) float image on the GPU; returns an
    (out_height, out_width) float32 image."""
    img = np.ascontiguousarray(image, np.float32)
    in_h, in_w = img.shape
    out = np.empty((out_height, out_width), np.float32)
    check(lib().wgpu_resample(ptr(img), in_w, in_h, ptr(out), out_width, out_height))
    return out


def resample_device(d_in, in_width, in_height, d_out, out_width, out_height, stream=None):
    """The same on device buffers (integer addresses), on `stream`."""
    check(lib().wgpu_resample_device(d_in, in_width, in_height, d_out, out_width, out_height,
                                     stream))
