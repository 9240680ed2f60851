"""Resampling, trimming and small-inversion sizing restated in numpy (TEST
INFRASTRUCTURE ONLY: the checker of wsclean_gb300's resample.cu).

The FFT resampler follows the published method of schaapcommon's Resampler
(absent from the reference tree, so parity with it is unpinned): r2c of the
real input, the rows [0, b_h // 2) and the last b_h // 2 rows of the first
b_w // 2 + 1 columns copied into a zero half spectrum of the output size (b =
the smaller size), c2r, factor 1 / (in_w * in_h); non-finite input pixels
count as zero.  numpy's irfft2 has c2r semantics (the imaginary parts of the
self-conjugate columns are ignored) and divides by the output size, which is
undone here.  Trim / untrim follow Image::Trim / Untrim: the centred window
starts at ((w - tw) // 2, (h - th) // 2).  The sizing functions restate
math/calculatefftsize.h:8-35, gridding/msgridder.cpp:42-75 and
wgridder/wgriddingmsgridder.cpp:243-260.
"""
import math

import numpy as np


def resample(img, out_w, out_h):
    a = np.asarray(img, np.float64)
    a = np.where(np.isfinite(a), a, 0.0)
    in_h, in_w = a.shape
    f = np.fft.rfft2(a)
    bw, bh = min(in_w, out_w), min(in_h, out_h)
    g = np.zeros((out_h, out_w // 2 + 1), np.complex128)
    g[:bh // 2, :bw // 2 + 1] = f[:bh // 2, :bw // 2 + 1]
    if bh // 2:
        g[out_h - bh // 2:, :bw // 2 + 1] = f[in_h - bh // 2:, :bw // 2 + 1]
    out = np.fft.irfft2(g, s=(out_h, out_w)) * (out_h * out_w)
    return out / (in_w * in_h)


def trim(img, tw, th):
    h, w = img.shape
    x0, y0 = (w - tw) // 2, (h - th) // 2
    return img[y0:y0 + th, x0:x0 + tw].copy()


def untrim(img, w, h):
    th, tw = img.shape
    out = np.zeros((h, w), img.dtype)
    x0, y0 = (w - tw) // 2, (h - th) // 2
    out[y0:y0 + th, x0:x0 + tw] = img
    return out


def _low_prime_factors(n):
    while n > 7:
        for p in (2, 3, 5, 7):
            if n % p == 0:
                n //= p
                break
        else:
            return False
    return True


def calculate_fft_size(size, pixel_scale, beam_size):
    total = float(size) * pixel_scale
    minimal = int(math.ceil(total * 2 / beam_size))
    opt = minimal
    if opt % 4:
        opt += 4 - opt % 4
    while not _low_prime_factors(opt) and opt < size:
        opt += 4
    return minimal, min(opt, size)


def small_inversion_size(width, height, psx, psy, beam):
    _, ow = calculate_fft_size(width, psx, beam)
    _, oh = calculate_fft_size(height, psy, beam)
    if ow < width or oh < height:
        nw, nh = max(min(ow, width), 32), max(min(oh, height), 32)
        return nw, nh, (float(width) * psx) / float(nw), (float(height) * psy) / float(nh)
    return width, height, psx, psy


def actual_trimmed_size(inv_w, inv_h, padding):
    tw, th = int(math.ceil(inv_w / padding)), int(math.ceil(inv_h / padding))
    tw += (4 - tw % 4) % 4
    th += (4 - th % 4) % 4
    return min(tw, inv_w), min(th, inv_h)
