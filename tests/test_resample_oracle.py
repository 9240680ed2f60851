"""Sizing around the gridder boundary and the resampling oracle (CPU).

CalculateFFTSize is pinned to the reference's own header (math/calculatefftsize.h,
compiled into oracle/_ref where the reference tree is present); the library's
host functions and the oracle's restatements must agree with it.  The numpy
resampler's conventions (normalisation, half-spectrum copy) are checked on
band-limited images, where FFT resampling is exact."""
import numpy as np
import pytest

from oracle import resample as ores
from wsclean_gb300 import resample as wres

ARCSEC = np.pi / 180 / 3600
FFT_CASES = [(8192, 3 * ARCSEC, 1 / 60000.0), (8192, 3 * ARCSEC, 1 / 2000.0), (1024, 10 * ARCSEC,
             1 / 3000.0), (5000, 1.5 * ARCSEC, 1 / 100000.0), (37, 0.01, 0.05), (4096, 1e-5, 1.0),
             (100, 1e-3, 0.0123), (7, 0.3, 0.2), (65536, 2e-6, 1 / 5000.0)]


def _random_fft_cases(n=300):
    rng = np.random.default_rng(1)
    sizes = rng.integers(8, 20000, n)
    scales = 10 ** rng.uniform(-6.5, -3.5, n)
    beams = 10 ** rng.uniform(-6, -2, n)
    return list(zip(sizes.tolist(), scales.tolist(), beams.tolist()))


def test_calculate_fft_size_matches_reference_header(oracle_lib):
    ref = oracle_lib.ref_calculate_fft_size()
    for size, scale, beam in FFT_CASES + _random_fft_cases():
        got = wres.calculate_fft_size(size, scale, beam)
        assert got == ores.calculate_fft_size(size, scale, beam), (size, scale, beam)
        if ref is not None:
            assert got == ref(size, scale, beam), (size, scale, beam)
    if ref is None:
        pytest.skip("reference tree absent: pinned against the restatement only")


def test_small_inversion_and_trimmed_sizes_match_restatement():
    for size, scale, beam in FFT_CASES + _random_fft_cases(100):
        got = wres.small_inversion_size(size, size + 6, scale, scale * 1.1, beam)
        exp = ores.small_inversion_size(size, size + 6, scale, scale * 1.1, beam)
        assert got[:2] == exp[:2] and got[2] == exp[2] and got[3] == exp[3]
        assert got[0] >= min(32, size) and got[0] <= size
    for w, h, pad in [(5000, 4000, 1.2), (1024, 1024, 1.0), (333, 97, 1.5), (30, 31, 2.0),
                      (8192, 6144, 1.3)]:
        assert wres.actual_trimmed_size(w, h, pad) == ores.actual_trimmed_size(w, h, pad)


def test_small_inversion_reduces_oversampled_images():
    w, h, px, py = wres.small_inversion_size(8192, 8192, 3 * ARCSEC, 3 * ARCSEC, 1 / 2000.0)
    assert w < 8192 and w % 4 == 0 and px > 3 * ARCSEC
    assert abs(w * px - 8192 * 3 * ARCSEC) < 1e-12


def _bandlimited(w, h, fx, fy, phase=0.3):
    y, x = np.mgrid[0:h, 0:w]
    return np.cos(2 * np.pi * (fx * x / w + fy * y / h) + phase)


@pytest.mark.parametrize("in_shape,out_shape", [((48, 64), (60, 80)), ((90, 100), (50, 64)),
                                                ((45, 63), (33, 77)), ((32, 32), (32, 32))])
def test_oracle_resample_is_exact_on_bandlimited_images(in_shape, out_shape):
    (ih, iw), (oh, ow) = in_shape, out_shape
    fx, fy = 3, -2  # well inside both spectra
    got = ores.resample(_bandlimited(iw, ih, fx, fy), ow, oh)
    np.testing.assert_allclose(got, _bandlimited(ow, oh, fx, fy), atol=1e-12)


def test_oracle_trim_untrim_and_nan_border():
    img = np.arange(7 * 9, dtype=np.float64).reshape(7, 9)
    t = ores.trim(img, 5, 3)
    np.testing.assert_array_equal(t, img[2:5, 2:7])
    np.testing.assert_array_equal(ores.untrim(t, 9, 7)[2:5, 2:7], t)
    assert ores.untrim(t, 9, 7).sum() == t.sum()
    a = _bandlimited(40, 30, 2, 1)
    b = a.copy()
    b[:3] = np.nan
    a[:3] = 0.0
    np.testing.assert_allclose(ores.resample(b, 50, 36), ores.resample(a, 50, 36), atol=0)
