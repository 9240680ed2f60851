"""Resampling around the gridder boundary on the GPU against the numpy oracle:
the FFT resampler (FP32 mixed-radix transforms; relative L2 error <= 1e-5
against the FP64 oracle), the trim / untrim and the FinishInversion /
StartPredict helpers of the gridder."""
import numpy as np
import pytest

from oracle import resample as ores
from wsclean_gb300 import _lib, synthetic
from wsclean_gb300 import resample as wres
from wsclean_gb300.gridder import WGriddingGridder_Simple

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    a = np.asarray(a)
    a = a.astype(np.complex128) if np.iscomplexobj(a) else a.astype(np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


SHAPES = [((48, 64), (60, 80)), ((90, 100), (50, 64)), ((45, 63), (33, 77)),
          ((96, 96), (96, 96)), ((91, 121), (143, 77)), ((2, 32), (4, 48)), ((120, 2), (80, 6)),
          ((256, 256), (200, 200)), ((343, 125), (343, 125 * 2))]


@pytest.mark.parametrize("in_shape,out_shape", SHAPES)
def test_resample_matches_oracle(in_shape, out_shape):
    rng = np.random.default_rng(sum(in_shape) + 3 * sum(out_shape))
    img = rng.standard_normal(in_shape).astype(np.float32)
    img[0, :] = np.nan  # a RealImage-like border counts as zero
    got = wres.resample(img, out_shape[1], out_shape[0])
    exp = ores.resample(img, out_shape[1], out_shape[0])
    assert got.shape == out_shape and np.all(np.isfinite(got))
    assert rel(got, exp) <= TOL


def test_resample_large_image():
    rng = np.random.default_rng(5)
    img = rng.standard_normal((2048, 2048)).astype(np.float32)
    got = wres.resample(img, 1536, 1680)
    assert rel(got, ores.resample(img, 1536, 1680)) <= TOL


def test_resample_rejects_large_prime_factors():
    with pytest.raises(_lib.WgpuError):
        wres.resample(np.zeros((67, 10), np.float32), 20, 20)


def _gridder_pair(n_inv, n_t, dl):
    g = WGriddingGridder_Simple(n_inv, n_inv, n_t, n_t, dl, dl, 0.0, 0.0, 1, epsilon=1e-5,
                                num_t=np.float64)
    return g


def test_finish_inversion_matches_oracle_pipeline():
    """RealImage at the inversion size (NaN border), resampled to the image size
    and trimmed, as FinishInversion does."""
    n_inv, n_t, dl = 200, 168, 5e-4
    image_w, trim_w = 240, 200
    uvw, freq, vis = synthetic.random_points(700, 4, n_t, dl, seed=9, w_scale=1.5)
    g = _gridder_pair(n_inv, n_t, dl)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    g.FinalizeImage(0.5)
    real = g.RealImage().reshape(n_inv, n_inv)
    got = g.FinishInversion(image_w, image_w, trim_w, trim_w)
    exp = ores.trim(ores.resample(real, image_w, image_w), trim_w, trim_w)
    assert got.shape == (trim_w, trim_w)
    assert rel(got, exp) <= TOL
    # without resampling the trim applies to RealImage itself (NaN border kept)
    same = g.FinishInversion(n_inv, n_inv, 180, 180)
    np.testing.assert_array_equal(same, ores.trim(real, 180, 180).astype(np.float32))


def test_start_predict_matches_oracle_pipeline():
    n_inv, n_t, dl = 200, 168, 5e-4
    image_w, trim_w = 240, 200
    uvw, freq, _ = synthetic.random_points(500, 3, n_t, dl, seed=10, w_scale=1.5)
    rng = np.random.default_rng(11)
    model = np.zeros((trim_w, trim_w), np.float32)
    model[rng.integers(40, 160, 12), rng.integers(40, 160, 12)] = rng.uniform(0.5, 2, 12)
    g1 = _gridder_pair(n_inv, n_t, dl)
    g1.StartPredict(model, image_w, image_w)
    got = g1.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    full = ores.resample(ores.untrim(model, image_w, image_w), n_inv, n_inv).astype(np.float32)
    g2 = _gridder_pair(n_inv, n_t, dl)
    g2.InitializePrediction(full)
    exp = g2.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    assert rel(got, exp) <= 1e-5
