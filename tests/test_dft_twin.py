"""The FP64 direct Fourier transform on the GPU (oracle/dft_cuda.cu) pinned to
the CPU oracle, and the product's error over EVERY visibility of the plain
1024^2 workload (64 antennas in a 3 km disk, 2016 baselines x 60 x 10 s, 16
channels 120-180 MHz: 1,935,360 samples) measured with it.

Tolerances: the twin and the CPU oracle are both FP64 and differ only in the
order of their sums and in the channel recurrence, so they agree to 1e-10
relative L2; the product must be within the requested epsilon (relative L2) of
the direct transform, as WSClean's -wgridder-accuracy defines it
(doc/source/wgridding.rst:16-20).
"""
import numpy as np
import pytest

from wsclean_gb300 import synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple

pytestmark = pytest.mark.gpu

TWIN_TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


@pytest.mark.parametrize("freqs", ["linear", "descending", "irregular"])
def test_twin_inversion_matches_cpu_dft(oracle_lib, freqs):
    W, dl = 256, 3e-4
    uvw, freq, vis = synthetic.random_points(3000, 24, W, dl, seed=11, w_scale=2.0, frac_zero=0.1)
    vis[5] = 0        # an empty row
    vis[7, 20:] = 0   # trailing zero channels
    if freqs == "descending":
        freq = freq[::-1].copy()
    elif freqs == "irregular":
        rng = np.random.default_rng(3)
        freq = np.sort(rng.uniform(1e8, 2e8, freq.size))
    rng = np.random.default_rng(12)
    pix = rng.choice(W * W, 64, replace=False)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, 0.01, -0.005, pixels=pix)
    got = oracle_lib.cuda_dft_invert(uvw, freq, vis, W, W, dl, dl, 0.01, -0.005, pixels=pix)
    assert rel(got, ref) < TWIN_TOL


@pytest.mark.parametrize("freqs", ["linear", "irregular"])
def test_twin_prediction_matches_cpu_dft(oracle_lib, freqs):
    W, dl = 128, 5e-4
    uvw, freq, _ = synthetic.random_points(500, 37, W, dl, seed=21, w_scale=1.5)
    if freqs == "irregular":
        rng = np.random.default_rng(4)
        freq = np.sort(rng.uniform(1e8, 2e8, freq.size))
    image = np.zeros(W * W)
    rng = np.random.default_rng(22)
    image[rng.choice(W * W, 150, replace=False)] = rng.uniform(-1, 1, 150)
    ref = oracle_lib.dft_predict(uvw, freq, image, W, W, dl, dl, 0.002, 0.001)
    vals, e2, r2 = oracle_lib.cuda_dft_predict(uvw, freq, image, W, W, dl, dl, 0.002, 0.001,
                                               want_values=True)
    assert rel(vals, ref) < TWIN_TOL
    assert abs(r2 - float(np.sum(np.abs(ref) ** 2))) <= 1e-9 * r2
    # error sums over a mask against a perturbed prediction
    pred = (ref + 1e-3 * (rng.standard_normal(ref.size) + 1j * rng.standard_normal(ref.size)))
    pred = pred.astype(np.complex64)
    mask = (rng.uniform(size=ref.size) < 0.7).astype(np.uint8)
    _, e2m, r2m = oracle_lib.cuda_dft_predict(uvw, freq, image, W, W, dl, dl, 0.002, 0.001,
                                              mask=mask, pred=pred)
    sel = mask != 0
    ee = float(np.sum(np.abs(pred[sel].astype(np.complex128) - ref[sel]) ** 2))
    rr = float(np.sum(np.abs(ref[sel]) ** 2))
    assert abs(e2m - ee) <= 1e-6 * ee
    assert abs(r2m - rr) <= 1e-9 * rr


@pytest.fixture(scope="module")
def plain1024():
    return synthetic.make_workload("plain1024", seed=1)


def _model_image(d):
    W, dl = d["width"], d["dl"]
    model = np.zeros(W * W, np.float32)
    for l, m, s in d["sources"]:
        x, y = int(round(W / 2 - l / dl)), int(round(m / dl + W / 2))
        if 0 <= x < W and 0 <= y < W:
            model[y * W + x] += s
    return model


@pytest.mark.parametrize("eps", [1e-4, 1e-5])
def test_plain1024_full_data_within_epsilon(wgpu_lib, oracle_lib, plain1024, eps):
    """Every one of the 1,935,360 samples gridded and predicted at full size."""
    d = plain1024
    uvw, freq, vis = d["uvw"], d["freq"], d["vis"]
    W, dl = d["width"], d["dl"]
    assert uvw.shape[0] * freq.size == 1935360
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    img = g.RealImage().astype(np.float64)
    rng = np.random.default_rng(5)
    pix = rng.choice(W * W, 65536, replace=False)
    ref = oracle_lib.cuda_dft_invert(uvw, freq, vis, W, W, dl, dl, pixels=pix)
    # the twin against the CPU oracle on these data (128 pixels)
    cpu = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, pixels=pix[:128])
    assert rel(ref[:128], cpu) < TWIN_TOL
    inv_err = rel(img[pix], ref)
    assert inv_err <= eps, inv_err
    model = _model_image(d)
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    _, e2, r2 = oracle_lib.cuda_dft_predict(uvw, freq, model, W, W, dl, dl, pred=pv)
    pred_err = float(np.sqrt(e2 / r2))
    assert pred_err <= eps, pred_err
    g.close()
