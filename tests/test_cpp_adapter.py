"""The C++ drop-in class (include/wgpu_gridder.h) compiled with g++ against
the library and driven like WSClean drives WGriddingGridder_Simple."""
import os
import subprocess

import numpy as np
import pytest

from wsclean_gb300 import synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_test.cpp")


def _build(tmp_path, wgpu_lib):
    exe = str(tmp_path / "adapter_test")
    lib_dir = os.path.join(ROOT, "wsclean_gb300", "_build")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", lib_dir, "-lwgpu", f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_adapter_compiles(tmp_path, wgpu_lib):
    assert os.path.exists(_build(tmp_path, wgpu_lib))


@pytest.mark.gpu
def test_adapter_matches_oracle(tmp_path, wgpu_lib, oracle_lib):
    exe = _build(tmp_path, wgpu_lib)
    W, Wt, dl, eps = 160, 128, 4e-4, 1e-5
    uvw, freq, vis = synthetic.random_points(600, 4, Wt, dl, seed=41, w_scale=2.0,
                                             frac_zero=0.05)
    model = np.zeros((W, W), np.float32)
    model[70, 60] = 1.0
    model[90, 100] = -0.5
    files = {}
    for name, arr in dict(uvw=uvw, freq=freq, vis=vis.astype(np.complex64), model=model).items():
        files[name] = str(tmp_path / f"{name}.bin")
        np.ascontiguousarray(arr).tofile(files[name])
    prefix = str(tmp_path / "out_")
    r = subprocess.run([exe, str(W), str(Wt), str(uvw.shape[0]), str(freq.size), repr(dl),
                        repr(eps), files["uvw"], files["freq"], files["vis"], files["model"],
                        prefix], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    img = np.fromfile(prefix + "image.bin", np.float32).reshape(W, W)
    d = (W - Wt) // 2
    ref = oracle_lib.dft_invert(uvw, freq, vis, Wt, Wt, dl, dl).reshape(Wt, Wt)
    got = img[d:d + Wt, d:d + Wt].astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= eps
    pred = np.fromfile(prefix + "pred.bin", np.complex64)
    trimmed = model[d:d + Wt, d:d + Wt].ravel()
    pr = oracle_lib.dft_predict(uvw, freq, trimmed, Wt, Wt, dl, dl)
    assert np.linalg.norm(pred - pr) / np.linalg.norm(pr) <= eps
    # FinishInversion: RealImage resampled to (W + 32)^2 and trimmed to Wt^2
    from oracle import resample as ores
    fin = np.fromfile(prefix + "finish.bin", np.float32).reshape(Wt, Wt)
    exp = ores.trim(ores.resample(img, W + 32, W + 32), Wt, Wt)
    assert np.linalg.norm(fin - exp) <= 1e-5 * np.linalg.norm(exp)
    # raw rows through GpuImageWeights + AddInversionRows = the Python API path
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    from wsclean_gb300.weights import UNIFORM, ImageWeights
    ones = np.ones((uvw.shape[0], freq.size, 1), np.float32)
    iw = ImageWeights(UNIFORM, Wt, Wt, dl, dl)
    iw.Grid(uvw, freq, ones)
    iw.FinishGridding()
    g = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps, num_t=np.float64)
    g.InitializeInversion()
    sums = g.AddInversionRows(iw, uvw, freq, ones, vis.astype(np.complex64)[:, :, None])
    g.FinalizeImage(1.0)
    py_rows = g.RealImage().reshape(W, W)[d:d + Wt, d:d + Wt]
    rows = np.fromfile(prefix + "rows.bin", np.float32).reshape(W, W)[d:d + Wt, d:d + Wt]
    # the same rows on the same plan through two front ends: the gridding kernel
    # adds footprints into its shared-memory tile with float atomics, so the two
    # runs differ only in the order of float additions (FP32 rounding, which the
    # grid correction magnifies at the image border)
    assert np.linalg.norm(rows - py_rows) <= 1e-6 * np.linalg.norm(py_rows)
    s4 = np.fromfile(prefix + "sums.bin", np.float64)
    assert s4[3] == sums.gridded_visibility_count > 0
    # uniform diagonal gain 1.5+0.5i, XX mode: |g|^2 = 2.5 times the prediction
    pred_corr = np.fromfile(prefix + "pred_corr.bin", np.complex64)
    np.testing.assert_allclose(pred_corr, 2.5 * pred, rtol=1e-5, atol=1e-6 * np.abs(pred).max())
