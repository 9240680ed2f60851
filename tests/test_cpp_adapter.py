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
    # the same rows on the same plan through two front ends: a uv tile whose
    # samples are split over several work items adds each item's cells to the
    # plane with float atomics, so the two runs can differ in the order of those
    # float additions (FP32 rounding, which the grid correction magnifies at the
    # image border)
    assert np.linalg.norm(rows - py_rows) <= 1e-6 * np.linalg.norm(py_rows)
    s4 = np.fromfile(prefix + "sums.bin", np.float64)
    assert s4[3] == sums.gridded_visibility_count > 0
    # uniform diagonal gain 1.5+0.5i, XX mode: |g|^2 = 2.5 times the prediction
    pred_corr = np.fromfile(prefix + "pred_corr.bin", np.complex64)
    np.testing.assert_allclose(pred_corr, 2.5 * pred, rtol=1e-5, atol=1e-6 * np.abs(pred).max())


CALLBACK_SRC = os.path.join(ROOT, "tests", "cpp", "wsclean_callback_test.cpp")
WSCLEAN_IFACE = os.path.join(ROOT, "tests", "cpp", "wsclean_iface")


def _build_callback(tmp_path):
    exe = str(tmp_path / "wsclean_callback_test")
    lib_dir = os.path.join(ROOT, "wsclean_gb300", "_build")
    cmd = ["g++", "-std=c++17", "-O1", "-DWGPU_WITH_WSCLEAN", "-I", os.path.join(ROOT, "include"),
           "-I", WSCLEAN_IFACE, CALLBACK_SRC, "-o", exe, "-L", lib_dir, "-lwgpu",
           f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_wsclean_callback_path_compiles(tmp_path, wgpu_lib):
    """The correction callback as WSClean builds it (WGPU_WITH_WSCLEAN): it names
    only existing MsGridder / VisibilityModifier members and the two accessors
    the drop-in adds."""
    assert os.path.exists(_build_callback(tmp_path))


@pytest.mark.gpu
def test_wsclean_callback_reads_cached_solutions(tmp_path, wgpu_lib, oracle_lib):
    """The callback reads the gridder's cached full-Jones solutions: the image
    equals the explicit-table path's; outside a facet it applies no gains (the
    rows are only collapsed, as the oracle collapses them); the direction-
    dependent PSF and facet beams are rejected."""
    exe = _build_callback(tmp_path)
    W, dl, n_chan, n_ant, n_t = 128, 4e-4, 4, 6, 3
    uvw, freq, _ = synthetic.random_points(600, n_chan, W, dl, seed=51, w_scale=1.0)
    rng = np.random.default_rng(52)
    n_rows = uvw.shape[0]
    vis4 = (rng.standard_normal((n_rows, n_chan, 4)) +
            1j * rng.standard_normal((n_rows, n_chan, 4))).astype(np.complex64)
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)],
                   1).astype(np.uint64)
    tof = rng.integers(0, n_t, n_rows).astype(np.uint64)
    eye = np.array([1, 0, 0, 1], np.complex64)
    sol = (eye + 0.2 * (rng.standard_normal((n_t, n_chan, n_ant, 4)) +
                        1j * rng.standard_normal((n_t, n_chan, n_ant, 4)))).astype(np.complex64)
    files = []
    for name, arr in (("uvw", uvw), ("freq", freq), ("vis", vis4), ("ant", ant), ("tof", tof),
                      ("sol", sol)):
        path = str(tmp_path / f"{name}.bin")
        np.ascontiguousarray(arr).tofile(path)
        files.append(path)
    prefix = str(tmp_path / "out_")
    r = subprocess.run([exe, str(W), str(n_rows), str(n_chan), str(n_ant), str(n_t), repr(dl)] +
                       files, capture_output=True, text=True, env=dict(os.environ, OUT=prefix))
    assert r.returncode == 0, r.stderr
    img = lambda n: np.fromfile(prefix + n + ".bin", np.float32).astype(np.float64)
    cb, ex, unc = img("callback"), img("explicit"), img("uncorrected")
    ok = np.isfinite(ex)
    assert np.linalg.norm(cb[ok] - ex[ok]) <= 1e-6 * np.linalg.norm(ex[ok])
    # outside a facet: identity gains, Stokes I collapse, plain gridding
    unit = np.broadcast_to(eye, sol.shape).copy()
    collapsed = oracle_lib.apply_gains(4, 4, vis4, ant, tof, unit, 4, n_ant)
    ref = oracle_lib.dft_invert(uvw, freq, collapsed, W, W, dl, dl)
    assert np.linalg.norm(unc - ref) <= 1e-4 * np.linalg.norm(ref)
    assert list(np.fromfile(prefix + "threw.bin", np.int32)) == [1, 1]
