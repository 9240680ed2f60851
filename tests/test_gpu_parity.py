"""GPU parity: the CUDA path through the C ABI against the oracle.

Tolerances: bucketing is bit-exact; images and predicted visibilities must be
within the requested epsilon (relative L2) of the FP64 direct FT and of the FP64
CPU w-gridder run on the same plan (the difference to the latter is the FP32
round-off that the planner budgets inside epsilon).
"""
import json
import os

import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple, bucket_debug, bucket_debug_rows

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
C = 299792458.0


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def _plan_for(uvw, freq, vis, W, dl, eps, shift=(0.0, 0.0), **kw):
    wl = uvw[:, 2:3] * (freq / C)[None, :]
    if vis is not None:
        wl = wl[vis != 0]
    return _lib.make_plan(width=W, height=W, dl=dl, dm=dl, l_shift=shift[0], m_shift=shift[1],
                          epsilon=eps, w_min=float(wl.min()), w_max=float(wl.max()),
                          n_vis=int(wl.size), **kw)


BUCKET_CASES = [
    dict(W=96, dl=1e-3, rows=700, chan=5, w_scale=1.0, zero=0.2, seed=1, shift=(0, 0), inv=True),
    dict(W=256, dl=3e-4, rows=3000, chan=8, w_scale=3.0, zero=0.0, seed=2, shift=(0.01, -0.02),
         inv=False),
    dict(W=128, dl=5e-4, rows=1500, chan=3, w_scale=0.0, zero=0.1, seed=3, shift=(0, 0), inv=True),
    dict(W=512, dl=1e-4, rows=5000, chan=16, w_scale=2.0, zero=0.3, seed=4, shift=(0, 0.003),
         inv=True),
    # 2.56 M samples: several hundred 4096-element sort tiles, more than the
    # sort's resident blocks, so blocks take several tiles each
    dict(W=1024, dl=5e-5, rows=40000, chan=64, w_scale=2.0, zero=0.25, seed=5, shift=(0, 0),
         inv=True),
]


@pytest.mark.parametrize("case", BUCKET_CASES)
def test_bucketing_bit_exact(wgpu_lib, oracle_lib, case):
    uvw, freq, vis = synthetic.random_points(case["rows"], case["chan"], case["W"], case["dl"],
                                             case["seed"], w_scale=case["w_scale"],
                                             frac_zero=case["zero"])
    if case["seed"] == 2:
        freq = freq[::-1].copy()  # descending frequencies
    p = _plan_for(uvw, freq, vis if case["inv"] else None, case["W"], case["dl"], 1e-4,
                  case["shift"])
    got = bucket_debug(p, uvw.shape[0], freq.size, uvw, freq, vis if case["inv"] else None,
                       case["inv"])
    ref = oracle_lib.bucket(p, uvw, freq, vis if case["inv"] else None, case["inv"])
    for k in ("perm", "iu", "iv", "ip", "fu", "fv", "fw"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["offsets"].astype(np.int64), ref["offsets"])


def test_bucketing_matches_golden_fixture(wgpu_lib):
    g = np.load(os.path.join(GOLDEN, "bucket_small.npz"))
    plan = json.loads(str(g["plan"]))
    p = _lib.Plan()
    for k, v in plan.items():
        setattr(p, k, v)
    got = bucket_debug(p, g["uvw"].shape[0], g["freq"].size, g["uvw"], g["freq"], g["vis"], True)
    for k in ("perm", "iu", "iv", "ip", "fu", "fv", "fw"):
        np.testing.assert_array_equal(got[k], g[k], err_msg=k)
    np.testing.assert_array_equal(got["offsets"].astype(np.int64), g["offsets"])


def _footprint_rows(iv, ip, n_planes, nv, W):
    """(plane, row) pairs the footprints with corners (ip, iv) cover: planes
    ip .. ip + W - 1 (one plane without w stacking), rows iv .. iv + W - 1
    cyclically."""
    corner = np.zeros((n_planes, nv), bool)
    corner[ip, iv] = True
    occ = np.zeros_like(corner)
    for a in range(W if n_planes > 1 else 1):
        for b in range(W):
            occ[a:] |= np.roll(corner, b, axis=1)[:n_planes - a]
    return occ


@pytest.mark.parametrize("case", BUCKET_CASES)
def test_row_occupancy_matches_oracle_footprints(wgpu_lib, oracle_lib, case):
    """The rows the row transforms process are exactly the (plane, row) pairs
    that the oracle's footprints cover, listed in plane-then-row order."""
    uvw, freq, vis = synthetic.random_points(case["rows"], case["chan"], case["W"], case["dl"],
                                             case["seed"], w_scale=case["w_scale"],
                                             frac_zero=case["zero"])
    v = vis if case["inv"] else None
    p = _plan_for(uvw, freq, v, case["W"], case["dl"], 1e-4, case["shift"])
    ref = oracle_lib.bucket(p, uvw, freq, v, case["inv"])
    got = bucket_debug_rows(p, uvw.shape[0], freq.size, uvw, freq, v, case["inv"])
    occ = _footprint_rows(np.asarray(ref["iv"]), np.asarray(ref["ip"]), p.n_planes, p.nv,
                          p.support)
    np.testing.assert_array_equal(got["flags"].astype(bool), occ)
    np.testing.assert_array_equal(got["list"], np.flatnonzero(occ.ravel()).astype(np.uint32))
    np.testing.assert_array_equal(got["start"].astype(np.int64),
                                  np.concatenate([[0], np.cumsum(occ.sum(axis=1))]))


def test_bucketing_bit_exact_near_cell_edges(wgpu_lib, oracle_lib):
    """Footprint corners within 1e-9 cells (or planes) of an integer: the FP32
    test cannot decide these samples and leaves them to the FP64 pass, whose
    corners and fractions must still equal the oracle's."""
    rng = np.random.default_rng(7)
    W, dl, n = 256, 3e-4, 4000
    uvw, freq, _ = synthetic.random_points(n, 1, W, dl, 7, w_scale=2.0)
    p = _plan_for(uvw, freq, None, W, dl, 1e-4)
    fl = freq[0] / C
    su, sv = fl * dl * p.nu, fl * dl * p.nv
    half = 0.5 * p.support
    wl = uvw[:, 2] * fl
    inner = np.ones(n, bool)
    inner[[int(np.argmin(wl)), int(np.argmax(wl))]] = False  # keep the w range
    d = rng.choice([-1e-9, 0.0, 1e-9], size=(n, 3))
    u = (np.round(uvw[:, 0] * su - half) + half + d[:, 0]) / su
    v = (np.round(uvw[:, 1] * sv - half) + half + d[:, 1]) / sv
    uvw[inner, 0] = u[inner]
    uvw[inner, 1] = v[inner]
    assert p.n_planes > 1
    q = np.round((wl - p.w0) / p.dw - half)
    w = ((q + half + d[:, 2]) * p.dw + p.w0) / fl
    uvw[inner, 2] = w[inner]
    got = bucket_debug(p, n, 1, uvw, freq, None, False)
    ref = oracle_lib.bucket(p, uvw, freq, None, False)
    for k in ("perm", "iu", "iv", "ip", "fu", "fv", "fw"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["offsets"].astype(np.int64), ref["offsets"])


INV_CASES = [
    dict(W=128, dl=4e-4, eps=1e-4, shift=(0.0, 0.0), num_t=np.float32, w_scale=3.0),
    dict(W=128, dl=4e-4, eps=1e-5, shift=(0.01, -0.005), num_t=np.float64, w_scale=3.0),
    dict(W=256, dl=2e-4, eps=1e-5, shift=(0.0, 0.0), num_t=np.float64, w_scale=1.0),
    dict(W=192, dl=3e-4, eps=1e-3, shift=(-0.004, 0.002), num_t=np.float32, w_scale=0.0),
]


@pytest.mark.parametrize("case", INV_CASES)
def test_inversion_matches_dft_and_cpu_gridder(wgpu_lib, oracle_lib, case):
    W, dl, eps = case["W"], case["dl"], case["eps"]
    uvw, freq, vis = synthetic.random_points(600, 4, W, dl, seed=5, w_scale=case["w_scale"],
                                             frac_zero=0.1)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, case["shift"][0], case["shift"][1], 1,
                                epsilon=eps, num_t=case["num_t"])
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    g.FinalizeImage(1.0)
    img = g.RealImage().astype(np.float64)
    plan = g.last_plan()
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, *case["shift"])
    assert rel(img, ref) <= eps
    cpu = oracle_lib.wgrid_invert(plan, uvw, freq, vis)
    assert rel(img, cpu) <= eps
    g.close()


def test_inversion_in_chunks_with_trim_and_descending_freq(wgpu_lib, oracle_lib):
    W, Wt, dl = 160, 128, 4e-4
    uvw, freq, vis = synthetic.random_points(900, 6, Wt, dl, seed=8, w_scale=2.0, frac_zero=0.05)
    freq = freq[::-1].copy()
    g = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=1e-4)
    g.InitializeInversion()
    for r0 in range(0, 900, 300):
        g.AddInversionData(300, freq.size, uvw[r0:r0 + 300], freq, vis[r0:r0 + 300])
    g.FinalizeImage(0.5)
    full = g.RealImage().reshape(W, W)
    d = (W - Wt) // 2
    assert np.all(np.isnan(full[:d, :])) and np.all(np.isnan(full[:, :d]))
    assert np.all(np.isnan(full[W - d:, :])) and np.all(np.isnan(full[:, W - d:]))
    img = full[d:d + Wt, d:d + Wt].astype(np.float64).ravel()
    ref = 0.5 * oracle_lib.dft_invert(uvw, freq, vis, Wt, Wt, dl, dl)
    assert rel(img, ref) <= 1e-4
    g.close()


# Grid sizes whose column split n1 x n2 uses the two-stage panel transforms
# (lengths 16 R2, R2 in 2, 3, 4, 5, 6, 8), with sigma pinned to 1.5.
PANEL_CASES = [
    dict(W=1024, dl=6e-5, split=(32, 48)),
    dict(W=2048, dl=3e-5, split=(48, 64)),
    dict(W=5120, dl=1.2e-5, split=(80, 96)),
    dict(W=8192, dl=8e-6, split=(96, 128)),
]


@pytest.mark.parametrize("case", PANEL_CASES)
def test_two_stage_column_transforms_match_dft(wgpu_lib, oracle_lib, case):
    """Inversion and prediction through the two-stage column passes against the
    FP64 direct transform (sampled pixels and visibilities), eps = 1e-5."""
    W, dl, eps = case["W"], case["dl"], 1e-5
    uvw, freq, vis = synthetic.random_points(800, 4, W, dl, seed=9, w_scale=0.5)
    wl = uvw[:, 2:3] * (freq / C)[None, :]
    p = _lib.make_plan(width=W, height=W, dl=dl, dm=dl, epsilon=eps, w_min=float(wl.min()),
                       w_max=float(wl.max()), n_vis=int(wl.size), force_sigma=1.5)
    assert (p.fft_n1, p.fft_n2) == case["split"]
    rng = np.random.default_rng(11)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps, num_t=np.float64)
    g.pin_plan(p)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    g.FinalizeImage(1.0)
    img = g.RealImage().astype(np.float64).ravel()
    pix = rng.choice(W * W, size=4096, replace=False)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, pixels=pix)
    assert rel(img[pix], ref) <= eps
    model = np.zeros(W * W, np.float32)
    src = rng.choice(W * W, size=6, replace=False)
    model[src] = rng.uniform(-1, 1, 6)
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq).ravel()
    pr = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl)
    assert rel(pv, np.asarray(pr).ravel()) <= eps
    g.close()


PRED_CASES = [
    dict(W=128, dl=4e-4, eps=1e-4, shift=(0.0, 0.0), w_scale=3.0, n_src=12),
    dict(W=256, dl=2e-4, eps=1e-5, shift=(0.01, -0.005), w_scale=2.0, n_src=40),
    dict(W=128, dl=4e-4, eps=1e-5, shift=(0.0, 0.0), w_scale=0.0, n_src=5),
]


@pytest.mark.parametrize("case", PRED_CASES)
def test_prediction_matches_dft_and_cpu_gridder(wgpu_lib, oracle_lib, case):
    W, dl, eps = case["W"], case["dl"], case["eps"]
    uvw, freq, _ = synthetic.random_points(800, 4, W, dl, seed=6, w_scale=case["w_scale"])
    rng = np.random.default_rng(3)
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, case["n_src"], replace=False)] = rng.uniform(-1, 1, case["n_src"])
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, case["shift"][0], case["shift"][1], 1,
                                epsilon=eps)
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    plan = g.last_plan()
    pr = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl, *case["shift"])
    assert rel(pv, pr) <= eps
    cpu = oracle_lib.wgrid_predict(plan, uvw, freq, model)
    assert rel(pv, cpu) <= eps
    g.close()


def test_prediction_is_adjoint_of_inversion(wgpu_lib):
    W, dl = 128, 4e-4
    uvw, freq, vis = synthetic.random_points(700, 4, W, dl, seed=12, w_scale=2.0)
    rng = np.random.default_rng(5)
    img = rng.standard_normal(W * W).astype(np.float32)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.003, 0.001, 1, epsilon=1e-5,
                                num_t=np.float64)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    a = g.RealImage().astype(np.float64)
    g.InitializePrediction(img)
    b = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq).astype(np.complex128)
    lhs = float(np.dot(a, img))
    rhs = float(np.real(np.vdot(b, vis.ravel().astype(np.complex128))))
    assert abs(lhs - rhs) <= 3e-5 * abs(lhs)
    g.close()


def test_golden_dft_fixture_through_gpu(wgpu_lib):
    gld = np.load(os.path.join(GOLDEN, "dft_small.npz"))
    W, dl = int(gld["width"]), float(gld["dl"])
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, float(gld["l_shift"]), float(gld["m_shift"]),
                                1, epsilon=1e-5, num_t=np.float64)
    g.InitializeInversion()
    g.AddInversionData(gld["uvw"].shape[0], gld["freq"].size, gld["uvw"], gld["freq"], gld["vis"])
    assert rel(g.RealImage(), gld["image"]) <= 1e-5
    g.InitializePrediction(gld["model"].astype(np.float32))
    pv = g.PredictVisibilities(gld["uvw"].shape[0], gld["freq"].size, gld["uvw"], gld["freq"])
    assert rel(pv, gld["pred"]) <= 1e-5
    g.close()


def test_empty_and_all_zero_inputs(wgpu_lib):
    W, dl = 64, 1e-3
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1)
    g.InitializeInversion()
    g.AddInversionData(0, 4, np.zeros((0, 3)), np.linspace(1e8, 2e8, 4),
                       np.zeros((0, 4), np.complex64))
    g.AddInversionData(10, 2, np.ones((10, 3)), np.array([1e8, 1.1e8]),
                       np.zeros((10, 2), np.complex64))
    assert np.all(g.RealImage() == 0)
    g.close()


def test_call_order_errors(wgpu_lib):
    g = WGriddingGridder_Simple(64, 64, 64, 64, 1e-3, 1e-3, 0, 0, 1)
    with pytest.raises(_lib.WgpuError) as e:
        g.AddInversionData(1, 1, np.zeros((1, 3)), np.array([1e8]), np.ones(1, np.complex64))
    assert e.value.status == _lib.WGPU_ERR_STATE
    with pytest.raises(_lib.WgpuError) as e:
        g.PredictVisibilities(1, 1, np.zeros((1, 3)), np.array([1e8]))
    assert e.value.status == _lib.WGPU_ERR_STATE
    g.close()


MODES = [("xx", 1, 2), ("yy", 1, 4), ("trace", 1, 4), ("diagonal", 2, 2), ("diagonal", 2, 4),
         ("full", 4, 4)]


@pytest.mark.parametrize("mode,n_pol,nparms", MODES)
def test_corrected_inversion_matches_oracle_gains(wgpu_lib, oracle_lib, mode, n_pol, nparms):
    from wsclean_gb300.gridder import GainMode
    W, dl = 128, 4e-4
    rng = np.random.default_rng(21)
    n_rows, n_chan, n_ant, n_t = 400, 4, 8, 3
    uvw, freq, _ = synthetic.random_points(n_rows, n_chan, W, dl, seed=22, w_scale=1.0)
    vis = (rng.standard_normal((n_rows, n_chan, n_pol)) +
           1j * rng.standard_normal((n_rows, n_chan, n_pol))).astype(np.complex64)
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], 1)
    tof = rng.integers(0, n_t, n_rows)
    sol = (1 + 0.3 * (rng.standard_normal((n_t, n_chan, n_ant, nparms)) +
                      1j * rng.standard_normal((n_t, n_chan, n_ant, nparms)))).astype(np.complex64)
    corrected = oracle_lib.apply_gains(GainMode[mode], n_pol, vis, ant, tof, sol, nparms, n_ant)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=1e-5, num_t=np.float64)
    g.InitializeInversion()
    g.AddInversionDataWithCorrectionCallback(mode, n_pol, n_rows, uvw, freq, n_chan, ant, vis,
                                             tof, sol, nparms, n_t, n_ant)
    got = g.RealImage().astype(np.float64)
    g.InitializeInversion()
    g.AddInversionData(n_rows, n_chan, uvw, freq, corrected)
    exp = g.RealImage().astype(np.float64)
    assert rel(got, exp) <= 2e-6
    ref = oracle_lib.dft_invert(uvw, freq, corrected, W, W, dl, dl)
    assert rel(got, ref) <= 1e-5
    g.close()


@pytest.mark.parametrize("mode,n_pol,nparms", MODES)
def test_corrected_prediction_matches_oracle_gains(wgpu_lib, oracle_lib, mode, n_pol, nparms):
    """Prediction write-back on the device (expansion + forward gains) against
    the oracle's write-back of the same predicted values and of the FP64
    direct prediction."""
    from wsclean_gb300.gridder import GainMode
    W, dl = 128, 4e-4
    rng = np.random.default_rng(23)
    n_rows, n_chan, n_ant, n_t = 400, 4, 8, 3
    uvw, freq, _ = synthetic.random_points(n_rows, n_chan, W, dl, seed=24, w_scale=1.0)
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], 1)
    tof = rng.integers(0, n_t, n_rows)
    sol = (1 + 0.3 * (rng.standard_normal((n_t, n_chan, n_ant, nparms)) +
                      1j * rng.standard_normal((n_t, n_chan, n_ant, nparms)))).astype(np.complex64)
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 8, replace=False)] = rng.uniform(-1, 1, 8)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=1e-5, num_t=np.float64)
    g.InitializePrediction(model)
    got = g.PredictVisibilitiesWithCorrection(mode, n_pol, n_rows, uvw, freq, n_chan, ant, tof,
                                              sol, nparms, n_t, n_ant)
    got = got.reshape(n_rows, n_chan, n_pol)
    plain = g.PredictVisibilities(n_rows, n_chan, uvw, freq).reshape(n_rows, n_chan)
    exp = oracle_lib.forward_gains(GainMode[mode], n_pol, plain, ant, tof, sol, nparms, n_ant)
    assert rel(got, exp) <= 1e-6
    dft = np.asarray(oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl)).reshape(n_rows, n_chan)
    ref = oracle_lib.forward_gains(GainMode[mode], n_pol, dft, ant, tof, sol, nparms, n_ant)
    assert rel(got, ref) <= 1e-5
    g.close()


def test_corrected_inversion_rejects_bad_indices(wgpu_lib):
    W, dl = 64, 1e-3
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1)
    g.InitializeInversion()
    uvw, freq, _ = synthetic.random_points(4, 2, W, dl, seed=1)
    vis = np.ones((4, 2, 1), np.complex64)
    ant = np.array([[0, 1], [0, 2], [1, 9], [0, 1]])
    sol = np.ones((1, 2, 3, 2), np.complex64)
    with pytest.raises(_lib.WgpuError) as e:
        g.AddInversionDataWithCorrectionCallback("xx", 1, 4, uvw, freq, 2, ant, vis,
                                                 np.zeros(4, np.uint64), sol, 2, 1, 3)
    assert e.value.status == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError):
        g.AddInversionDataWithCorrectionCallback("full", 1, 4, uvw, freq, 2, ant, vis,
                                                 np.zeros(4, np.uint64), sol, 2, 1, 3)
    g.close()


def test_bound_cycles_match_unbound_calls(wgpu_lib, oracle_lib):
    """Device-resident state across major cycles: bind once, then grid and
    predict twice through the captured graphs; each result equals the plain
    per-call path (same plan) and the DFT within epsilon."""
    W, dl, eps = 192, 3e-4, 1e-5
    uvw, freq, vis1 = synthetic.random_points(900, 6, W, dl, seed=51, w_scale=2.0)
    _, _, vis2 = synthetic.random_points(900, 6, W, dl, seed=52, w_scale=2.0)
    rng = np.random.default_rng(9)
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 25, replace=False)] = rng.uniform(-1, 1, 25)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.002, -0.001, 1, epsilon=eps,
                                num_t=np.float64)
    g.Bind(uvw.shape[0], freq.size, uvw, freq)
    bound_plan = g.last_plan()
    ref_g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.002, -0.001, 1, epsilon=eps,
                                    num_t=np.float64)
    ref_g.pin_plan(bound_plan)
    for cycle, vis in enumerate((vis1, vis2, vis1)):
        g.InitializeInversion()
        g.InvertBound(vis)
        img = g.RealImage().astype(np.float64)
        ref_g.InitializeInversion()
        ref_g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
        assert rel(img, ref_g.RealImage()) <= 2e-6, cycle
        if cycle < 2:
            dft = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, 0.002, -0.001)
            assert rel(img, dft) <= eps
        g.InitializePrediction(model)
        pv = g.PredictBound()
        ref_g.InitializePrediction(model)
        pr = ref_g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
        assert rel(pv, pr) <= 2e-6, cycle
    g.close()
    ref_g.close()


def test_bound_mask_selects_samples(wgpu_lib):
    W, dl = 128, 4e-4
    uvw, freq, vis = synthetic.random_points(500, 4, W, dl, seed=53, w_scale=1.0)
    mask = (np.random.default_rng(2).uniform(size=vis.shape) > 0.3).astype(np.uint8)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=1e-4)
    g.Bind(uvw.shape[0], freq.size, uvw, freq, mask)
    g.InitializeInversion()
    g.InvertBound(vis)
    img = g.RealImage()
    g.pin_plan(g.last_plan())
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, np.where(mask > 0, vis, 0))
    assert rel(img, g.RealImage()) <= 2e-6
    model = np.zeros(W * W, np.float32)
    model[1234] = 1.0
    g.InitializePrediction(model)
    pv = g.PredictBound().reshape(vis.shape)
    assert np.all(pv[mask == 0] == 0)
    pm = g.PredictVisibilitiesMasked(uvw.shape[0], freq.size, uvw, freq, mask).reshape(vis.shape)
    assert rel(pv, pm) <= 2e-6
    g.close()


def test_bound_split_units_over_plane_batches(wgpu_lib, oracle_lib):
    """Dense set over two plane batches in which 72 gridding units need more
    than one work item (more than 2048 visibility reads): the bound graphs
    equal the plain path with the same plan, and the DFT within epsilon."""
    W, dl, eps = 64, 5e-3, 1e-4
    uvw, freq, vis = synthetic.random_points(8000, 32, W, dl, seed=71, w_scale=3.0)
    plan = _plan_for(uvw, freq, None, W, dl, eps, max_plane_batch=16)
    assert plan.n_planes > plan.plane_batch
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=eps)
    g.pin_plan(plan)
    g.Bind(uvw.shape[0], freq.size, uvw, freq)
    ref_g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=eps)
    ref_g.pin_plan(plan)
    rng = np.random.default_rng(12)
    for cycle in range(2):
        g.InitializeInversion()
        g.InvertBound(vis)
        img = g.RealImage().astype(np.float64)
        ref_g.InitializeInversion()
        ref_g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
        assert rel(img, ref_g.RealImage()) <= 2e-6, cycle
    pix = rng.choice(W * W, 512, replace=False)
    dft = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, pixels=pix)
    assert rel(img[pix], dft) <= eps
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 10, replace=False)] = rng.uniform(-1, 1, 10)
    g.InitializePrediction(model)
    pv = g.PredictBound()
    ref_g.InitializePrediction(model)
    pr = ref_g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    assert rel(pv, pr) <= 2e-6
    sel = rng.choice(pv.size, 4096, replace=False)
    pd = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl, vis_index=sel)
    assert rel(pv[sel], pd) <= eps
    g.close()
    ref_g.close()


@pytest.mark.parametrize("shift", [(0.0, 0.0), (0.03, -0.02)])
def test_many_w_planes_within_epsilon(wgpu_lib, oracle_lib, shift):
    """A wide field (0.5 rad across) with large w needs about 650 w planes in
    batches of 32: the screen phase of plane q, formed from per-pixel
    fixed-point terms as (a + q k) 2^-32 + q r turns, stays within epsilon of
    the FP64 direct transform for every q, in both directions."""
    W, dl, eps = 64, 8e-3, 1e-5
    uvw, freq, vis = synthetic.random_points(300, 4, W, dl, seed=81, w_scale=60.0)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, shift[0], shift[1], 1, epsilon=eps)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    plan = g.last_plan()
    assert plan.n_planes > 600 and plan.n_planes > 8 * plan.plane_batch
    img = g.RealImage().astype(np.float64)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, *shift)
    assert rel(img, ref) <= eps
    rng = np.random.default_rng(5)
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 20, replace=False)] = rng.uniform(-1, 1, 20)
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    pr = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl, *shift)
    assert rel(pv.ravel(), pr.ravel()) <= eps
    g.close()


def test_bounded_wait_expires_and_device_stays_usable(wgpu_lib):
    """A bounded device wait on a barrier that nothing arrives at expires,
    is reported as WGPU_ERR_TIMEOUT, and later work runs normally."""
    st = wgpu_lib.wgpu_selftest_bounded_wait(50.0)
    assert st == _lib.WGPU_ERR_TIMEOUT
    assert b"expired" in wgpu_lib.wgpu_last_error()
    W, dl = 64, 1e-3
    uvw, freq, vis = synthetic.random_points(100, 2, W, dl, seed=91)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=1e-4)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    assert np.isfinite(g.RealImage()).all()
    g.close()


def test_row_length_6912_inversion_and_prediction(wgpu_lib, oracle_lib):
    """A 5088-pixel image plans 6912-cell rows, the longest row the one-CTA-per-
    row transform takes: its thread count is clamped to the kernel's launch
    bound (6912 / 16 = 432 threads, not a whole number of warps)."""
    W, dl, eps = 5088, 4.848e-5, 1e-4
    uvw, freq, vis = synthetic.random_points(400, 4, W, dl, seed=61, w_scale=0.02)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    assert g.last_plan().nu == 6912
    img = g.RealImage().astype(np.float64)
    rng = np.random.default_rng(62)
    pix = rng.choice(W * W, 256, replace=False)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, pixels=pix)
    assert rel(img[pix], ref) <= eps
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 5, replace=False)] = 1.0
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    pr = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl)
    assert rel(pv.ravel(), pr) <= eps
    g.close()


@pytest.mark.parametrize("n_chan,order", [(24, "ascending"), (24, "descending"), (24, "shuffled"),
                                          (24, "repeated"), (8, "ascending"), (64, "ascending")])
def test_device_w_extent_gives_the_host_plan(wgpu_lib, n_chan, order):
    """The w range a call plans from (the device extent pass over the selected
    samples) equals the host's FP64 extent exactly, so the call's plan is the
    host plan bit for bit, for inversions (zero visibilities skipped) and
    masked predictions, with ascending, descending, unordered and repeated
    channel frequencies, with 16 or more channels (one warp per row, two
    products per row) and with fewer (one product per sample)."""
    W, dl = 192, 3e-4
    uvw, freq, vis = synthetic.random_points(900, n_chan, W, dl, seed=71, w_scale=3.0,
                                             frac_zero=0.3)
    if order == "descending":
        freq = freq[::-1].copy()
    elif order == "shuffled":
        freq = np.random.default_rng(5).permutation(freq)
    elif order == "repeated":  # equal frequencies: ranks tie-broken by channel
        freq = np.random.default_rng(6).permutation(np.repeat(freq[: n_chan // 3], 3))
    vis[:40] = 0  # whole rows without a sample
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=1e-4)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    got = g.last_plan()
    ref = _plan_for(uvw, freq, vis, W, dl, 1e-4)
    assert (got.w0, got.dw, got.n_planes) == (ref.w0, ref.dw, ref.n_planes)
    mask = (vis != 0).astype(np.uint8)
    model = np.zeros(W * W, np.float32)
    model[W * W // 2 + 7] = 1.0
    g.InitializePrediction(model)
    g.PredictVisibilitiesMasked(uvw.shape[0], freq.size, uvw, freq, mask)
    got = g.last_plan()
    assert (got.w0, got.dw, got.n_planes) == (ref.w0, ref.dw, ref.n_planes)
