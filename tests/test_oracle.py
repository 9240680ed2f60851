"""Oracle checks (CPU): golden vectors, analytic known answers, and the FP64
CPU w-gridder against the direct Fourier transform."""
import json
import os

import numpy as np
import pytest

from wsclean_gb300 import synthetic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
C = 299792458.0


def _cplx(lst):
    return np.array([a + 1j * b for a, b in lst], np.complex64)


def test_gain_known_answers(oracle_lib):
    """tests/gridding/tvisibilitymodifier.cpp apply_h5parm / apply_conjugate_h5parm."""
    kat = json.load(open(os.path.join(GOLDEN, "gains_kat.json")))
    for case in kat["cases"]:
        vis, g1, g2 = _cplx(case["vis"]), _cplx(case["g1"]), _cplx(case["g2"])
        fn = oracle_lib.apply_gain if case["direction"] == "forward" else \
            oracle_lib.apply_conjugated_gain
        out = fn(case["mode"], vis, g1, g2)
        exp = _cplx(case["expected"])
        # BOOST_CHECK_CLOSE_FRACTION(a, b, 1e-5) on real and imaginary parts
        np.testing.assert_allclose(out.real, exp.real, rtol=kat["tolerance"])
        np.testing.assert_allclose(out.imag, exp.imag, rtol=kat["tolerance"])


def test_gain_modes_against_matrix_algebra(oracle_lib):
    rng = np.random.default_rng(2)
    g1 = (rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64)
    g2 = (rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64)
    v = (rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64)
    G1, G2, V = g1.reshape(2, 2), g2.reshape(2, 2), v.reshape(2, 2)
    full = oracle_lib.apply_conjugated_gain(4, v, g1, g2)
    np.testing.assert_allclose(full, (G1.conj().T @ V @ G2).ravel(), rtol=1e-5, atol=1e-5)
    xx = oracle_lib.apply_conjugated_gain(0, v[:1], g1, g2)
    np.testing.assert_allclose(xx[0], np.conj(g1[0]) * v[0] * g2[0], rtol=1e-5)
    yy = oracle_lib.apply_conjugated_gain(1, v[:1], g1, g2)
    np.testing.assert_allclose(yy[0], np.conj(g1[3]) * v[0] * g2[3], rtol=1e-5)
    tr = oracle_lib.apply_conjugated_gain(2, v[:1], g1, g2)
    np.testing.assert_allclose(tr[0], v[0] * 0.5 * np.sum(g2 * np.conj(g1)), rtol=1e-5)
    dg = oracle_lib.apply_conjugated_gain(3, v[:2], g1, g2)
    v0 = np.conj(g1[0]) * v[0] * g2[0] + np.conj(g1[2]) * v[1] * g2[2]
    v1 = np.conj(g1[3]) * v[1] * g2[3] + np.conj(g1[1]) * v0 * g2[1]
    np.testing.assert_allclose(dg, [v0, v1], rtol=1e-5, atol=1e-5)


def test_gains_table_layout_and_collapse(oracle_lib):
    rng = np.random.default_rng(4)
    n_rows, n_chan, n_ant, n_t = 12, 3, 5, 2
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], 1)
    tof = rng.integers(0, n_t, n_rows)
    sol = (rng.standard_normal((n_t, n_chan, n_ant, 4)) +
           1j * rng.standard_normal((n_t, n_chan, n_ant, 4))).astype(np.complex64)
    vis = (rng.standard_normal((n_rows, n_chan, 4)) +
           1j * rng.standard_normal((n_rows, n_chan, 4))).astype(np.complex64)
    out = oracle_lib.apply_gains(4, 4, vis, ant, tof, sol, 4, n_ant, polarization=0)
    for r in range(n_rows):
        for c in range(n_chan):
            G1 = sol[tof[r], c, ant[r, 0]].reshape(2, 2)
            G2 = sol[tof[r], c, ant[r, 1]].reshape(2, 2)
            M = G1.conj().T @ vis[r, c].reshape(2, 2) @ G2
            np.testing.assert_allclose(out[r, c], 0.5 * (M[0, 0] + M[1, 1]), rtol=1e-4, atol=1e-5)
    # 2-pol: diagonal solutions, collapse = v0 + v1
    sol2 = sol[..., :2].copy()
    vis2 = vis[..., :2].copy()
    out2 = oracle_lib.apply_gains(3, 2, vis2, ant, tof, sol2, 2, n_ant)
    r, c = 3, 1
    a, b = sol2[tof[r], c, ant[r, 0]], sol2[tof[r], c, ant[r, 1]]
    exp = np.conj(a[0]) * vis2[r, c, 0] * b[0] + np.conj(a[1]) * vis2[r, c, 1] * b[1]
    np.testing.assert_allclose(out2[r, c], exp, rtol=1e-4)
    with pytest.raises(ValueError):
        oracle_lib.apply_gains(0, 2, vis2, ant, tof, sol2, 2, n_ant)


def test_forward_gains_expand_and_match_matrix_algebra(oracle_lib):
    """Prediction write-back: with identity gains the 4-correlation expansion
    collapses back to the predicted value for every polarisation; with random
    gains each mode equals its matrix form (G1 V G2^H on the expanded value)."""
    rng = np.random.default_rng(9)
    n_rows, n_chan, n_ant, n_t = 5, 3, 4, 2
    vis = (rng.standard_normal((n_rows, n_chan)) +
           1j * rng.standard_normal((n_rows, n_chan))).astype(np.complex64)
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], 1)
    tof = rng.integers(0, n_t, n_rows)
    eye = np.zeros((n_t, n_chan, n_ant, 4), np.complex64)
    eye[..., 0] = eye[..., 3] = 1
    for pol in range(8):
        lin = oracle_lib.forward_gains(4, 4, vis, ant, tof, eye, 4, n_ant, polarization=pol)
        back = oracle_lib.apply_gains(4, 4, lin, ant, tof, eye, 4, n_ant, polarization=pol)
        np.testing.assert_allclose(back, vis, rtol=1e-6, atol=1e-6)
    sol = (rng.standard_normal((n_t, n_chan, n_ant, 4)) +
           1j * rng.standard_normal((n_t, n_chan, n_ant, 4))).astype(np.complex64)
    full = oracle_lib.forward_gains(4, 4, vis, ant, tof, sol, 4, n_ant, polarization=0)
    xx = oracle_lib.forward_gains(0, 1, vis, ant, tof, sol, 4, n_ant)
    dg = oracle_lib.forward_gains(3, 2, vis, ant, tof, sol, 4, n_ant)
    for r in range(n_rows):
        for c in range(n_chan):
            g1 = sol[tof[r], c, ant[r, 0]].astype(np.complex128).reshape(2, 2)
            g2 = sol[tof[r], c, ant[r, 1]].astype(np.complex128).reshape(2, 2)
            v = vis[r, c]
            want = g1 @ np.array([[v, 0], [0, v]]) @ g2.conj().T
            np.testing.assert_allclose(full[r, c], want.ravel(), rtol=1e-5, atol=1e-5)
            np.testing.assert_allclose(xx[r, c, 0], g1[0, 0] * v * np.conj(g2[0, 0]),
                                       rtol=1e-5, atol=1e-5)
            # diagonal mode: the second value uses the updated first one
            # (visibilitymodifier.h:359-362)
            v0 = g1[0, 0] * v * np.conj(g2[0, 0]) + g1[0, 1] * v * np.conj(g2[0, 1])
            v1 = g1[1, 1] * v * np.conj(g2[1, 1]) + g1[1, 0] * v0 * np.conj(g2[1, 0])
            np.testing.assert_allclose(dg[r, c], [v0, v1], rtol=1e-5, atol=1e-5)


def test_dft_constant_visibility_gives_flat_image(oracle_lib):
    uvw = np.zeros((1, 3))
    freq = np.array([1e8])
    vis = np.array([[1.0 + 0.0j]], np.complex64)
    img = oracle_lib.dft_invert(uvw, freq, vis, 16, 16, 1e-3, 1e-3)
    np.testing.assert_allclose(img, 1.0, atol=1e-12)


def test_dft_point_source_orientation(oracle_lib):
    """A source at l > 0, m > 0 lands left of centre (x < W/2) and above it
    (y > H/2): l = (W/2 - x) dl + l_shift, m = (y - H/2) dm + m_shift
    (directmsgridder.cpp:113-124, :70-82)."""
    W, dl = 32, 2e-3
    x0, y0 = 10, 21
    l0 = (W / 2 - x0) * dl + 0.001
    m0 = (y0 - W / 2) * dl - 0.002
    rng = np.random.default_rng(0)
    uvw = rng.uniform(-150, 150, (400, 3))
    freq = np.array([1e8, 1.5e8])
    vis = synthetic.model_vis_numpy(uvw, freq, np.array([[l0, m0, 2.0]])).astype(np.complex64)
    img = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, 0.001, -0.002)
    assert int(np.argmax(img)) == x0 + y0 * W
    assert abs(img[x0 + y0 * W] - 2.0 * 800) < 1e-2


def test_dft_golden_fixture(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "dft_small.npz"))
    W = int(g["width"])
    img = oracle_lib.dft_invert(g["uvw"], g["freq"], g["vis"], W, W, float(g["dl"]),
                                float(g["dl"]), float(g["l_shift"]), float(g["m_shift"]))
    np.testing.assert_allclose(img, g["image"], rtol=1e-9, atol=1e-9)
    pred = oracle_lib.dft_predict(g["uvw"], g["freq"], g["model"], W, W, float(g["dl"]),
                                  float(g["dl"]), float(g["l_shift"]), float(g["m_shift"]))
    np.testing.assert_allclose(pred, g["pred"], rtol=1e-9, atol=1e-9)


def test_dft_predict_is_adjoint_of_invert(oracle_lib):
    W, dl = 24, 2e-3
    uvw, freq, vis = synthetic.random_points(50, 3, W, dl, seed=9, w_scale=2.0)
    rng = np.random.default_rng(1)
    img = rng.standard_normal(W * W)
    a = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, 0.01, 0.02)
    b = oracle_lib.dft_predict(uvw, freq, img, W, W, dl, dl, 0.01, 0.02)
    lhs = np.dot(a, img)
    rhs = np.real(np.vdot(b, vis.ravel().astype(np.complex128)))
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)


def test_bucket_golden_fixture(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "bucket_small.npz"))
    plan = json.loads(str(g["plan"]))
    b = oracle_lib.bucket(plan, g["uvw"], g["freq"], g["vis"], True)
    for k in ("perm", "key", "iu", "iv", "ip", "fu", "fv", "fw", "offsets"):
        np.testing.assert_array_equal(b[k], g[k], err_msg=k)
    # properties: sorted by (key, corner inside the tile, element index), offsets
    tile = int(plan["tile"])
    corner = (b["iv"] % tile) * tile + b["iu"] % tile
    order = np.lexsort((b["perm"], corner, b["key"]))
    np.testing.assert_array_equal(order, np.arange(b["perm"].size))
    assert b["offsets"][-1] == b["perm"].size
    assert np.all(g["vis"].ravel()[b["perm"]] != 0)


@pytest.mark.parametrize("eps,shift", [(1e-4, (0.0, 0.0)), (1e-5, (0.01, -0.005))])
def test_cpu_wgridder_matches_dft(oracle_lib, wgpu_lib, eps, shift):
    from wsclean_gb300 import _lib
    W, dl = 96, 4e-4
    uvw, freq, vis = synthetic.random_points(250, 4, W, dl, seed=3, w_scale=3.0, frac_zero=0.1)
    wl = (uvw[:, 2:3] * (freq / C)[None, :])[vis != 0]
    p = _lib.make_plan(width=W, height=W, dl=dl, dm=dl, l_shift=shift[0], m_shift=shift[1],
                       epsilon=eps, w_min=wl.min(), w_max=wl.max(), n_vis=int((vis != 0).sum()))
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl, *shift)
    img = oracle_lib.wgrid_invert(p, uvw, freq, vis)
    assert np.linalg.norm(img - ref) / np.linalg.norm(ref) <= eps
    model = np.zeros(W * W)
    model[[5, 4000, 7777]] = [1.0, 0.3, -0.2]
    pv = oracle_lib.wgrid_predict(p, uvw, freq, model)
    pr = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl, *shift)
    assert np.linalg.norm(pv - pr) / np.linalg.norm(pr) <= eps


def test_es_fourier_matches_numeric_integral(oracle_lib):
    beta, W = 14.65, 8
    z = np.linspace(-1, 1, 200001)
    phi = np.exp(beta * (np.sqrt(1 - z * z) - 1))
    for f in (0.0, 0.1, 0.37):
        num = (W / 2) * np.trapezoid(phi * np.cos(np.pi * f * W * z), z)
        assert abs(oracle_lib.es_fourier(beta, W, f) - num) < 1e-6 * abs(num)


def test_correction_matrix_known_answers(oracle_lib):
    """AverageCorrection::Add in matrix form against the correction-sum known
    answers of tests/gridding/tvisibilitymodifier.cpp:128-136 (diagonal gains,
    unit weights), and its algebra: Hermitian, and for full Jones the
    symmetrised Kronecker form 0.5 w (P (x) Q + Q (x) P), P = G1^H G1,
    Q = G2^H G2."""
    kat = json.load(open(os.path.join(GOLDEN, "gains_kat.json")))
    case = next(c for c in kat["cases"] if "correction_sum" in c)
    m = oracle_lib.correction_matrix_add(_cplx(case["g1"]), _cplx(case["g2"]), 1.0)
    for k, v in case["correction_sum"].items():
        np.testing.assert_allclose(m.ravel()[int(k)].real, v, rtol=kat["tolerance"])
    rng = np.random.default_rng(8)
    g1 = (rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64)
    g2 = (rng.standard_normal(4) + 1j * rng.standard_normal(4)).astype(np.complex64)
    m = oracle_lib.correction_matrix_add(g1, g2, 0.7)
    np.testing.assert_allclose(m, m.conj().T, atol=1e-12)
    G1, G2 = g1.astype(np.complex128).reshape(2, 2), g2.astype(np.complex128).reshape(2, 2)
    P, Q = G1.conj().T @ G1, G2.conj().T @ G2
    np.testing.assert_allclose(m, 0.5 * 0.7 * (np.kron(P, Q) + np.kron(Q, P)), rtol=1e-12)
    # sums accumulate
    np.testing.assert_allclose(oracle_lib.correction_matrix_add(g1, g2, 0.7, total=m), 2 * m,
                               rtol=1e-12)
