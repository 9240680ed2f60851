"""Imaging weights and raw-row weighting on the GPU against the oracle.

Cell indices, the natural / uniform grids (dyadic weights, whose sums are exact
in any order), the rank filter, the uv limits, GetGrid, GetWeight and the
prepared rows are bit-exact.  Sums formed by parallel reductions (the Briggs
sum of squares, the gridded weight total with arbitrary weights, the weight
sums of ApplyWeights) agree to 1e-12 relative; tapers evaluated with cos / exp
to 1e-14; PSF phasors (double sincos rounded to float) to 2 float ulps."""
import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple
from wsclean_gb300.weights import BRIGGS, NATURAL, UNIFORM, ImageWeights, prepare_rows

from test_weights_oracle import PREP_CASES, TAPERS

pytestmark = pytest.mark.gpu

PSX = 0.004


def big_rows(seed, n_rows=3000, n_chan=16, n_pol=4, dyadic=True):
    rng = np.random.default_rng(seed)
    uvw = rng.normal(0.0, 160.0, (n_rows, 3))
    freq = np.linspace(1.0e8, 1.6e8, n_chan)
    if dyadic:
        weights = (rng.integers(0, 17, (n_rows, n_chan, n_pol)) / 8.0).astype(np.float32)
    else:
        weights = rng.uniform(0.0, 3.0, (n_rows, n_chan, n_pol)).astype(np.float32)
    vis = (rng.standard_normal((n_rows, n_chan, n_pol)) +
           1j * rng.standard_normal((n_rows, n_chan, n_pol))).astype(np.complex64)
    return uvw, freq, weights, vis


def pair(oracle_lib, mode, robust=0.0, as_taper=False, size=(300, 220), super_weight=1.0,
         data=None):
    args = (mode, size[0], size[1], PSX, PSX * 1.2, as_taper, super_weight, robust)
    dev, ref = ImageWeights(*args), oracle_lib.ImageWeights(*args)
    uvw, freq, weights, _ = data if data is not None else big_rows(7)
    half = uvw.shape[0] // 2
    for sl in (slice(0, half), slice(half, None)):  # two chunks, as Grid is called per chunk
        dev.Grid(uvw[sl], freq, weights[sl])
        ref.grid_rows(uvw[sl], freq, weights[sl])
    return dev, ref


@pytest.mark.parametrize("mode,robust,as_taper", [(NATURAL, 0.0, False),
                                                   (UNIFORM, 0.0, False),
                                                   (UNIFORM, 0.0, True),
                                                   (BRIGGS, 0.5, False),
                                                   (BRIGGS, -1.5, False)])
def test_weight_grid_matches_oracle(oracle_lib, mode, robust, as_taper):
    dev, ref = pair(oracle_lib, mode, robust, as_taper)
    assert (dev.Width(), dev.Height()) == (ref.width, ref.height)
    np.testing.assert_array_equal(dev.half_grid(), ref.grid)
    assert dev.TotalSum() == ref.total
    assert np.count_nonzero(ref.grid) > 1000
    dev.FinishGridding()
    ref.finish()
    if mode == BRIGGS:
        np.testing.assert_allclose(dev.half_grid(), ref.grid, rtol=1e-12, atol=0)
    else:
        np.testing.assert_array_equal(dev.half_grid(), ref.grid)


def test_weight_grid_arbitrary_weights_and_super_weight(oracle_lib):
    dev, ref = pair(oracle_lib, UNIFORM, super_weight=2.5,
                    data=big_rows(8, dyadic=False))
    assert (dev.Width(), dev.Height()) == (ref.width, ref.height) == (120, 88)
    np.testing.assert_allclose(dev.half_grid(), ref.grid, rtol=1e-12, atol=0)
    assert np.array_equal(dev.half_grid() != 0, ref.grid != 0)
    np.testing.assert_allclose(dev.TotalSum(), ref.total, rtol=1e-12)


@pytest.mark.parametrize("kind,a,b", TAPERS + [(1, 80.0, 0.0), (6, 0.02, 0.0)])
def test_weight_tapers_match_oracle(oracle_lib, kind, a, b):
    dev, ref = pair(oracle_lib, UNIFORM)
    dev.FinishGridding()
    ref.finish()
    dev._taper(kind, a, b)
    ref.taper(kind, a, b)
    if kind in (2, 3, 5, 6):  # cos / exp in double
        np.testing.assert_allclose(dev.half_grid(), ref.grid, rtol=1e-14, atol=0)
    else:
        np.testing.assert_array_equal(dev.half_grid(), ref.grid)


def test_weight_get_grid_and_get_weight_match_oracle(oracle_lib):
    dev, ref = pair(oracle_lib, BRIGGS, 0.0)
    dev.FinishGridding()
    ref.finish()
    ref.grid[:] = dev.half_grid()  # sample the same values
    np.testing.assert_array_equal(dev.GetGrid(), ref.mirrored())
    rng = np.random.default_rng(9)
    u = rng.uniform(-140, 140, 20000)
    v = rng.uniform(-110, 110, 20000)
    u[:3], v[:3] = [0.0, -0.0, 1e300], [-0.0, 0.0, 1.0]
    np.testing.assert_array_equal(dev.GetWeight(u, v), ref.sample(u, v))
    assert dev.GetWeight(0.0, 0.0) == ref.sample([0.0], [0.0])[0]
    dev.SetAllValues(3.14)
    assert np.all(dev.half_grid() == 3.14)


def test_weight_call_order_errors():
    iw = ImageWeights(UNIFORM, 64, 64, PSX, PSX)
    uvw, freq, weights, _ = big_rows(1, n_rows=10, n_chan=2, n_pol=1)
    iw.Grid(uvw, freq, weights)
    iw.Grid(uvw[:0], freq, weights[:0])  # empty chunk
    iw.FinishGridding()
    with pytest.raises(_lib.WgpuError) as e:
        iw.FinishGridding()
    assert e.value.status == _lib.WGPU_ERR_STATE
    with pytest.raises(_lib.WgpuError):
        iw.Grid(uvw, freq, weights)
    with pytest.raises(_lib.WgpuError):
        ImageWeights(5, 64, 64, PSX, PSX)
    with pytest.raises(_lib.WgpuError):
        iw.RankFilter(1.0, -3)


def _prepare_pair(oracle_lib, case, n_rows=2500, n_chan=12):
    dev, ref = pair(oracle_lib, BRIGGS, 0.0)
    dev.FinishGridding()
    ref.finish()
    ref.grid[:] = dev.half_grid()  # same imaging weights on both sides
    uvw, freq, weights, vis = big_rows(21, n_rows=n_rows, n_chan=n_chan, n_pol=case["n_pol"],
                                       dyadic=False)
    rng = np.random.default_rng(22)
    model = (rng.standard_normal(vis.shape) + 1j * rng.standard_normal(vis.shape)).astype(
        np.complex64) if case["model"] else None
    sel = rng.random((n_rows, n_chan)) > 0.3 if case["sel"] else None
    dl, dm = case.get("dl", 0.0), case.get("dm", 0.0)
    settings = dict(psf_mode=case["psf_mode"], psf_dl=dl, psf_dm=dm,
                    subtract_model=case["model"], visibility_weighting=case["visw"],
                    polarization=case["pol"])
    return dev, ref, (uvw, freq, weights, vis, model, sel), settings


@pytest.mark.parametrize("case", PREP_CASES)
def test_prepare_rows_match_oracle(oracle_lib, case):
    dev, ref, (uvw, freq, weights, vis, model, sel), st = _prepare_pair(oracle_lib, case)
    got = prepare_rows(dev, uvw, freq, weights, vis, model, sel, **st)
    exp = ref.prepare_rows(uvw, freq, weights, None if st["psf_mode"] else vis, model, sel,
                           st["psf_mode"], st["psf_dl"], st["psf_dm"],
                           st["visibility_weighting"], st["polarization"])
    if st["psf_mode"] and (st["psf_dl"] or st["psf_dm"]):
        tol = 2 * np.finfo(np.float32).eps * np.abs(exp[0]).max()
        np.testing.assert_allclose(got[0], exp[0], rtol=0, atol=tol)
    else:
        np.testing.assert_array_equal(got[0], exp[0])
    np.testing.assert_array_equal(got[1], exp[1])
    np.testing.assert_array_equal(got[2], exp[2])
    s = got[3]
    assert s["gridded_visibility_count"] == exp[3][3] > 0
    assert s["max_gridded_weight"] == exp[3][1]
    np.testing.assert_allclose(s["visibility_weight_sum"], exp[3][0], rtol=1e-12)
    np.testing.assert_allclose(s["total_weight"], exp[3][2], rtol=1e-12)


def test_prepare_rows_nothing_selected(oracle_lib):
    case = dict(n_pol=2, psf_mode=0, visw=0, model=False, sel=True, pol=0)
    dev, _, (uvw, freq, weights, vis, _, sel), st = _prepare_pair(oracle_lib, case, 50, 3)
    out, w, iw, s = prepare_rows(dev, uvw, freq, weights, vis, None, np.zeros_like(sel), **st)
    assert not out.any() and not w.any()
    assert s["gridded_visibility_count"] == 0 and s["total_weight"] == 0.0
    empty = prepare_rows(dev, uvw[:0], freq, weights[:0], vis[:0], **st)
    assert empty[0].shape == (0, freq.size)


@pytest.mark.parametrize("n_pol,pol", [(1, 0), (4, 0)])
def test_add_inversion_rows_matches_prepared_inversion(oracle_lib, n_pol, pol):
    """Raw rows gridded through wgpu_gridder_add_inversion_rows give the image
    of the oracle-prepared visibilities gridded by AddInversionData, and that
    image matches the direct transform of the prepared visibilities."""
    W, Wt, dl, eps = 160, 128, 4e-4, 1e-5
    uvw, freq, vis1 = synthetic.random_points(900, 6, Wt, dl, seed=31, w_scale=2.0)
    rng = np.random.default_rng(32)
    vis = np.repeat(vis1[:, :, None], n_pol, axis=2) * (1.0 + 0.1 * rng.standard_normal(
        (vis1.shape[0], vis1.shape[1], n_pol)))
    vis = vis.astype(np.complex64)
    weights = rng.uniform(0.2, 2.0, vis.shape).astype(np.float32)
    sel = rng.random(vis.shape[:2]) > 0.1
    args = (BRIGGS, Wt, Wt, dl, dl, False, 1.0, 0.3)
    dev, ref = ImageWeights(*args), oracle_lib.ImageWeights(*args)
    dev.Grid(uvw, freq, weights)
    dev.FinishGridding()
    ref.grid[:] = dev.half_grid()
    prepared, _, _, sums = ref.prepare_rows(uvw, freq, weights, vis, None, sel, 0, 0.0, 0.0, 0,
                                            pol)
    assert np.count_nonzero(prepared) > prepared.size // 2

    g1 = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps,
                                 num_t=np.float64)
    g1.InitializeInversion()
    half = uvw.shape[0] // 2
    acc = None
    for sl in (slice(0, half), slice(half, None)):
        acc = g1.AddInversionRows(dev, uvw[sl], freq, weights[sl], vis[sl], selected=sel[sl],
                                  sums=acc, polarization=pol)
    g1.FinalizeImage(1.0)
    img_rows = g1.RealImage().reshape(W, W)

    g2 = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps,
                                 num_t=np.float64)
    g2.InitializeInversion()
    for sl in (slice(0, half), slice(half, None)):  # the same chunks, so the same plans
        g2.AddInversionData(uvw[sl].shape[0], freq.size, uvw[sl], freq, prepared[sl])
    g2.FinalizeImage(1.0)
    img_prep = g2.RealImage().reshape(W, W)

    d = (W - Wt) // 2
    a = img_rows[d:d + Wt, d:d + Wt].astype(np.float64)
    b = img_prep[d:d + Wt, d:d + Wt].astype(np.float64)
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    dft = oracle_lib.dft_invert(uvw, freq, prepared, Wt, Wt, dl, dl).reshape(Wt, Wt)
    assert np.linalg.norm(a - dft) <= eps * np.linalg.norm(dft)
    assert acc.gridded_visibility_count == sums[3]
    assert acc.max_gridded_weight == sums[1]
    np.testing.assert_allclose(acc.total_weight, sums[2], rtol=1e-12)
    np.testing.assert_allclose(acc.visibility_weight_sum, sums[0], rtol=1e-12)


def test_device_variants_match_host_variants(oracle_lib):
    torch = pytest.importorskip("torch")
    from wsclean_gb300.weights import prepare_rows_device
    dev = torch.device("cuda", 0)
    uvw, freq, weights, vis = big_rows(41, n_rows=1200, n_chan=8, n_pol=4, dyadic=False)
    a = ImageWeights(UNIFORM, 300, 220, PSX, PSX)
    b = ImageWeights(UNIFORM, 300, 220, PSX, PSX)
    a.Grid(uvw, freq, weights)
    t_uvw, t_freq = torch.as_tensor(uvw, device=dev), torch.as_tensor(freq, device=dev)
    t_w = torch.as_tensor(weights, device=dev)
    torch.cuda.synchronize()
    b.grid_device(uvw.shape[0], freq.size, 4, t_uvw.data_ptr(), t_freq.data_ptr(),
                  t_w.data_ptr())
    np.testing.assert_allclose(b.half_grid(), a.half_grid(), rtol=1e-12, atol=0)
    a.FinishGridding()
    st = dict(visibility_weighting=_lib.VISW_SQUARED, polarization=_lib.POL_Q)
    out, w, iw, s = prepare_rows(a, uvw, freq, weights, vis, **st)
    t_vis = torch.as_tensor(vis.view(np.float32), device=dev)
    t_out = torch.empty(out.size * 2, dtype=torch.float32, device=dev)
    t_wo = torch.empty(w.size, dtype=torch.float32, device=dev)
    sd = prepare_rows_device(a, 4, uvw.shape[0], freq.size, t_uvw.data_ptr(), t_freq.data_ptr(),
                             t_w.data_ptr(), t_out.data_ptr(), d_vis=t_vis.data_ptr(),
                             d_weights_out=t_wo.data_ptr(), **st)
    np.testing.assert_array_equal(t_out.cpu().numpy().view(np.complex64).reshape(out.shape), out)
    np.testing.assert_array_equal(t_wo.cpu().numpy().reshape(w.shape), w)
    assert sd["gridded_visibility_count"] == s["gridded_visibility_count"] > 0
    np.testing.assert_allclose(sd["total_weight"], s["total_weight"], rtol=1e-12)


def test_cells_exact_on_and_near_cell_edges(oracle_lib):
    """Samples placed on cell edges and within 1e-12 .. 1e-3 of them (wavelength
    1 m, W psx = 2^-6, so u = 64 k metres is an edge) must take the cell the
    host's double arithmetic gives: the FP32 decision defers them to the exact
    pass.  Grid and prepared rows are compared bit for bit."""
    c = 299792458.0
    rng = np.random.default_rng(77)
    k = rng.integers(-100, 100, (4000, 2)).astype(np.float64)
    delta = rng.choice([0.0, 1e-12, -1e-12, 3e-9, -3e-9, 1e-6, -1e-6, 1e-3, -1e-3, 0.37],
                       (4000, 2))
    uvw = np.zeros((4000, 3))
    uvw[:, :2] = 64.0 * k + 64.0 * delta
    uvw[:, 2] = rng.normal(0, 10, 4000)
    freq = np.array([c, c / 3.0, 1.4e9, c * 0.5])
    weights = (rng.integers(0, 9, (4000, freq.size, 2)) / 4.0).astype(np.float32)
    vis = (rng.standard_normal(weights.shape) + 1j * rng.standard_normal(weights.shape)).astype(
        np.complex64)
    args = (UNIFORM, 256, 256, 2.0 ** -14, 2.0 ** -14, False, 1.0, 0.0)
    dev, ref = ImageWeights(*args), oracle_lib.ImageWeights(*args)
    dev.Grid(uvw, freq, weights)
    ref.grid_rows(uvw, freq, weights)
    np.testing.assert_array_equal(dev.half_grid(), ref.grid)
    assert dev.TotalSum() == ref.total
    dev.FinishGridding()
    ref.finish()
    np.testing.assert_array_equal(dev.half_grid(), ref.grid)
    got = prepare_rows(dev, uvw, freq, weights, vis, visibility_weighting=_lib.VISW_UNIT)
    exp = ref.prepare_rows(uvw, freq, weights, vis, None, None, 0, 0.0, 0.0, 2, 0)
    for g, e in zip(got[:3], exp[:3]):
        np.testing.assert_array_equal(g, e)
    assert got[3]["gridded_visibility_count"] == exp[3][3] > 0


@pytest.mark.parametrize("mode,n_pol,nparms", [(0, 1, 2), (1, 1, 4), (2, 1, 4), (3, 2, 2),
                                               (4, 4, 4)])
def test_add_inversion_rows_corrected_matches_oracle(oracle_lib, mode, n_pol, nparms):
    """Raw rows with h5parm gains: weighting, conjugated gains before
    ApplyWeights, collapse and gridding on the device give the image of the
    oracle-prepared rows (gains in FP32 with fused multiply-adds: 1e-5), and
    the correction sum (TRACE: scalar; the other modes: the 4 x 4 matrix of
    AverageCorrection::Add) matches the oracle's to 1e-5."""
    from wsclean_gb300.weights import add_inversion_rows_corrected
    W, Wt, dl, eps = 160, 128, 4e-4, 1e-5
    uvw, freq, vis1 = synthetic.random_points(700, 5, Wt, dl, seed=51, w_scale=2.0)
    rng = np.random.default_rng(52 + mode)
    n_rows, n_chan, n_ant, n_t = uvw.shape[0], freq.size, 7, 3
    vis = (np.repeat(vis1[:, :, None], n_pol, axis=2) *
           (1.0 + 0.2 * rng.standard_normal((n_rows, n_chan, n_pol)))).astype(np.complex64)
    weights = rng.uniform(0.2, 2.0, vis.shape).astype(np.float32)
    sel = rng.random((n_rows, n_chan)) > 0.1
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], axis=1)
    tof = rng.integers(0, n_t, n_rows).astype(np.uint64)
    sol = (1.0 + 0.3 * (rng.standard_normal((n_t, n_chan, n_ant, nparms)) +
                        1j * rng.standard_normal((n_t, n_chan, n_ant, nparms)))).astype(
        np.complex64)
    args = (UNIFORM, Wt, Wt, dl, dl, False, 1.0, 0.0)
    dev, ref = ImageWeights(*args), oracle_lib.ImageWeights(*args)
    dev.Grid(uvw, freq, weights)
    dev.FinishGridding()
    ref.grid[:] = dev.half_grid()
    full = np.zeros((n_t, n_chan, n_ant, 4), np.complex64)
    if nparms == 2:
        full[..., 0], full[..., 3] = sol[..., 0], sol[..., 1]
    else:
        full[:] = sol
    prepared, _, _, sums = ref.prepare_rows(uvw, freq, weights, vis, None, sel, 0, 0.0, 0.0, 0,
                                            _lib.POL_I, gains=(mode, ant, tof, full, 4, n_ant))

    g1 = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps,
                                 num_t=np.float64)
    g1.InitializeInversion()
    acc, corr = add_inversion_rows_corrected(g1, dev, mode, uvw, freq, weights, vis, ant, tof,
                                             sol, nparms, n_t, n_ant, selected=sel,
                                             with_correction_sum=True)
    g1.FinalizeImage(1.0)
    a = g1.RealImage().reshape(W, W)
    g2 = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps,
                                 num_t=np.float64)
    g2.InitializeInversion()
    g2.AddInversionData(n_rows, n_chan, uvw, freq, prepared)
    g2.FinalizeImage(1.0)
    b = g2.RealImage().reshape(W, W)
    d = (W - Wt) // 2
    a, b = a[d:d + Wt, d:d + Wt].astype(np.float64), b[d:d + Wt, d:d + Wt].astype(np.float64)
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    assert acc.gridded_visibility_count == sums[3] > 0
    np.testing.assert_allclose(acc.total_weight, sums[2], rtol=1e-12)
    if mode == 2:
        assert corr > 0
        np.testing.assert_allclose(corr, sums[4], rtol=1e-5)
    else:
        mat = ref.correction_matrix
        assert np.abs(mat).max() > 0
        np.testing.assert_allclose(corr, corr.conj().T, atol=1e-9 * np.abs(mat).max())
        assert np.abs(corr - mat).max() <= 1e-5 * np.abs(mat).max()
    # an antenna index outside the table is reported
    bad = ant.copy()
    bad[3, 0] = n_ant
    g3 = WGriddingGridder_Simple(W, W, Wt, Wt, dl, dl, 0.0, 0.0, 1, epsilon=eps)
    g3.InitializeInversion()
    with pytest.raises(_lib.WgpuError):
        add_inversion_rows_corrected(g3, dev, mode, uvw, freq, weights, vis, bad, tof, sol,
                                     nparms, n_t, n_ant)
