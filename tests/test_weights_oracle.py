"""Imaging weights and raw-row weighting: the oracle (C) against an independent
pure-Python restatement of ImageWeights (structures/imageweights.{h,cpp}) and
MsGridderData::CalculateWeightsImplementation / ApplyWeights / CollapseData
(gridding/msgridderdata.h:36-52, 760-886).  Both add in the reference's serial
order with one rounding per operation, so the comparison is exact except for
the Gaussian taper's long-double factor (checked to 1 ulp)."""
import math

import numpy as np
import pytest

C_LIGHT = 299792458.0
F32 = np.float32

# ---- pure-Python restatement ----------------------------------------------


def py_dims(image_width, image_height, super_weight):
    w = int(math.floor(image_width / super_weight + 0.5))
    h = int(math.floor(image_height / super_weight + 0.5))
    return w + (w % 2), h + (h % 2)


def py_cell(u, v, W, H, psx, psy):
    if v < 0.0:
        u, v = -u, -v
    x = math.floor(u * W * psx + float(W // 2))
    y = math.floor(v * H * psy)
    if 0 <= x < W and 0 <= y < H // 2:
        return int(y), int(x)
    return None


def py_uv(x, y, W, H, psx, psy):
    return float(x - W // 2) / (W * psx), float(y) / (H * psy)


def py_grid(grid, W, H, psx, psy, as_taper, uvw, freq, weights):
    total = 0.0
    for r in range(uvw.shape[0]):
        um, vm = float(uvw[r, 0]), float(uvw[r, 1])
        if vm < 0.0:
            um, vm = -um, -vm
        for ch in range(freq.size):
            lam = C_LIGHT / float(freq[ch])
            for p in range(weights.shape[2]):
                w = F32(weights[r, ch, p])
                if as_taper and w != 0:
                    w = F32(1.0)
                c = py_cell(um / lam, vm / lam, W, H, psx, psy)
                if c is not None:
                    grid[c] += float(w)
                    total += float(w)
    return total


def py_finish(grid, mode, robustness, total):
    flat = grid.reshape(-1)
    if mode == 2:
        avg = 0.0
        for val in flat:
            avg += float(val) * float(val)
        avg /= total
        ns = 5.0 * math.exp(-math.log(10.0) * robustness)
        ssq = ns * ns / avg
        for i, val in enumerate(flat):
            if val != 0.0:
                flat[i] = 1.0 / (1.0 + float(val) * ssq)
    elif mode == 1:
        for i, val in enumerate(flat):
            flat[i] = 1.0 / float(val) if val != 0.0 else 0.0
    else:
        for i, val in enumerate(flat):
            if val != 0.0:
                flat[i] = 1.0


def py_tukey(x, n):
    return 0.5 * (1.0 + math.cos((math.pi / n) * (x - n)))


def py_taper(grid, W, H, psx, psy, kind, a, b):
    Hh = H // 2
    if kind == 7:
        src = grid.copy()
        d = int(b) // 2
        for y in range(Hh):
            for x in range(W):
                w = float(src[y, x])
                if w == 0.0:
                    continue
                x1, y1 = max(x - d, 0), max(y - d, 0)
                x2, y2 = min(x + d, W), min(y + d, Hh)
                cnt, s = 0, 0.0
                for yi in range(y1, y2):
                    for xi in range(x1, x2):
                        if src[yi, xi] != 0.0:
                            cnt += 1
                            s += float(src[yi, xi])
                mean = s / cnt if cnt else float("nan")
                if w > mean * a:
                    grid[y, x] = mean * a
        return
    if kind == 6:
        hp = 1.0 / (a * 2.0 * math.pi)
        s2hp = np.longdouble(2) * np.sqrt(np.longdouble(2) * np.log(np.longdouble(2)))
        m = float(np.longdouble(hp) * s2hp)
        m *= -2.0 * m
    max_u, max_v = py_uv(W, Hh, W, H, psx, psy)
    for y in range(Hh):
        for x in range(W):
            u, v = py_uv(x, y, W, H, psx, psy)
            d2 = u * u + v * v
            g = float(grid[y, x])
            if kind == 0 and d2 < a * a:
                g = 0.0
            elif kind == 1 and d2 > a * a:
                g = 0.0
            elif kind == 2:
                if d2 > b * b:
                    g = 0.0
                elif d2 > (b - a) * (b - a):
                    g *= py_tukey(b - math.sqrt(d2), a)
            elif kind == 3:
                if d2 < b * b:
                    g = 0.0
                elif d2 < (b + a) * (b + a):
                    g *= py_tukey(math.sqrt(d2) - b, a)
            elif kind == 4:
                if max_u - abs(u) < a or max_v - abs(v) < a:
                    g = 0.0
            elif kind == 5:
                ud, vd = max_u - abs(u), max_v - abs(v)
                if ud < b or vd < b:
                    g = 0.0
                elif ud < a + b or vd < a + b:
                    ru, rv = min(ud - b, a), min(vd - b, a)
                    g *= py_tukey(ru, a) * py_tukey(rv, a)
            elif kind == 6 and g != 0.0:
                g = g * math.exp(d2 / m)
            grid[y, x] = g


def py_collapse4(c, pol):
    xx, xy, yx, yy = c
    h = F32(0.5)
    if pol == 0:
        return (F32(xx[0] + yy[0]) * h, F32(xx[1] + yy[1]) * h)
    if pol == 1:
        return (h * F32(xx[0] - yy[0]), h * F32(xx[1] - yy[1]))
    if pol == 2:
        return (F32(xy[0] + yx[0]) * h, F32(xy[1] + yx[1]) * h)
    if pol == 3:
        d = (F32(yx[0] - xy[0]), F32(yx[1] - xy[1]))
        return (F32(-0.5) * d[1], h * d[0])
    return c[pol - 4]


def py_prepare(grid, W, H, psx, psy, uvw, freq, weights, vis, model, selected, psf_mode,
               dl, dm, visw, pol):
    n_rows, n_chan, n_pol = weights.shape
    out = np.zeros((n_rows, n_chan), np.complex64)
    w_out = np.zeros(weights.shape, np.float32)
    iw_out = np.zeros((n_rows, n_chan), np.float32)
    sums = [0.0, 0.0, 0.0, 0.0]
    for r in range(n_rows):
        u_m, v_m, w_m = (float(t) for t in uvw[r])
        if psf_mode and (dl != 0.0 or dm != 0.0):
            dn = math.sqrt(1.0 - dl * dl - dm * dm) - 1.0
            shift = 2.0 * math.pi * (u_m * dl + v_m * dm + w_m * dn)
        for ch in range(n_chan):
            lam = C_LIGHT / float(freq[ch])
            c = py_cell(u_m / lam, v_m / lam, W, H, psx, psy)
            iw = F32(grid[c]) if c is not None else F32(0.0)
            iw_out[r, ch] = iw
            corr = []
            for p in range(n_pol):
                if psf_mode:
                    if dl != 0.0 or dm != 0.0:
                        rad = shift / lam
                        re, im = F32(math.cos(rad)), F32(math.sin(rad))
                    else:
                        re, im = F32(1.0), F32(0.0)
                else:
                    re, im = F32(vis[r, ch, p].real), F32(vis[r, ch, p].imag)
                if model is not None:
                    re, im = F32(re - F32(model[r, ch, p].real)), F32(im - F32(model[r, ch, p].imag))
                w = F32(weights[r, ch, p])
                if selected is not None and not selected[r, ch]:
                    w = F32(0.0)
                if visw == 1:
                    w = F32(w * w)
                elif visw == 2 and w != 0:
                    w = F32(1.0)
                cum = F32(w * iw)
                has = cum != 0
                if p == 0:
                    sums[0] += float(w) if has else 0.0
                    sums[1] = max(sums[1], float(cum))
                    sums[3] += 1.0 if has else 0.0
                sums[2] += float(cum)
                w_out[r, ch, p] = cum
                corr.append((F32(re * cum), F32(im * cum)))
            if n_pol == 1:
                v = corr[0]
            elif n_pol == 2:
                v = (F32(corr[0][0] + corr[1][0]), F32(corr[0][1] + corr[1][1]))
            else:
                v = py_collapse4(corr, pol)
            out[r, ch] = complex(v[0], v[1])
    return out, w_out, iw_out, np.array(sums)


# ---- synthetic rows ----------------------------------------------------------


def rows(seed, n_rows=40, n_pol=4, extent=170.0):
    rng = np.random.default_rng(seed)
    uvw = rng.uniform(-extent, extent, (n_rows, 3))
    uvw[:4, :2] = [[3.0, 1.0], [-3.0, -1.0], [0.0, 0.0], [1.5, -0.0]]  # mirrored pair, centre
    freq = np.array([1.0e8, 1.13e8, 1.27e8])
    weights = (rng.integers(0, 9, (n_rows, freq.size, n_pol)) / 4.0).astype(np.float32)
    vis = (rng.standard_normal((n_rows, freq.size, n_pol)) +
           1j * rng.standard_normal((n_rows, freq.size, n_pol))).astype(np.complex64)
    return uvw, freq, weights, vis


PSX = 0.011  # radians per pixel: the uv half-width is 1 / (2 * PSX) ~ 45 wavelengths


def oracle_weights(oracle_lib, mode, robust=0.0, as_taper=False, seed=3, size=(40, 28)):
    iw = oracle_lib.ImageWeights(mode, size[0], size[1], PSX, PSX * 1.3, as_taper, 1.0, robust)
    uvw, freq, weights, _ = rows(seed)
    iw.grid_rows(uvw, freq, weights)
    return iw, (uvw, freq, weights)


@pytest.mark.parametrize("mode,robust,as_taper", [(0, 0.0, False), (1, 0.0, False),
                                                   (1, 0.0, True), (2, 0.5, False),
                                                   (2, -1.0, False)])
def test_weight_grid_and_finish_match_restatement(oracle_lib, mode, robust, as_taper):
    iw, (uvw, freq, weights) = oracle_weights(oracle_lib, mode, robust, as_taper)
    W, H = iw.width, iw.height
    grid = np.zeros((H // 2, W))
    total = py_grid(grid, W, H, iw.psx, iw.psy, as_taper, uvw, freq, weights)
    np.testing.assert_array_equal(iw.grid, grid)
    assert iw.total == total and total > 0
    assert np.count_nonzero(grid) > 10
    iw.finish()
    py_finish(grid, mode, robust, total)
    np.testing.assert_array_equal(iw.grid, grid)


def test_weight_dims_follow_super_weight(oracle_lib):
    for args in ((40, 28, 1.0), (41, 27, 1.0), (100, 60, 3.0), (64, 64, 2.5)):
        iw = oracle_lib.ImageWeights(1, args[0], args[1], PSX, PSX, False, args[2])
        assert (iw.width, iw.height) == py_dims(*args)
        assert iw.width % 2 == 0 and iw.height % 2 == 0


TAPERS = [(0, 12.0, 0.0), (1, 30.0, 0.0), (2, 8.0, 30.0), (3, 6.0, 10.0), (4, 5.0, 0.0),
          (5, 4.0, 3.0), (6, 0.05, 0.0), (7, 1.2, 4.0), (7, 0.9, 7.0), (7, 2.0, 1.0)]


@pytest.mark.parametrize("kind,a,b", TAPERS)
def test_weight_tapers_match_restatement(oracle_lib, kind, a, b):
    iw, _ = oracle_weights(oracle_lib, 1)
    iw.finish()
    grid = iw.grid.copy()
    iw.taper(kind, a, b)
    py_taper(grid, iw.width, iw.height, iw.psx, iw.psy, kind, a, b)
    if kind == 6:
        np.testing.assert_allclose(iw.grid, grid, rtol=4e-16, atol=0)
    else:
        np.testing.assert_array_equal(iw.grid, grid)
    if kind in (0, 1, 4):
        assert np.count_nonzero(iw.grid) < np.count_nonzero(oracle_weights(oracle_lib, 1)[0].grid)


def test_weight_mirror_and_sample_match_restatement(oracle_lib):
    iw, _ = oracle_weights(oracle_lib, 1)
    iw.finish()
    W, H = iw.width, iw.height
    img = iw.mirrored()
    for y in range(H // 2):
        for x in range(W):
            assert img[H // 2 + y, x] == iw.grid[y, x]
            assert img[H // 2 - 1 - y, W - 1 - x] == iw.grid[y, x]
    rng = np.random.default_rng(5)
    u = rng.uniform(-60, 60, 500)
    v = rng.uniform(-50, 50, 500)
    got = iw.sample(u, v)
    for k in range(u.size):
        c = py_cell(u[k], v[k], W, H, iw.psx, iw.psy)
        assert got[k] == (iw.grid[c] if c is not None else 0.0)
    assert np.count_nonzero(got) > 5


PREP_CASES = [
    dict(n_pol=1, psf_mode=0, visw=0, model=False, sel=False, pol=0),
    dict(n_pol=2, psf_mode=0, visw=1, model=False, sel=True, pol=0),
    dict(n_pol=4, psf_mode=0, visw=2, model=True, sel=True, pol=0),
    dict(n_pol=4, psf_mode=0, visw=0, model=False, sel=False, pol=1),
    dict(n_pol=4, psf_mode=0, visw=0, model=True, sel=False, pol=3),
    dict(n_pol=4, psf_mode=0, visw=1, model=False, sel=True, pol=5),
    dict(n_pol=2, psf_mode=1, visw=0, model=False, sel=True, pol=0, dl=0.013, dm=-0.021),
    dict(n_pol=1, psf_mode=2, visw=2, model=False, sel=False, pol=0),
]


@pytest.mark.parametrize("case", PREP_CASES)
def test_prepare_rows_match_restatement(oracle_lib, case):
    iw, _ = oracle_weights(oracle_lib, 2, 0.0)
    iw.finish()
    uvw, freq, weights, vis = rows(11, n_rows=30, n_pol=case["n_pol"])
    rng = np.random.default_rng(12)
    model = (rng.standard_normal(vis.shape) + 1j * rng.standard_normal(vis.shape)).astype(
        np.complex64) if case["model"] else None
    sel = rng.random((uvw.shape[0], freq.size)) > 0.3 if case["sel"] else None
    dl, dm = case.get("dl", 0.0), case.get("dm", 0.0)
    got = iw.prepare_rows(uvw, freq, weights, None if case["psf_mode"] else vis, model, sel,
                          case["psf_mode"], dl, dm, case["visw"], case["pol"])
    exp = py_prepare(iw.grid, iw.width, iw.height, iw.psx, iw.psy, uvw, freq, weights, vis,
                     model, sel, case["psf_mode"], dl, dm, case["visw"], case["pol"])
    for g, e in zip(got[:3], exp[:3]):
        np.testing.assert_array_equal(g, e)
    np.testing.assert_array_equal(got[3], exp[3])
    assert exp[3][3] > 0 and np.count_nonzero(got[0]) > 0


@pytest.mark.parametrize("mode,n_pol,pol", [(0, 1, 0), (1, 1, 0), (2, 1, 0), (3, 2, 0), (4, 4, 0),
                                            (4, 4, 3)])
def test_prepare_rows_corrected_composition(oracle_lib, mode, n_pol, pol):
    """Gains applied between weighting and ApplyWeights: identity gains leave
    the rows as they are; a real gain of 2 on both antennas (conj(2) V 2 = 4 V,
    exact in float) scales every prepared value by exactly 4, and the TRACE
    correction sum is |(2*2 + 2*2) / 2|^2 = 16 times the sum of w[0] * iw."""
    iw, _ = oracle_weights(oracle_lib, 1)
    iw.finish()
    uvw, freq, weights, vis = rows(21, n_rows=25, n_pol=n_pol)
    n_rows, n_chan, n_ant = uvw.shape[0], freq.size, 5
    ant = np.stack([np.arange(n_rows) % n_ant, (np.arange(n_rows) + 2) % n_ant], axis=1)
    tof = np.zeros(n_rows, np.uint64)
    base = iw.prepare_rows(uvw, freq, weights, vis, None, None, 0, 0.0, 0.0, 0, pol)
    for value, factor in ((1.0, 1.0), (2.0, 4.0)):
        sol = np.zeros((1, n_chan, n_ant, 4), np.complex64)
        sol[..., 0] = value
        sol[..., 3] = value
        got = iw.prepare_rows(uvw, freq, weights, vis, None, None, 0, 0.0, 0.0, 0, pol,
                              gains=(mode, ant, tof, sol, 4, n_ant))
        np.testing.assert_array_equal(got[0], base[0] * np.float32(factor))
        np.testing.assert_array_equal(got[1], base[1])
        np.testing.assert_array_equal(got[3][:4], base[3])
        if mode == 2:
            w0 = base[1][:, :, 0].astype(np.float64)  # w[0] * iw
            np.testing.assert_allclose(got[3][4], factor * factor * w0.sum(), rtol=1e-12)
