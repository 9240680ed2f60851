"""C-ABI and host-side logic on the CPU: exported symbols, planner invariants,
argument validation and the loud failure without a CUDA device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from wsclean_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not hdr.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", hdr)).read()
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(wgpu_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(wgpu_lib):
    declared = _declared_functions()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(wgpu_lib, name), name
    assert set(declared) == set(_lib.exported_symbols())


def _plan(**kw):
    base = dict(width=1024, height=1024, dl=4.848e-5, dm=4.848e-5, epsilon=1e-4,
                w_min=-1500.0, w_max=1800.0, n_vis=2_000_000)
    base.update(kw)
    return _lib.make_plan(**base)


def _smooth(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


@pytest.mark.parametrize("eps", [1e-3, 1e-4, 1e-5])
@pytest.mark.parametrize("npix", [256, 1024, 8192])
def test_planner_invariants(wgpu_lib, eps, npix):
    p = _plan(epsilon=eps, width=npix, height=npix, dl=3 * 4.848e-6, dm=3 * 4.848e-6)
    assert p.nu % p.tile == 0 and p.nv % p.tile == 0
    assert _smooth(p.nu) and _smooth(p.nv)
    assert p.nu >= 1.1 * npix and p.nu <= 2.0 * npix * 1.1
    assert p.support <= p.tile and 4 <= p.support <= 16
    assert p.est_error <= eps
    assert p.fft_n1 * p.fft_n2 == p.nv and p.fft_n2 <= 256
    # every sample's w footprint lies inside the planes
    if p.n_planes > 1:
        assert p.w0 + (p.support / 2) * p.dw <= -1500.0 + 1e-6
        last = p.w0 + (p.n_planes - 1) * p.dw
        assert last - (p.support / 2 - 1) * p.dw >= 1800.0 - 1e-6
        # w sampling: dw * half-range of n-1 <= 1 / (2 sigma)
        assert p.dw * 0.5 * (p.nm1_max - p.nm1_min) <= 0.5 / p.sigma + 1e-12


def test_planner_single_plane_when_w_is_flat(wgpu_lib):
    p = _plan(w_min=0.0, w_max=0.0)
    assert p.n_planes == 1


def test_planner_rejects_bad_requests(wgpu_lib):
    with pytest.raises(_lib.WgpuError) as e:
        _plan(width=1023)
    assert e.value.status == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError):
        _plan(epsilon=-1.0)
    with pytest.raises(_lib.WgpuError):
        _plan(w_min=5.0, w_max=1.0)


def test_planner_prefers_cheaper_plans_for_more_visibilities(wgpu_lib):
    few = _plan(n_vis=1000, epsilon=1e-5)
    many = _plan(n_vis=10**10, epsilon=1e-5)
    # more visibilities -> gridding dominates -> smaller kernel support
    assert many.support <= few.support


def test_create_validates_arguments_before_touching_a_device(wgpu_lib):
    h = C.c_void_p()
    st = wgpu_lib.wgpu_gridder_create(64, 64, 64, 64, 1e-3, 1e-3, 0, 0, 1, 1e-4, 3, 0, 4,
                                      C.byref(h))
    assert st == _lib.WGPU_ERR_INVALID
    assert b"verbosity" in wgpu_lib.wgpu_last_error()
    st = wgpu_lib.wgpu_gridder_create(64, 64, 66, 64, 1e-3, 1e-3, 0, 0, 1, 1e-4, 0, 0, 4,
                                      C.byref(h))
    assert st == _lib.WGPU_ERR_INVALID
    st = wgpu_lib.wgpu_gridder_create(64, 64, 64, 64, 1e-3, 1e-3, 0, 0, 1, 1e-4, 0, 0, 2,
                                      C.byref(h))
    assert st == _lib.WGPU_ERR_INVALID


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a CUDA device")
def test_no_device_fails_loudly(wgpu_lib):
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    with pytest.raises(_lib.WgpuError) as e:
        WGriddingGridder_Simple(64, 64, 64, 64, 1e-3, 1e-3, 0, 0, 1)
    assert e.value.status == _lib.WGPU_ERR_CUDA
    p = _plan(width=64, height=64, dl=1e-3, dm=1e-3)
    uvw = np.zeros((1, 3))
    with pytest.raises(_lib.WgpuError):
        from wsclean_gb300.gridder import bucket_debug
        bucket_debug(p, 1, 1, uvw, np.array([1e8]), np.ones(1, np.complex64), True)
    from wsclean_gb300.server import GriddingServer
    with pytest.raises(_lib.WgpuError) as e:
        GriddingServer(1e9, max_active=2)
    assert e.value.status == _lib.WGPU_ERR_CUDA


def test_server_validates_arguments(wgpu_lib):
    from wsclean_gb300.server import GriddingServer
    for args in ((0.0, 2), (1e9, 0), (1e9, 65), (-1.0, 1)):
        with pytest.raises(_lib.WgpuError) as e:
            GriddingServer(*args)
        assert e.value.status == _lib.WGPU_ERR_INVALID


def test_constant_memory_formula_matches_reference():
    # gridder_simple_implementation.h:53-61: sigma_max^2 * w_t * h_t * 8 + w_t * h_t * sizeof(NumT)
    w_t, h_t = 1000, 800
    assert int(4.0 * w_t * h_t * 8) + w_t * h_t * 4 == 4 * 8 * 800_000 + 3_200_000


def test_weighting_and_resampling_validate_then_need_a_device(wgpu_lib):
    """Imaging weights, row preparation and resampling check their arguments
    first (WGPU_ERR_INVALID) and fail loudly without a device (WGPU_ERR_CUDA):
    there is no CPU fallback."""
    import ctypes as C
    from wsclean_gb300 import resample as wres
    from wsclean_gb300.weights import ImageWeights
    L = _lib.lib()
    out = C.c_void_p()
    for args in ((5, 0.0, 64, 64, 1e-3, 1e-3, 0, 1.0),    # weighting mode
                 (1, 0.0, 64, 64, 0.0, 1e-3, 0, 1.0),    # pixel scale
                 (1, 0.0, 64, 64, 1e-3, 1e-3, 0, 0.0),   # super weight
                 (1, 0.0, 0, 64, 1e-3, 1e-3, 0, 1.0)):   # empty grid (odd sizes round up)
        assert L.wgpu_imageweights_create(*args, C.byref(out)) == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError) as e:
        ImageWeights(1, 64, 64, 1e-3, 1e-3)
    assert e.value.status == _lib.WGPU_ERR_CUDA
    rw = _lib.RowWeighting(0, 0.0, 0.0, 0, 0, 0)
    sums = _lib.WeightSums()
    assert L.wgpu_prepare_rows(None, C.byref(rw), 1, 1, 1, None, None, None, None, None, None,
                               None, None, None, C.byref(sums)) == _lib.WGPU_ERR_INVALID
    assert L.wgpu_gridder_add_inversion_rows(None, None, C.byref(rw), 1, 1, 1, None, None, None,
                                             None, None, None, None) == _lib.WGPU_ERR_INVALID
    img = np.zeros((8, 8), np.float32)
    with pytest.raises(_lib.WgpuError) as e:
        wres.resample(img, 0, 8)
    assert e.value.status == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError) as e:
        wres.resample(img, 16, 16)
    assert e.value.status == _lib.WGPU_ERR_CUDA
    with pytest.raises(_lib.WgpuError) as e:
        wres.calculate_fft_size(100, 0.0, 1e-3)
    assert e.value.status == _lib.WGPU_ERR_INVALID
    assert L.wgpu_facets_invert_corrected(None, 4, 4, None, None, None, None, 4, 1, 1, 0,
                                          None) == _lib.WGPU_ERR_INVALID
    assert L.wgpu_gridder_finish_inversion(None, 8, 8, 8, 8, None) == _lib.WGPU_ERR_INVALID


def test_sizing_functions_run_without_a_device(wgpu_lib):
    """CalculateFFTSize, the small-inversion size and the gridder's trimmed
    size are host functions."""
    from wsclean_gb300 import resample as wres
    assert wres.calculate_fft_size(1000, 1e-4, 1e-3) == (200, 200)
    mn, opt = wres.calculate_fft_size(1000, 1e-4, 0.9e-3)
    assert mn == 223 and opt % 4 == 0 and opt >= mn
    assert wres.actual_trimmed_size(1000, 600, 1.2) == (836, 500)
    w, h, px, py = wres.small_inversion_size(1000, 1000, 1e-4, 1e-4, 1e-3)
    assert (w, h) == (200, 200) and abs(px - 5e-4) < 1e-15


def test_gain_mode_visibility_counts(wgpu_lib):
    """GetNVisibilities, gridding/gainmode.h:33-46."""
    assert [_lib.gain_mode_n_visibilities(m) for m in range(5)] == [1, 1, 1, 2, 4]
    assert _lib.gain_mode_n_visibilities(5) == 0
    assert _lib.gain_mode_n_visibilities(-1) == 0


def test_select_gain_mode_every_combination(wgpu_lib):
    """SelectGainMode, gridding/gainmode.h:52-95, over every polarisation the
    library names and stored-polarisation counts 0..5: the accepted pairs and
    their modes, everything else rejected."""
    P = _lib
    stokes = {P.POL_I, P.POL_Q, P.POL_U, P.POL_V}
    all_pols = list(range(15))
    expected = {}
    for pol in all_pols:
        # one stored polarisation: XX, YY, or the trace for anything else
        expected[(pol, 1)] = (P.GAIN_XX if pol == P.POL_XX else
                              P.GAIN_YY if pol == P.POL_YY else P.GAIN_TRACE)
        if pol in (P.POL_I, P.POL_DIAGONAL_INSTRUMENTAL, P.POL_XX, P.POL_YY):
            expected[(pol, 2)] = P.GAIN_2VIS_DIAGONAL
        if pol in stokes | {P.POL_FULL_STOKES, P.POL_INSTRUMENTAL, P.POL_XX, P.POL_YY}:
            expected[(pol, 4)] = P.GAIN_FULL
    for pol in all_pols:
        for n in range(6):
            if (pol, n) in expected:
                assert P.select_gain_mode(pol, n) == expected[(pol, n)], (pol, n)
            else:
                with pytest.raises(P.WgpuError):
                    P.select_gain_mode(pol, n)
    with pytest.raises(P.WgpuError):
        P.select_gain_mode(15, 1)
