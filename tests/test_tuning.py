"""The `tuning` flag: candidate plans timed on the call's own samples.

The reference's flag selects ducc0's ms2dirty_tuning / dirty2ms_tuning
(wgridder/gridder_simple.h:216-225, gridder_simple_implementation.h:185-194).
Here it makes the plan a measured choice among the entries that meet epsilon;
whatever is chosen, results must stay within epsilon of the FP64 direct FT.
"""
import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple

C = 299792458.0


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def _request(eps, w_range=(-300.0, 300.0), **kw):
    return dict(width=512, height=512, dl=2e-4, dm=2e-4, epsilon=eps, w_min=w_range[0],
                w_max=w_range[1], n_vis=10_000_000, **kw)


@pytest.mark.parametrize("eps", [1e-2, 1e-4, 1e-5])
def test_candidates_meet_epsilon_in_cost_order(wgpu_lib, eps):
    req = _request(eps)
    cands = _lib.plan_candidates(**req)
    first = _lib.make_plan(**req)
    assert len(cands) >= 2
    assert cands[0].as_dict() == first.as_dict()
    est = [c.est_seconds for c in cands]
    assert est == sorted(est)
    assert all(c.est_error <= eps for c in cands)
    keys = {(c.support, round(c.sigma, 6)) for c in cands}
    assert len(keys) == len(cands)
    for c in cands:
        assert c.nu % c.tile == 0 and c.nv % c.tile == 0
        assert c.nv == c.fft_n1 * c.fft_n2 and 1 <= c.plane_batch <= c.n_planes
    assert len(_lib.plan_candidates(max_plans=2, **req)) == 2


def test_candidates_without_any_plan_meeting_epsilon(wgpu_lib):
    # nothing reaches 1e-12: the single candidate is the most accurate entry,
    # as make_plan falls back to it
    req = _request(1e-12)
    cands = _lib.plan_candidates(**req)
    assert len(cands) == 1
    assert cands[0].as_dict() == _lib.make_plan(**req).as_dict()


def test_candidates_reject_invalid_requests(wgpu_lib):
    with pytest.raises(_lib.WgpuError):
        _lib.plan_candidates(**_request(0.0))
    with pytest.raises(_lib.WgpuError):
        _lib.plan_candidates(**_request(1e-4, w_range=(5.0, -5.0)))


def _case(seed, W=256, dl=3e-4, rows=2500, chan=8):
    uvw, freq, vis = synthetic.random_points(rows, chan, W, dl, seed=seed, w_scale=2.0)
    return W, dl, uvw, freq, vis


@pytest.mark.gpu
def test_tuned_inversion_times_candidates_and_remembers_the_choice(wgpu_lib, oracle_lib):
    _lib.tuning_cache_clear()
    W, dl, uvw, freq, vis = _case(61)
    eps = 1e-4
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps, tuning=True)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    img = g.RealImage().astype(np.float64)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl)
    assert rel(img, ref) <= eps
    trials = g.last_tuning()
    assert len(trials) >= 2
    chosen = [t for t in trials if t["chosen"]]
    assert len(chosen) == 1
    assert chosen[0]["measured_ms"] == min(t["measured_ms"] for t in trials)
    assert all(t["measured_ms"] > 0 for t in trials)
    plan = g.last_plan()
    assert (plan.support, plan.sigma) == (chosen[0]["support"], chosen[0]["sigma"])
    assert "tune" in g.last_timings()
    # a new gridder of the same shape (as WSClean makes per major cycle) takes
    # the remembered choice without timing
    g2 = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps, tuning=True)
    g2.InitializeInversion()
    g2.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    assert g2.last_tuning() == []
    p2 = g2.last_plan()
    assert (p2.support, p2.sigma) == (plan.support, plan.sigma)
    assert rel(g2.RealImage(), img) <= 2e-6
    # forgetting the choices times again
    _lib.tuning_cache_clear()
    g2.InitializeInversion()
    g2.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    assert len(g2.last_tuning()) >= 2


@pytest.mark.gpu
def test_tuned_prediction_within_epsilon(wgpu_lib, oracle_lib):
    _lib.tuning_cache_clear()
    W, dl, uvw, freq, _ = _case(62)
    eps = 1e-5
    rng = np.random.default_rng(3)
    model = np.zeros(W * W, np.float32)
    model[rng.choice(W * W, 30, replace=False)] = rng.uniform(-1, 1, 30)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps, tuning=True)
    g.InitializePrediction(model)
    pv = g.PredictVisibilities(uvw.shape[0], freq.size, uvw, freq)
    ref = oracle_lib.dft_predict(uvw, freq, model, W, W, dl, dl)
    assert rel(pv.ravel(), ref.ravel()) <= eps
    trials = g.last_tuning()
    assert len(trials) >= 2 and sum(t["chosen"] for t in trials) == 1


@pytest.mark.gpu
def test_tuned_bound_set_times_both_directions(wgpu_lib, oracle_lib):
    _lib.tuning_cache_clear()
    W, dl, uvw, freq, vis = _case(63, rows=1500)
    eps = 1e-4
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=eps, tuning=True)
    g.Bind(uvw.shape[0], freq.size, uvw, freq)
    trials = g.last_tuning()
    assert len(trials) >= 2 and sum(t["chosen"] for t in trials) == 1
    g.InitializeInversion()
    g.InvertBound(vis)
    ref = oracle_lib.dft_invert(uvw, freq, vis, W, W, dl, dl)
    assert rel(g.RealImage(), ref) <= eps


@pytest.mark.gpu
def test_pinned_plan_is_not_tuned(wgpu_lib):
    W, dl, uvw, freq, vis = _case(64, rows=800)
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, 1, epsilon=1e-4, tuning=True)
    wl = uvw[:, 2:3] * (freq / C)[None, :]
    p = _lib.make_plan(width=W, height=W, dl=dl, dm=dl, epsilon=1e-4, w_min=float(wl.min()),
                       w_max=float(wl.max()), n_vis=int(wl.size), force_support=6)
    g.pin_plan(p)
    g.InitializeInversion()
    g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, vis)
    assert g.last_tuning() == []
    assert g.last_plan().support == 6


def test_fallback_plan_fits_the_row_transform(wgpu_lib):
    """When no entry meets epsilon the plan is the most accurate one whose grid
    the transforms take: at 8192 pixels sigma = 2 would need 16384-point rows,
    above the 12288 the row transform holds, so the fallback keeps sigma <= 1.5
    rather than failing."""
    req = dict(width=8192, height=8192, dl=1.4544e-5, dm=1.4544e-5, epsilon=1e-7,
               w_min=-9000.0, w_max=9000.0, n_vis=473_000_000)
    p = _lib.make_plan(**req)
    assert p.nu <= 12288 and p.nv <= 12288
    assert p.est_error > 1e-7  # the best available, reported honestly
    tighter = [c for c in _lib.plan_candidates(**dict(req, epsilon=1e-5))]
    assert p.est_error <= min(c.est_error for c in tighter)
