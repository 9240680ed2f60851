"""Request server (continuous batching) through the C ABI.

The reference's scheduler tests (tests/scheduling/tthreadedscheduler.cpp) check
that tasks run and that results reach their callers; here, in addition, every
result of a mixed concurrent stream must equal the same request run alone.
Tolerance: 1e-6 relative L2 between the two runs (the inversion accumulates with
float atomics, whose order differs between runs), and each result within its
epsilon of the FP64 direct FT.
"""
import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple
from wsclean_gb300.server import GriddingServer

pytestmark = pytest.mark.gpu

SAME = 1e-6
PLANES = 2e9  # the same plane budget (hence the same plans) in every server


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def _stream():
    """Mixed request set: sizes 96-256 pixels, epsilon 1e-4 / 1e-5, inversions
    and predictions, one-off requests and two sessions with several cycles."""
    reqs = []
    rng = np.random.default_rng(77)
    specs = [(96, 1e-3, 1e-4, 300, 3), (128, 4e-4, 1e-5, 700, 4), (256, 2e-4, 1e-4, 1500, 6),
             (192, 3e-4, 1e-5, 900, 5), (160, 5e-4, 1e-4, 400, 2), (224, 2.5e-4, 1e-5, 1100, 4)]
    for i, (W, dl, eps, rows, chan) in enumerate(specs):
        uvw, freq, vis = synthetic.random_points(rows, chan, W, dl, seed=100 + i, w_scale=2.0)
        geom = dict(width=W, height=W, dl=dl, dm=dl, epsilon=eps,
                    l_shift=0.001 * (i % 3), m_shift=-0.0005 * (i % 2))
        model = np.zeros(W * W, np.float32)
        model[rng.choice(W * W, 12, replace=False)] = rng.uniform(-1, 1, 12)
        session = 0 if i < 4 else 1000 + i
        kinds = ["invert", "predict"] if session == 0 else ["invert", "predict", "invert",
                                                              "predict"]
        for k in kinds:
            reqs.append(dict(kind=k, geom=geom, uvw=uvw, freq=freq, vis=vis, model=model,
                             session=session))
    return reqs


def _submit(srv, r):
    if r["kind"] == "invert":
        return srv.submit_invert(r["geom"], r["uvw"], r["freq"], r["vis"], 1.0,
                                 session=r["session"])
    return srv.submit_predict(r["geom"], r["uvw"], r["freq"], r["model"], session=r["session"])


def _run_alone(reqs):
    out = []
    with GriddingServer(8e9, max_active=1, plane_budget_bytes=PLANES) as srv:
        for r in reqs:
            out.append(srv.wait(_submit(srv, r)).copy())
    return out


def test_results_same_alone_and_in_mix(wgpu_lib, oracle_lib):
    reqs = _stream()
    alone = _run_alone(reqs)
    with GriddingServer(16e9, max_active=4, plane_budget_bytes=PLANES) as srv:
        tickets = [_submit(srv, r) for r in reqs]
        mixed = [srv.wait(t).copy() for t in tickets]
        stats = srv.stats()
        lat = [t.latency_ms for t in tickets]
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["peak_running"] >= 2  # requests overlapped on the device
    assert all(x > 0 for x in lat)
    for i, (r, a, m) in enumerate(zip(reqs, alone, mixed)):
        assert rel(m, a) <= SAME, (i, r["kind"])
    # each result against the FP64 direct FT
    for r, a in zip(reqs, alone):
        g = r["geom"]
        W, dl = g["width"], g["dl"]
        if r["kind"] == "invert":
            ref = oracle_lib.dft_invert(r["uvw"], r["freq"], r["vis"], W, W, dl, dl,
                                        g["l_shift"], g["m_shift"])
        else:
            ref = oracle_lib.dft_predict(r["uvw"], r["freq"], r["model"], W, W, dl, dl,
                                         g["l_shift"], g["m_shift"]).reshape(-1)
        assert rel(a, ref) <= g["epsilon"], r["kind"]


def test_session_matches_plain_gridder(wgpu_lib):
    W, dl, eps = 160, 4e-4, 1e-5
    uvw, freq, vis1 = synthetic.random_points(800, 4, W, dl, seed=61, w_scale=2.0)
    _, _, vis2 = synthetic.random_points(800, 4, W, dl, seed=62, w_scale=2.0)
    geom = dict(width=W, height=W, dl=dl, dm=dl, epsilon=eps)
    with GriddingServer(8e9, max_active=2) as srv:
        imgs = [srv.wait(srv.submit_invert(geom, uvw, freq, v, 0.5, session=7))
                for v in (vis1, vis2, vis1)]
        held = srv.stats()["device_bytes_in_use"]
        assert held > 0  # the session stays resident between cycles
        srv.close_session(7)
        assert srv.stats()["device_bytes_in_use"] == pytest.approx(0.0, abs=1.0)
    for v, img in zip((vis1, vis2, vis1), imgs):
        g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0, 0, 1, epsilon=eps, num_t=np.float64)
        g.InitializeInversion()
        g.AddInversionData(uvw.shape[0], freq.size, uvw, freq, v)
        g.FinalizeImage(0.5)
        assert rel(img, g.RealImage()) <= eps
        g.close()
    assert rel(imgs[0], imgs[2]) <= SAME


def test_admission_by_device_memory(wgpu_lib):
    """A budget smaller than any request admits one request at a time; all
    still complete with the same results."""
    reqs = [r for r in _stream() if r["session"] == 0]
    with GriddingServer(1.0, max_active=4, plane_budget_bytes=PLANES) as srv:
        tickets = [_submit(srv, r) for r in reqs]
        out = [srv.wait(t).copy() for t in tickets]
        stats = srv.stats()
    assert stats["peak_running"] == 1
    assert stats["held_for_memory"] >= 1  # later requests waited for the budget
    alone = _run_alone(reqs)
    for a, b in zip(out, alone):
        assert rel(a, b) <= SAME


def test_failed_request_is_reported_and_server_continues(wgpu_lib):
    W, dl = 96, 1e-3
    uvw, freq, vis = synthetic.random_points(200, 2, W, dl, seed=3)
    geom = dict(width=W, height=W, dl=dl, dm=dl, epsilon=1e-4)
    with GriddingServer(8e9, max_active=2) as srv:
        srv.wait(srv.submit_invert(geom, uvw, freq, vis, session=5))
        # same session, different shape: rejected when it runs
        t = srv.submit_invert(geom, uvw[:100], freq, vis[:100], session=5)
        with pytest.raises(_lib.WgpuError) as e:
            srv.wait(t)
        assert e.value.status == _lib.WGPU_ERR_INVALID
        bad = dict(geom, epsilon=0.0)  # rejected by the planner at submission
        with pytest.raises(_lib.WgpuError):
            srv.submit_invert(bad, uvw, freq, vis)
        img = srv.wait(srv.submit_invert(geom, uvw, freq, vis))
        assert np.isfinite(img).sum() > 0
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 2
