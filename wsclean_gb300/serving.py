"""Mixed-size request stream for the request server, and its three drivers.

The stream follows the serving workload: grid (inversion) and degrid
(prediction) requests in a 60/40 mix, image sides log-uniform between two
bounds, visibility counts log-uniform between two bounds drawn from the
64-antenna 3 km array (16 channels 120-180 MHz, 10" pixels, 20 point sources),
epsilon 1e-4 or 1e-5 with equal probability, each request running several major
cycles on the same visibilities.

Drivers (all through wsclean_gb300.server.GriddingServer, host buffers, with
one plane budget so that every driver runs the same plans):
  one_at_a_time : one worker slot, no sessions: every cycle of every request is
                  a plain inversion / prediction call, the next submitted when
                  the previous has finished (the plain per-request GPU path).
  saturated     : every request arrives at once; `slots` workers, one session
                  per request (state resident across its cycles).
  poisson       : requests arrive as a Poisson process at a given rate; same
                  server set-up as `saturated`; per-request latency (arrival to
                  the end of its last cycle) gives p50 / p99.
"""
import math
import threading
import time

import numpy as np

from . import synthetic
from .server import GriddingServer

N_CHAN = 16
ARRAY = "plain1024"  # the 64-antenna, 3 km array workload (2016 baselines per step)


def make_pool(max_vis, seed=11):
    """Visibility pool of the 3 km array with enough time steps for the largest
    request: uvw, freq, vis (model of 20 sources plus noise) on the host."""
    n_bl = 64 * 63 // 2
    n_t = max(1, math.ceil(max_vis / (N_CHAN * n_bl)))
    d = synthetic.make_workload(ARRAY, seed=seed, with_model=False, n_t=n_t)
    try:
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        v = synthetic.model_vis_torch(d["uvw"], d["freq"], d["sources"], dev)
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        v = v + 0.01 * math.sqrt(2.0) * torch.randn(v.shape, generator=g, dtype=v.dtype,
                                                    device=dev)
        vis = v.cpu().numpy()
        del v
    except Exception as e:  # data generation only; the gridding itself has no fallback
        raise RuntimeError(f"pool generation needs a CUDA device: {e}")
    d["vis"] = np.ascontiguousarray(vis.reshape(-1, N_CHAN))
    return d


def make_stream(n_requests, seed=5, vis_range=(1e5, 1e7), side_range=(512, 4096),
                grid_fraction=0.6, eps_choices=(1e-4, 1e-5), cycles=5, pool_rows=None):
    """Request descriptions (no data): kind, side, rows, first pool row, epsilon."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_requests):
        n_vis = math.exp(rng.uniform(math.log(vis_range[0]), math.log(vis_range[1])))
        rows = max(1, int(n_vis) // N_CHAN)
        side = math.exp(rng.uniform(math.log(side_range[0]), math.log(side_range[1])))
        side = max(32, int(round(side / 32)) * 32)
        row0 = 0
        if pool_rows is not None and pool_rows > rows:
            row0 = int(rng.integers(0, pool_rows - rows))
        reqs.append(dict(id=i + 1, kind="invert" if rng.uniform() < grid_fraction else "predict",
                         side=side, rows=rows, row0=row0,
                         eps=float(eps_choices[int(rng.integers(0, len(eps_choices)))]),
                         cycles=cycles))
    return reqs


def _model_image(pool, side):
    """The pool's sources as pixels of a side x side image (those inside it)."""
    img = np.zeros(side * side, np.float32)
    dl = pool["dl"]
    for l, m, s in pool["sources"]:
        x = int(round(side / 2 - l / dl))
        y = int(round(m / dl + side / 2))
        if 0 <= x < side and 0 <= y < side:
            img[y * side + x] += s
    return img


class _Prepared:
    """Per-request views into the pool plus a reusable output buffer."""

    def __init__(self, pool, r, models):
        self.r = r
        sl = slice(r["row0"], r["row0"] + r["rows"])
        self.uvw = pool["uvw"][sl]
        self.vis = pool["vis"][sl]
        self.freq = pool["freq"]
        self.geom = dict(width=r["side"], height=r["side"], dl=pool["dl"], dm=pool["dl"],
                         epsilon=r["eps"])
        if r["kind"] == "predict":
            if r["side"] not in models:
                models[r["side"]] = _model_image(pool, r["side"])
            self.model = models[r["side"]]
        self.out = None

    def buffer(self):
        if self.out is None:
            n = self.r["side"] ** 2 if self.r["kind"] == "invert" else self.r["rows"] * N_CHAN
            self.out = np.empty(n, np.float32 if self.r["kind"] == "invert" else np.complex64)
        return self.out

    def submit(self, srv, session):
        if self.r["kind"] == "invert":
            return srv.submit_invert(self.geom, self.uvw, self.freq, self.vis, 1.0,
                                     session=session, out=self.buffer())
        return srv.submit_predict(self.geom, self.uvw, self.freq, self.model, session=session,
                                  out=self.buffer())


def _percentiles(lat_ms):
    a = np.asarray(lat_ms, np.float64)
    return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)),
            "mean_ms": float(a.mean()), "max_ms": float(a.max())}


def total_vis(reqs):
    return float(sum(r["rows"] * N_CHAN * r["cycles"] for r in reqs))


def one_at_a_time(pool, reqs, device_bytes, plane_budget, keep_ids=()):
    models = {}
    kept = {}
    lat = []
    with GriddingServer(device_bytes, max_active=1, plane_budget_bytes=plane_budget) as srv:
        t0 = time.perf_counter()
        for r in reqs:
            p = _Prepared(pool, r, models)
            a = time.perf_counter()
            for _ in range(r["cycles"]):
                srv.wait(p.submit(srv, 0))
            lat.append((time.perf_counter() - a) * 1e3)
            if r["id"] in keep_ids:
                kept[r["id"]] = p.out.copy()
        wall = time.perf_counter() - t0
    return dict(wall_s=wall, gvis_s=total_vis(reqs) / wall / 1e9, **_percentiles(lat)), kept


def _serve(pool, reqs, device_bytes, plane_budget, slots, arrivals, keep_ids=()):
    """Submits each request's cycles at its arrival time (one session per
    request), waits for them on a helper thread, closes the session."""
    models = {}
    prepared = [_Prepared(pool, r, models) for r in reqs]
    lat = [None] * len(reqs)
    errors = []
    kept = {}
    with GriddingServer(device_bytes, max_active=slots, plane_budget_bytes=plane_budget) as srv:
        def finish(i, tickets, p):
            try:
                for t in tickets:
                    srv.wait(t)
                lat[i] = tickets[-1].latency_ms
                if p.r["id"] in keep_ids:
                    kept[p.r["id"]] = p.out.copy()
                srv.close_session(p.r["id"])
                p.out = None
            except Exception as e:  # reported after the run
                errors.append(f"request {p.r['id']}: {e}")

        threads = []
        t0 = time.perf_counter()
        for i, (p, at) in enumerate(zip(prepared, arrivals)):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            tickets = [p.submit(srv, p.r["id"]) for _ in range(p.r["cycles"])]
            th = threading.Thread(target=finish, args=(i, tickets, p), daemon=True)
            th.start()
            threads.append(th)
        for th in threads:
            th.join()
        wall = time.perf_counter() - t0
        stats = srv.stats()
    if errors:
        raise RuntimeError("; ".join(errors[:5]))
    return dict(wall_s=wall, gvis_s=total_vis(reqs) / wall / 1e9,
                peak_running=int(stats["peak_running"]),
                peak_device_gb=stats["peak_device_bytes"] / 1e9,
                submissions_held_for_memory=int(stats["held_for_memory"]),
                **_percentiles(lat)), kept


def saturated(pool, reqs, device_bytes, plane_budget, slots, keep_ids=()):
    return _serve(pool, reqs, device_bytes, plane_budget, slots, [0.0] * len(reqs), keep_ids)


def poisson(pool, reqs, device_bytes, plane_budget, slots, rate_per_s, seed=17):
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, len(reqs)))
    res, _ = _serve(pool, reqs, device_bytes, plane_budget, slots, list(arrivals))
    res["offered_rate_per_s"] = rate_per_s
    return res
