"""Writes oracle/plans.json: the gridding plans (grid size, kernel support and
beta, w planes) of the named synthetic workloads, as the library's planner
chooses them for the samples it grids.

TEST INFRASTRUCTURE.  bench.py's reference arm times the oracle's CPU
w-gridder with these plans, so that it never loads the product library; a
CPU test checks that the file still matches the planner.

    python -m oracle.make_plans
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PLANS = os.path.join(HERE, "plans.json")
WORKLOADS = ("wide8192", "wide2048", "plain1024")
FIELDS = ("width", "height", "nu", "nv", "support", "tile", "n_planes", "plane_batch", "sigma",
          "beta", "dl", "dm", "l_shift", "m_shift", "w0", "dw", "nm1_center", "est_error")


def plan_request(name):
    """Planner inputs of a workload: image geometry, epsilon, and the w range
    and count of its non-zero samples (those inside the Nyquist limit), with
    the geometry of synthetic.make_workload(name)."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from wsclean_gb300 import synthetic
    cfg = synthetic.WORKLOADS[name]
    rng = np.random.default_rng(2)  # make_workload's seed in the bench
    enu = synthetic.antenna_enu(cfg["n_ant"], cfg["layout"], cfg["radius_m"], rng)
    bxyz, _, _ = synthetic.baselines_xyz(enu)
    uvw = synthetic.uvw_tracks(bxyz, cfg["n_t"], cfg["dt"], cfg["dec_deg"])
    freq = np.linspace(cfg["f0"], cfg["f1"], cfg["n_chan"])
    dl = cfg["pix_arcsec"] * synthetic.ARCSEC
    inv_lambda = freq / synthetic.C_LIGHT
    w_min, w_max, n = np.inf, -np.inf, 0
    for r0 in range(0, uvw.shape[0], 1 << 20):
        u = uvw[r0:r0 + (1 << 20)]
        keep = ((np.abs(u[:, 0:1]) * inv_lambda * dl < 0.5) &
                (np.abs(u[:, 1:2]) * inv_lambda * dl < 0.5))
        wl = u[:, 2:3] * inv_lambda
        if keep.any():
            w_min = min(w_min, float(wl[keep].min()))
            w_max = max(w_max, float(wl[keep].max()))
        n += int(keep.sum())
    return dict(width=cfg["npix"], height=cfg["npix"], dl=dl, dm=dl, epsilon=cfg["epsilon"],
                w_min=w_min, w_max=w_max, n_vis=n)


def product_plan(name):
    from wsclean_gb300 import _lib
    p = _lib.make_plan(**plan_request(name))
    return {k: getattr(p, k) for k in FIELDS}


def load(name):
    with open(PLANS) as fh:
        return json.load(fh)[name]


def main():
    out = {name: product_plan(name) for name in WORKLOADS}
    with open(PLANS, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(PLANS)


if __name__ == "__main__":
    main()
