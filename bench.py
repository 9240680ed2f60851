#!/usr/bin/env python
"""Grid + degrid throughput of the GB300 w-gridder.

One step = one inversion (AddInversionData of the whole visibility set, the
ms2dirty path behind WGriddingGridder_Simple) followed by one prediction of the
model image at the same visibilities (PredictVisibilities, the dirty2ms path),
on the wide-field workload: 8192 x 8192 image, 3" pixels, 256 antennas
log-radial to 20 km, 32640 baselines x 300 x 8 s, 64 channels 0.9-1.7 GHz,
500 point sources, epsilon 1e-5 (synthetic data of those shapes).

value  : visibilities per second (Gvis/s) with inputs resident in HBM, through
         the _device entry points of the C ABI.
e2e    : the same step through the host-pointer entry points (pinned host
         buffers; host<->device copies inside the timed region).
Prints one JSON line (rank 0).  --impl reference times the CPU implementation
(the oracle's FP64 w-gridder port) on the host cores instead.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD_TEXT = {
    "wide8192": ("wide-field 8192x8192, 3arcsec pixels, 256 antennas log-radial to 20 km, "
                 "32640 baselines x 300 x 8 s, 64 channels 0.9-1.7 GHz, 500 sources, eps 1e-5"),
    "wide2048": ("profiling-size wide field: the wide-field array, 3arcsec pixels and band on "
                 "a 2048x2048 image, 32640 baselines x 8 x 8 s, 64 channels, eps 1e-5"),
    "fullpol4096": ("full polarisation 4096x4096, 10arcsec pixels, 64 antennas in a 3 km disk, "
                    "2016 baselines x 60 x 10 s, 32 channels 120-180 MHz, XX/XY/YX/YY from 20 "
                    "sources with random Stokes Q, U, V (|pol frac| <= 0.3), per-antenna full "
                    "Jones solutions per time step and channel, eps 1e-4"),
    "facets": ("batched facets: 37 facets of 512-3072 pixels (multiples of 4), 10arcsec "
               "pixels, centres within a 6 deg field, x 8 output channels of 2 channels; "
               "64 antennas in a 3 km disk, 2016 baselines x 620 x 10 s (scaled from 6200), "
               "16 channels 120-180 MHz, 20 sources, eps 1e-4"),
    "plain1024": ("plain 1024x1024, 10arcsec pixels, 64 antennas in a 3 km disk, 2016 baselines "
                  "x 60 x 10 s, 16 channels 120-180 MHz, 20 sources, eps 1e-4"),
    "resample": ("boundary resampling: an 8192x8192 image resampled to the 5120x5120 small-"
                 "inversion size and back (FinishInversion / StartPredict resampler), FFT "
                 "method, FP32"),
    "rowweights": ("raw-row weighting: the wide-field array and band, 32640 baselines x 75 x 8 s, "
                   "64 channels 0.9-1.7 GHz, 4 correlations (XX, XY, YX, YY) with visibility "
                   "weights, Briggs 0 imaging weights on the 8192x8192 3arcsec grid; "
                   "CalculateWeights + ApplyWeights + collapse to Stokes I per sample"),
}
METRIC = "Gvis/s grid+degrid at rel.err <=1e-5 vs FP64 DFT"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ----------------------------------------------------------------- clocks ---
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------- data ---
def build_data(name, device, seed, max_rows=None):
    import torch
    from wsclean_gb300 import synthetic
    d = synthetic.make_workload(name, seed=seed, max_rows=max_rows, with_model=False)
    uvw, freq, wts = d["uvw"], d["freq"], d["weights"]
    cfg = synthetic.WORKLOADS[name]
    vis = synthetic.model_vis_torch(uvw, freq, d["sources"], device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    noise = torch.randn(vis.shape, generator=g, dtype=torch.complex64, device=device)
    d_w = torch.as_tensor(wts, device=device)
    vis = (vis + cfg["noise"] * math.sqrt(2.0) * noise) * d_w
    del noise
    d["d_vis"] = vis.contiguous()
    d["d_mask"] = (d_w > 0).to(torch.uint8).contiguous()
    del d_w
    d["d_uvw"] = torch.as_tensor(uvw, device=device).contiguous()
    d["d_freq"] = torch.as_tensor(freq, device=device).contiguous()
    W = d["width"]
    model = np.zeros(W * W, np.float32)
    for l, m, s in d["sources"]:
        x = int(round(W / 2 - l / d["dl"]))
        y = int(round(m / d["dl"] + W / 2))
        if 0 <= x < W and 0 <= y < W:
            model[y * W + x] += s
    d["model"] = model
    return d


def pinned_copy(t):
    import torch
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h


# ------------------------------------------------------- algorithmic bytes ---
def stage_bytes(stage, direction, p, n_vis, n_rows, n_batch_avg, n_batches):
    """Minimum HBM bytes of one launch of `stage` (per plane batch), from the
    per-request terms of the survey's byte count: the gridded planes written
    (read when degridding) once, and the samples' 8 B plus 24 B of uvw per
    row spread over the batches (the samples are read by the inversion and
    written by the prediction)."""
    nu, nv, W, H = p.nu, p.nv, p.width, p.height
    rs = (W + 31) // 32 * 32
    nb = n_batch_avg
    plane = 8.0 * nu * nv * nb
    rows = 8.0 * rs * nv * nb
    samples = (8.0 * n_vis + 24.0 * n_rows) / n_batches
    if stage in ("grid", "degrid"):
        return plane + samples
    if stage == "fft_rows":
        return plane + rows
    if stage == "fft_cols_a":
        return 2 * rows
    if stage == "fft_cols_b_screen":
        if direction == "invert":
            return rows + 8.0 * W * H + 16.0 * W * H
        return rows + 8.0 * W * H + 4.0 * W * H
    return None


def survey_request_bytes(p, n_vis, n_rows):
    """Per-request algorithmic bytes: 8 N_vis + 24 N_rows + n_w (40 sigma^2 + 16)
    Nx Ny + 4 Nx Ny, with sigma^2 Nx Ny the padded grid actually used."""
    npix = p.width * p.height
    return 8.0 * n_vis + 24.0 * n_rows + p.n_planes * (40.0 * p.nu * p.nv + 16.0 * npix) + 4.0 * npix


# ------------------------------------------------------------ CPU baseline ---
def cpu_sample_step(d, plan, vis_rows, n_baselines, plane_fraction, seed):
    """One bounded CPU step on a sample of the workload: the oracle's FP64 CPU
    w-gridder (all host threads) grids, then predicts, the samples of
    n_baselines random baselines (every time step and channel: whole uv
    tracks, so the sample keeps the data's locality along a track) over all
    the planes they touch, and runs plane_fraction of one plane pass in each
    direction.  Returns (measured seconds, extrapolated seconds of the whole
    inversion + prediction, sample description).  vis_rows(rows) returns the
    visibilities of the sampled rows (zero where the sample is not gridded)."""
    import oracle
    rng = np.random.default_rng(seed)
    n_rows = d["uvw"].shape[0]
    n_bl = d["n_ant"] * (d["n_ant"] - 1) // 2
    n_t = -(-n_rows // n_bl)
    bls = np.sort(rng.choice(n_bl, size=min(n_baselines, n_bl), replace=False))
    rows = (np.arange(n_t)[:, None] * n_bl + bls[None, :]).ravel()
    rows = np.sort(rows[rows < n_rows])
    uvw = d["uvw"][rows]
    vis = vis_rows(rows)
    n_sample = int(np.count_nonzero(vis))
    cores = os.cpu_count()
    w0 = time.perf_counter()
    t_grid, t_pi = oracle.wgrid_time_parts(plan, uvw, d["freq"], vis, n_threads=cores,
                                           plane_fraction=plane_fraction)
    t_degrid, t_pp = oracle.wgrid_time_predict_parts(plan, uvw, d["freq"], vis, n_threads=cores,
                                                     plane_fraction=plane_fraction)
    wall = time.perf_counter() - w0
    n_gridded = int(d["n_gridded"])
    n_planes = int(plan["n_planes"])
    full = ((t_grid + t_degrid) * n_gridded / max(n_sample, 1) +
            (t_pi + t_pp) / plane_fraction * n_planes)
    text = (f"FP64 CPU w-gridder (oracle port, {cores} threads): {bls.size} random baselines "
            f"x {n_t} time steps ({rows.size} rows, {n_sample} gridded samples) gridded in "
            f"{t_grid:.2f} s and predicted in {t_degrid:.2f} s over all their planes; "
            f"{plane_fraction:g} of one {plan['nu']}x{plan['nv']} plane pass in each direction "
            f"in {t_pi:.2f} s + {t_pp:.2f} s; extrapolated to {n_gridded} samples x "
            f"{n_planes} planes per direction ({full:.0f} s per inversion + prediction)")
    return wall, full, text


def cpu_baseline(d, vis_rows, plan, n_vis_total, n_baselines, plane_fraction, seed=3):
    """The CPU baseline of the GPU arm: one bounded CPU step (cpu_sample_step)."""
    wall, full, text = cpu_sample_step(d, plan, vis_rows, n_baselines, plane_fraction, seed)
    return dict(value=n_vis_total / full / 1e9, unit="Gvis/s", cores=os.cpu_count(),
                kind="port", sample=text, seconds_measured=round(wall, 2))


def accuracy_full(d, g, d_out, n_pix=4096, cpu_rows=20000, cpu_pix=64, seed=4):
    """The product's error over EVERY gridded sample: the inversion at n_pix
    seeded pixels and the prediction at every gridded sample, both against the
    FP64 direct transform on the GPU (oracle/dft_cuda.cu, the checker, outside
    the timed region).  The twin itself is cross-checked against the CPU
    oracle on cpu_pix of those pixels over a cpu_rows row subset."""
    import torch
    import oracle
    rng = np.random.default_rng(seed)
    W, dl = d["width"], d["dl"]
    n_rows, n_chan = d["uvw"].shape[0], d["freq"].size
    g.InitializeInversion()
    g.AddInversionDataDevice(n_rows, n_chan, d["d_uvw"].data_ptr(), d["d_freq"].data_ptr(),
                             d["d_vis"].data_ptr())
    img = g.RealImage().astype(np.float64)
    g.InitializePrediction(d["model"])
    g.PredictVisibilitiesMaskedDevice(n_rows, n_chan, d["d_uvw"].data_ptr(),
                                      d["d_freq"].data_ptr(), d["d_mask"].data_ptr(),
                                      d_out.data_ptr())
    torch.cuda.synchronize()
    pix = rng.choice(W * W, size=n_pix, replace=False)
    t0 = time.perf_counter()
    ref = oracle.cuda_dft_invert(d["d_uvw"], d["freq"], d["d_vis"], W, W, dl, dl, pixels=pix)
    t_inv = time.perf_counter() - t0
    inv_err = float(np.linalg.norm(img[pix] - ref) / np.linalg.norm(ref))
    t0 = time.perf_counter()
    _, e2, r2 = oracle.cuda_dft_predict(d["d_uvw"], d["freq"], d["model"], W, W, dl, dl,
                                        mask=d["d_mask"], pred=d_out)
    t_pred = time.perf_counter() - t0
    pred_err = float(math.sqrt(e2 / r2))
    # the twin against the CPU oracle on a row subset
    rows = np.sort(rng.choice(n_rows, size=min(cpu_rows, n_rows), replace=False))
    uvw_s = d["uvw"][rows]
    vis_s = d["d_vis"][torch.as_tensor(rows, device=d["d_vis"].device)].cpu().numpy()
    twin = oracle.cuda_dft_invert(uvw_s, d["freq"], vis_s, W, W, dl, dl, pixels=pix[:cpu_pix])
    cpu = oracle.dft_invert(uvw_s, d["freq"], vis_s, W, W, dl, dl, pixels=pix[:cpu_pix],
                            n_threads=os.cpu_count())
    twin_err = float(np.linalg.norm(twin - cpu) / np.linalg.norm(cpu))
    n_g = int(d["n_gridded"])
    return {"invert_rel_l2": inv_err, "predict_rel_l2": pred_err,
            "sample": (f"all {n_g} gridded samples: inversion at {n_pix} seeded pixels, "
                       f"prediction at every gridded sample; FP64 direct transform on the GPU "
                       f"({t_inv:.1f} s + {t_pred:.1f} s)"),
            "twin_vs_cpu_rel_l2": twin_err,
            "twin_vs_cpu_sample": f"{rows.size} rows x {n_chan} channels x {cpu_pix} pixels"}


def run_bound(d, g, d_out, inv_weight, stream, cycles=4, warmup=1):
    """Major cycles on a bound visibility set, as WSClean runs them: the rows
    (uvw, frequencies, the gridded-sample mask) are bound once
    (wgpu_gridder_bind: plan, bucketing and the two captured pipelines), then
    every cycle grids the visibilities and predicts the model image by
    replaying the graphs.  Reports the bind time, the per-cycle time and the
    agreement with the plain (per-call) path on the same data."""
    import torch
    n_rows, n_chan = d["uvw"].shape[0], d["freq"].size
    n_vis = n_rows * n_chan
    mask = d["d_mask"].cpu().numpy()
    # the plain path's image and prediction of this data, for the agreement
    g.InitializeInversion()
    g.AddInversionDataDevice(n_rows, n_chan, d["d_uvw"].data_ptr(), d["d_freq"].data_ptr(),
                             d["d_vis"].data_ptr())
    g.FinalizeImage(inv_weight)
    img_plain = g.RealImage().astype(np.float64)
    g.InitializePrediction(d["model"])
    g.PredictVisibilitiesMaskedDevice(n_rows, n_chan, d["d_uvw"].data_ptr(),
                                      d["d_freq"].data_ptr(), d["d_mask"].data_ptr(),
                                      d_out.data_ptr())
    pred_plain = d_out.clone()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.Bind(n_rows, n_chan, d["uvw"], d["freq"], mask)
    torch.cuda.synchronize()
    bind_s = time.perf_counter() - t0
    trials = g.last_tuning()
    bp = g.last_plan()
    stages = {}

    def cycle(keep_image=False):
        g.InitializeInversion()
        g.InvertBoundDevice(d["d_vis"].data_ptr())
        stages["invert"] = g.last_timings()
        g.FinalizeImage(inv_weight)
        if keep_image:
            stages["image"] = g.RealImage().astype(np.float64)
        g.InitializePrediction(d["model"])
        g.PredictBoundDevice(d_out.data_ptr())
        stages["predict"] = g.last_timings()

    for _ in range(warmup):
        cycle()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(cycles):
        cycle()
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / cycles
    cycle(keep_image=True)  # one more cycle, outside the timed region, for the comparison
    img_bound = stages.pop("image")
    ok = np.isfinite(img_plain)
    img_rel = float(np.linalg.norm(img_bound[ok] - img_plain[ok]) / np.linalg.norm(img_plain[ok]))
    pred_rel = float(torch.linalg.vector_norm(d_out - pred_plain).item() /
                     torch.linalg.vector_norm(pred_plain).item())
    g.Unbind()
    out = {"ms_per_cycle": ms, "gvis_s": n_vis / (ms * 1e-3) / 1e9, "cycles": cycles,
           "bind_s": round(bind_s, 2),
           "plan": {"support": bp.support, "sigma": bp.sigma, "nu": bp.nu,
                    "n_planes": bp.n_planes, "plane_batch": bp.plane_batch},
           "stages": {f"{k}:{n}": round(v[0], 3) for k, st in stages.items()
                      for n, v in st.items()},
           "bound_vs_plain_rel_l2": {"image": img_rel, "prediction": pred_rel},
           "cycle": "InitializeInversion + invert_bound (graph replay) + FinalizeImage + "
                    "InitializePrediction + predict_bound (graph replay), device buffers; "
                    "bucketing paid once at bind"}
    if trials:
        out["tuning"] = [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in t.items()}
                         for t in trials]
    return out


# -------------------------------------------------------------- GPU arm -----
def run_gpu(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from wsclean_gb300 import _lib, replicas
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    _lib.lib()

    t0 = time.time()
    d = build_data(args.workload, dev, seed=2 + rank, max_rows=args.max_rows)
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    n_rows, n_chan = d["uvw"].shape[0], d["freq"].size
    n_vis = n_rows * n_chan
    d["n_gridded"] = int(d["d_mask"].sum().item())
    eps = d["epsilon"]
    W = d["width"]
    # the reference picks the double instantiation at this accuracy
    num_t = np.float64 if eps <= 1.01e-5 else np.float32
    g = WGriddingGridder_Simple(W, W, W, W, d["dl"], d["dl"], 0.0, 0.0, os.cpu_count(),
                                epsilon=eps, num_t=num_t)
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    d_out = torch.empty(n_vis, dtype=torch.complex64, device=dev)
    inv_weight = 1.0 / d["image_weight"]

    timings = {}
    # Inputs smaller than twice the L2 (129 MB): a 256 MB buffer is written on
    # the gridder stream before every step, inside the timed region.
    l2_flush = None
    if n_vis * 8 < 2 * 129e6:
        l2_flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step_device():
        if l2_flush is not None:
            with torch.cuda.stream(stream):
                l2_flush.fill_(1)
        g.InitializeInversion()
        g.AddInversionDataDevice(n_rows, n_chan, d["d_uvw"].data_ptr(), d["d_freq"].data_ptr(),
                                 d["d_vis"].data_ptr())
        timings["invert"] = g.last_timings()
        g.FinalizeImage(inv_weight)
        g.InitializePrediction(d["model"])
        g.PredictVisibilitiesMaskedDevice(n_rows, n_chan, d["d_uvw"].data_ptr(),
                                          d["d_freq"].data_ptr(), d["d_mask"].data_ptr(),
                                          d_out.data_ptr())
        timings["predict"] = g.last_timings()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = _lib.lib().wgpu_kernel_launch_count()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        start.record(stream)
        for _ in range(steps):
            fn()
        end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        ms = start.elapsed_time(end)
        launches = _lib.lib().wgpu_kernel_launch_count() - launches0
        if world > 1:
            # replicas: the slowest rank's time (no collective on the data path)
            ms = replicas.max_over_ranks(ms, device=dev)
            torch.distributed.barrier()
        return ms, wall, launches

    clocks = ClockSampler(local)
    clocks.start()
    ms, wall, launches = timed(step_device, args.steps, args.warmup)
    clk = clocks.stop()
    ms_per_step = ms / args.steps
    value = replicas.aggregate_rate([n_vis] * world, ms_per_step * 1e-3) / 1e9

    # plans of the last step
    g.InitializeInversion()
    g.AddInversionDataDevice(n_rows, n_chan, d["d_uvw"].data_ptr(), d["d_freq"].data_ptr(),
                             d["d_vis"].data_ptr())
    plan_inv = g.last_plan()
    inv_stage = g.last_timings()
    g.InitializePrediction(d["model"])
    g.PredictVisibilitiesMaskedDevice(n_rows, n_chan, d["d_uvw"].data_ptr(),
                                      d["d_freq"].data_ptr(), d["d_mask"].data_ptr(),
                                      d_out.data_ptr())
    plan_pred = g.last_plan()
    pred_stage = g.last_timings()
    torch.cuda.synchronize()

    # ---- roofline of the dominant kernel
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    rows = []
    for direction, stages, plan in (("invert", inv_stage, plan_inv), ("predict", pred_stage, plan_pred)):
        n_batches = math.ceil(plan.n_planes / plan.plane_batch)
        nb_avg = plan.n_planes / n_batches
        for name, (sms, cnt) in stages.items():
            b = stage_bytes(name, direction, plan, d["n_gridded"], n_rows, nb_avg, n_batches)
            rows.append(dict(direction=direction, stage=name, ms=sms, launches=cnt,
                             bytes_per_launch=b))
    dom = max(rows, key=lambda r: r["ms"])
    per_launch_ms = dom["ms"] / max(dom["launches"], 1)
    achieved = (dom["bytes_per_launch"] / (per_launch_ms * 1e-3) / 1e9
                if dom["bytes_per_launch"] else None)
    roofline = {"bound": "hbm", "kernel": f"{dom['direction']}:{dom['stage']}",
                "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak if achieved else None), "traffic": None,
                "peak_source": peak_src,
                "stages": {f"{r['direction']}:{r['stage']}": round(r["ms"], 3) for r in rows}}
    if args.traffic:
        roofline["traffic"] = args.traffic
    elif args.workload == "wide8192" and dom["stage"] == "grid":
        # DRAM bytes of one launch of the dominant kernel from a committed ncu
        # capture (scaled from the profiling-size case; see profiles/)
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            t = json.load(open(tpath)).get("grid_kernel")
            if t:
                roofline["traffic"] = float(t["traffic_bytes_per_launch"]) / 1e9
                roofline["traffic_unit"] = "GB per launch"
                roofline["achieved_bytes_per_launch_gb"] = dom["bytes_per_launch"] / 1e9
                roofline["traffic_source"] = t["how"]
                if "shared_pipe_frac" in t:
                    roofline["shared_pipe_frac"] = t["shared_pipe_frac"]
                    roofline["shared_pipe_source"] = t["shared_pipe_how"]

    # ---- e2e through the host-pointer API (pinned buffers)
    e2e = None
    if not args.no_e2e:
        h_uvw = pinned_copy(d["d_uvw"]).numpy()
        h_freq = d["freq"]
        h_vis = pinned_copy(d["d_vis"]).numpy()
        h_mask = pinned_copy(d["d_mask"]).numpy()
        h_out = pinned_copy(d_out).numpy()
        h_model = pinned_copy(torch.from_numpy(d["model"])).numpy()
        h_img = torch.empty(W * W, dtype=torch.float32, pin_memory=True).numpy()

        def step_host():
            g.InitializeInversion()
            g.AddInversionData(n_rows, n_chan, h_uvw, h_freq, h_vis)
            g.FinalizeImage(inv_weight)
            g.RealImage(out=h_img)
            g.InitializePrediction(h_model)
            g.PredictVisibilitiesMasked(n_rows, n_chan, h_uvw, h_freq, h_mask, out=h_out)

        e_ms, e_wall, _ = timed(step_host, max(1, args.steps // 2), 1)
        e_steps = max(1, args.steps // 2)
        e_ms_step = max(e_ms, e_wall * 1e3) / e_steps
        h2d = (h_uvw.nbytes * 2 + h_freq.nbytes * 2 + h_vis.nbytes + h_mask.nbytes +
               d["model"].nbytes)
        d2h = h_out.nbytes + W * W * 4
        e2e = {"value": world * n_vis / (e_ms_step * 1e-3) / 1e9, "unit": "Gvis/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "ms_per_step": e_ms_step}
        d["h_vis"] = h_vis.reshape(n_rows, n_chan)
    else:
        d["h_vis"] = d["d_vis"].cpu().numpy().reshape(n_rows, n_chan)

    result = {
        "metric": METRIC, "value": value, "unit": "Gvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD_TEXT.get(args.workload, args.workload),
            "n_vis": n_vis, "n_vis_gridded": d["n_gridded"], "n_rows": n_rows,
            "flagged_fraction": d["flagged_fraction"],
            "step": "InitializeInversion + AddInversionData + FinalizeImage + "
                    "InitializePrediction + PredictVisibilities(masked to the gridded set)",
            "plan_invert": {k: getattr(plan_inv, k) for k in ("nu", "support", "sigma",
                                                              "n_planes", "plane_batch",
                                                              "est_error")},
            "plan_predict": {k: getattr(plan_pred, k) for k in ("nu", "support", "sigma",
                                                                "n_planes", "plane_batch",
                                                                "est_error")},
            "l2": (f"inputs larger than L2 (visibilities {n_vis * 8 / 1e9:.1f} GB, planes "
                   f"{plan_inv.nu * plan_inv.nv * 8 / 1e9:.2f} GB each)" if l2_flush is None
                   else "L2 flushed before each step (256 MB written on the gridder stream, "
                        "inside the timed region)"),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "request_bytes_roofline_frac": None,
            "datagen_s": round(gen_s, 1),
        },
        "roofline": roofline,
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": int(launches),
    }
    req_bytes = (survey_request_bytes(plan_inv, d["n_gridded"], n_rows) +
                 survey_request_bytes(plan_pred, d["n_gridded"], n_rows))
    result["config"]["request_bytes_roofline_frac"] = (req_bytes / (ms_per_step * 1e-3) / 1e9) / peak
    # the plan-independent ratio: only the visibility term, both directions
    vis_bytes = 2.0 * (8.0 * d["n_gridded"] + 24.0 * n_rows)
    result["config"]["visibility_bytes_roofline_frac"] = (
        (vis_bytes / (ms_per_step * 1e-3) / 1e9) / peak)
    result["config"]["request_bytes_plan"] = {
        "sigma": plan_inv.sigma, "support": plan_inv.support, "n_w": plan_inv.n_planes,
        "nu": plan_inv.nu, "nv": plan_inv.nv}
    # `value` counts every sample handed to the step, as the reference's calls
    # receive them; the samples beyond the image's Nyquist limit are zero and
    # neither gridded nor predicted, so the rate of processed samples is lower
    result["config"]["gridded_gvis_s"] = (world * d["n_gridded"] / (ms_per_step * 1e-3) / 1e9)

    if rank == 0 and not args.no_accuracy:
        result["config"]["accuracy"] = accuracy_full(d, g, d_out)
    if not args.no_bound:
        result["bound"] = run_bound(d, g, d_out, inv_weight, stream)
    if args.tune_bound:
        # the same major cycles on a gridder created with tuning = 1: the bind
        # times the best candidate plans on these rows and keeps the fastest
        # (the untuned gridder's buffers are released first)
        g.close()
        torch.cuda.empty_cache()
        gt = WGriddingGridder_Simple(W, W, W, W, d["dl"], d["dl"], 0.0, 0.0, os.cpu_count(),
                                     epsilon=eps, num_t=num_t, tuning=True)
        st = torch.cuda.ExternalStream(gt.stream(), device=dev)
        result["bound_tuned"] = run_bound(d, gt, d_out, inv_weight, st)
        gt.close()
    if args.serve_requests > 0:
        g.close()  # release the wide-field gridder's planes before serving
        del d_out
        d.pop("d_vis", None)
        torch.cuda.empty_cache()
        free_b, _ = torch.cuda.mem_get_info()
        result["serving"] = run_serving(args, 0.7 * free_b)
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(d, lambda r: d["h_vis"][r], plan_inv.as_dict(),
                                              n_vis, args.cpu_baselines, args.cpu_plane_fraction)
        result["cpu_baseline"].pop("seconds_per_step", None)
    g.close()
    return result


# ------------------------------------------------------- full polarisation ---
def run_fullpol(args):
    """Corrected inversion (full-Jones gains applied on the device, collapsed to
    Stokes I) followed by prediction of the model image, through the host API;
    accuracy over every sample against the oracle's gain application and the
    FP64 direct transform on the GPU."""
    import torch
    import oracle
    from wsclean_gb300 import synthetic
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    d = synthetic.make_workload("fullpol4096", seed=3, with_model=False)
    vis4, ant, tof, sol, n_t = synthetic.full_polarisation(d, dev)
    gen_s = time.time() - t0
    n_rows, n_chan, n_ant = d["uvw"].shape[0], d["freq"].size, d["n_ant"]
    W, dl, eps = d["width"], d["dl"], d["epsilon"]
    model = np.zeros(W * W, np.float32)
    for l, m, sflux in d["sources"]:
        x, y = int(round(W / 2 - l / dl)), int(round(m / dl + W / 2))
        if 0 <= x < W and 0 <= y < W:
            model[y * W + x] += sflux
    uvw = pinned_copy(torch.as_tensor(d["uvw"])).numpy()
    freq = d["freq"]
    vis_p = pinned_copy(torch.as_tensor(vis4)).numpy()
    g = WGriddingGridder_Simple(W, W, W, W, dl, dl, 0.0, 0.0, os.cpu_count(), epsilon=eps)
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    out = {}

    def step():
        g.InitializeInversion()
        g.AddInversionDataWithCorrectionCallback("full", 4, n_rows, uvw, freq, n_chan, ant, vis_p,
                                                 tof, sol, 4, n_t, n_ant)
        g.FinalizeImage(1.0)
        out["img"] = g.RealImage()
        g.InitializePrediction(model)
        out["pv"] = g.PredictVisibilities(n_rows, n_chan, uvw, freq)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib_launches()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    start.record(stream)
    for _ in range(args.steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    launches = _lib_launches() - l0
    ms = max(start.elapsed_time(end), wall * 1e3) / args.steps
    n_vis = n_rows * n_chan
    plan = g.last_plan()
    # accuracy over every sample: the oracle's gain application and collapse of
    # all rows, then the FP64 direct transform on the GPU (the checker, outside
    # the timed region) at 4096 seeded pixels for the inversion and at every
    # sample for the prediction of the model image
    rng = np.random.default_rng(7)
    corrected = oracle.apply_gains(4, 4, vis4, ant, tof, sol, 4, n_ant)
    img = out["img"].astype(np.float64)
    pix = rng.choice(W * W, 4096, replace=False)
    ref = oracle.cuda_dft_invert(d["uvw"], freq, corrected, W, W, dl, dl, pixels=pix)
    inv_err = float(np.linalg.norm(img[pix] - ref) / np.linalg.norm(ref))
    _, e2, r2 = oracle.cuda_dft_predict(d["uvw"], freq, model, W, W, dl, dl,
                                        pred=np.ascontiguousarray(out["pv"]).ravel())
    pred_err = float(math.sqrt(e2 / r2))
    g.close()
    value = n_vis / (ms * 1e-3) / 1e9
    h2d = uvw.nbytes * 2 + freq.nbytes * 2 + vis_p.nbytes + ant.nbytes + tof.nbytes + sol.nbytes + model.nbytes
    d2h = n_vis * 8 + W * W * 4
    return {
        "metric": "Gvis/s corrected inversion + prediction (full-Jones gains, Stokes I)",
        "value": value, "unit": "Gvis/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT["fullpol4096"], "n_rows": n_rows,
                   "n_vis": n_vis, "correlations_per_vis": 4,
                   "l2": (f"working set larger than L2 ({plan.n_planes} w planes of "
                          f"{plan.nu * plan.nv * 8 / 1e9:.2f} GB per step direction, "
                          f"{n_vis * 32 / 1e9:.2f} GB of 4-correlation visibilities)"),
                   "step": "InitializeInversion + AddInversionDataWithCorrectionCallback(full, "
                           "4 pol, Stokes I) + FinalizeImage + RealImage + InitializePrediction "
                           "+ PredictVisibilities, host buffers",
                   "plan": {k: getattr(plan, k) for k in ("nu", "support", "sigma", "n_planes",
                                                          "plane_batch", "est_error")},
                   "accuracy": {"invert_rel_l2": inv_err, "predict_rel_l2": pred_err,
                                "sample": (f"all {n_vis} samples: the oracle's gains and "
                                           "collapse, then the FP64 direct transform on the GPU "
                                           "at 4096 seeded pixels (inversion) and at every "
                                           "sample (prediction)")},
                   "datagen_s": round(gen_s, 1)},
        "clocks": clk,
        "e2e": {"value": value, "unit": "Gvis/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
    }


def _facet_layout(rng, dl):
    """37 facets of seeded uniform 512-3072 pixels (multiples of 4), centres
    within a 6 degree field."""
    half = math.radians(3.0)
    facets = []
    for _ in range(37):
        side = int(rng.uniform(512, 3072)) // 4 * 4
        facets.append(dict(width=side, height=side, dl=dl, dm=dl,
                           l_shift=float(rng.uniform(-half, half)),
                           m_shift=float(rng.uniform(-half, half))))
    return facets


def run_facets_full(args):
    """The batched-facet workload at its full size (6200 time steps, 2.0e8
    samples): the 296 jobs' sorted records (about 240 GB) cannot all stay on
    the device, so every step binds and inverts one output-channel group at a
    time: 37 facets sharing that group's two channels, bucketed, gridded in one
    multi-job launch per wave and transformed from one CUDA graph, then
    released.  Compared with the same 296 jobs through the plain per-call
    path; job 0 is checked against the plain path on its plan and against the
    FP64 direct transform on the GPU (all of its samples, 4096 pixels)."""
    import torch
    import oracle
    from wsclean_gb300 import synthetic
    from wsclean_gb300.facets import FacetBatch
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    t0 = time.time()
    d = synthetic.make_workload("plain1024", seed=4, with_model=False, n_t=args.facet_times)
    vis = synthetic.model_vis_torch(d["uvw"], d["freq"], d["sources"], dev)
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    vis = vis + 0.01 * math.sqrt(2.0) * torch.randn(vis.shape, generator=g, dtype=vis.dtype,
                                                    device=dev)
    groups = list(range(0, 17, 2))
    n_groups = len(groups) - 1
    # each group's two channels as their own contiguous [row][2] input
    d_vis_g = [vis[:, c0:c0 + 2].contiguous() for c0 in groups[:-1]]
    del vis
    gen_s = time.time() - t0
    dl, eps = d["dl"], 1e-4
    facets = _facet_layout(rng, dl)
    n_rows = d["uvw"].shape[0]
    freq = d["freq"]
    img_elems = sum(f["width"] * f["height"] for f in facets)
    outs = [torch.empty(img_elems, dtype=torch.float32, device=dev) for _ in range(n_groups)]
    info = {}

    # one batch object re-bound per channel group: its device memory and
    # bucketing scratch stay allocated from one bind to the next
    fb = FacetBatch(facets, [0, 2], epsilon=eps)

    phase_s = {"bind": 0.0, "invert": 0.0}
    bind_phases = [0.0] * 4  # upload and planning, bucketing, waves, graph capture

    def step():
        for gi in range(n_groups):
            c0 = groups[gi]
            t0 = time.perf_counter()
            fb.bind(d["uvw"], freq[c0:c0 + 2])
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            for k, v in enumerate(fb.info()["bind_ms"]):
                bind_phases[k] += v
            fb.invert_device(d_vis_g[gi].data_ptr(), outs[gi].data_ptr())
            torch.cuda.synchronize()
            phase_s["bind"] += t1 - t0
            phase_s["invert"] += time.perf_counter() - t1
            if gi == 0:
                info.update(fb.info())
                info["plan0"] = fb.job_plan(0)

    for _ in range(min(args.warmup, 1)):
        step()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib_launches()
    torch.cuda.synchronize()
    phase_s.update(bind=0.0, invert=0.0)
    bind_phases[:] = [0.0] * 4
    w0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    ms = (time.perf_counter() - w0) * 1e3 / args.steps
    clk = clocks.stop()
    launches = _lib_launches() - l0
    fb.close()
    per_group_ms = {k: round(v * 1e3 / (args.steps * n_groups), 1) for k, v in phase_s.items()}
    per_group_ms["bind_phases"] = {
        name: round(v / (args.steps * n_groups), 1)
        for name, v in zip(("upload_extents_planning", "bucketing_and_job_tables", "waves",
                            "graph_capture_instantiate"), bind_phases)}
    job_vis = float(n_rows) * 16 * len(facets)
    # the same jobs one at a time through the plain per-call path
    d_uvw = torch.as_tensor(d["uvw"], device=dev)
    d_freq = torch.as_tensor(freq, device=dev)
    gp = [WGriddingGridder_Simple(f["width"], f["height"], f["width"], f["height"], dl, dl,
                                  f["l_shift"], f["m_shift"], 1, epsilon=eps) for f in facets]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for gi in range(n_groups):
        c0 = groups[gi]
        for gg in gp:
            gg.InitializeInversion()
            gg.AddInversionDataDevice(n_rows, 2, d_uvw.data_ptr(), d_freq[c0:c0 + 2].data_ptr(),
                                      d_vis_g[gi].data_ptr())
            gg.FinalizeImage(1.0)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - w0
    for gg in gp:
        gg.close()
    # job 0 (facet 0, first group) against the plain path on its plan and the DFT
    f = facets[0]
    n0 = f["width"] * f["height"]
    img = outs[0][:n0].cpu().numpy().astype(np.float64)
    gg = WGriddingGridder_Simple(f["width"], f["height"], f["width"], f["height"], dl, dl,
                                 f["l_shift"], f["m_shift"], 1, epsilon=eps)
    gg.pin_plan(info["plan0"])
    gg.InitializeInversion()
    gg.AddInversionDataDevice(n_rows, 2, d_uvw.data_ptr(), d_freq[0:2].data_ptr(),
                              d_vis_g[0].data_ptr())
    gg.FinalizeImage(1.0)
    ref = gg.RealImage().astype(np.float64)
    gg.close()
    pix = rng.choice(n0, 4096, replace=False)
    dft = oracle.cuda_dft_invert(d_uvw, freq[0:2], d_vis_g[0], f["width"], f["height"], dl, dl,
                                 f["l_shift"], f["m_shift"], pixels=pix)
    checks = {"job0_vs_plain_rel_l2": rel_l2(img, ref),
              "job0_vs_fp64_dft_rel_l2": rel_l2(img[pix], dft),
              "dft_sample": f"all {n_rows * 2} samples of job 0 at 4096 pixels, FP64 direct "
                            "transform on the GPU"}
    value = job_vis / (ms * 1e-3) / 1e9
    plain_value = job_vis / plain_s / 1e9
    sides = [f["width"] for f in facets]
    return {
        "metric": "Gvis/s batched facet inversion (job-samples: facets x channel groups)",
        "value": value, "unit": "Gvis/s", "n_gpus": 1, "steps": args.steps,
        "warmup": min(args.warmup, 1), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT["facets"].replace(" (scaled from 6200)", "")
                   .replace("620", str(args.facet_times)),
                   "n_rows": n_rows, "n_chan": 16, "samples": n_rows * 16,
                   "facet_sides": [min(sides), max(sides)], "jobs": len(facets) * n_groups,
                   "per_group": {k: int(info[k]) for k in ("n_jobs", "n_waves", "support",
                                                           "graph_kernels")},
                   "job_samples": job_vis,
                   "plain_one_at_a_time_gvis_s": plain_value,
                   "batched_over_plain": value / plain_value, "checks": checks,
                   "per_group_ms": per_group_ms,
                   "datagen_s": round(gen_s, 1),
                   "l2": "working set larger than L2 (planes of every wave, 1.6 GB of samples)",
                   "step": "per output-channel group: re-bind of one batch object (upload, "
                           "plan, bucket 37 jobs, capture; device memory kept from the previous "
                           "bind) + one graph replay; host wall time with the device "
                           "synchronised on both sides"},
        "clocks": clk,
        "gpu_launches": int(launches),
    }


def run_facets(args):
    """Batched facet inversion (all facet x channel jobs, one multi-job gridding
    launch per wave, one CUDA graph) against the same jobs run one at a time
    through the plain per-call path."""
    if args.facet_times > args.facet_resident_times:
        return run_facets_full(args)
    import torch
    import oracle
    from wsclean_gb300 import synthetic
    from wsclean_gb300.facets import FacetBatch
    from wsclean_gb300.gridder import WGriddingGridder_Simple
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    t0 = time.time()
    d = synthetic.make_workload("plain1024", seed=4, with_model=False, n_t=args.facet_times)
    vis = synthetic.model_vis_torch(d["uvw"], d["freq"], d["sources"], dev)
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    vis = vis + 0.01 * math.sqrt(2.0) * torch.randn(vis.shape, generator=g, dtype=vis.dtype,
                                                    device=dev)
    d_vis = vis.contiguous()
    h_vis = pinned_copy(d_vis).numpy()
    gen_s = time.time() - t0
    dl = d["dl"]
    half = math.radians(3.0)
    facets = []
    for _ in range(37):
        side = int(rng.uniform(512, 3072)) // 4 * 4
        facets.append(dict(width=side, height=side, dl=dl, dm=dl,
                           l_shift=float(rng.uniform(-half, half)),
                           m_shift=float(rng.uniform(-half, half))))
    groups = list(range(0, 17, 2))
    n_rows, n_chan = d["uvw"].shape[0], d["freq"].size
    eps = 1e-4
    t0 = time.time()
    fb = FacetBatch(facets, groups, epsilon=eps)
    fb.bind(d["uvw"], d["freq"])
    torch.cuda.synchronize()
    bind_s = time.time() - t0
    info = fb.info()
    out = torch.empty(int(info["image_elems"]), dtype=torch.float32, device=dev)
    stream = torch.cuda.ExternalStream(fb.stream(), device=dev)

    def step():
        fb.invert_device(d_vis.data_ptr(), out.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib_launches()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = _lib_launches() - l0
    ms = start.elapsed_time(end) / args.steps
    job_vis = float(info["job_visibilities"])
    # end to end: host visibilities in, host images out
    h_img = np.empty(int(info["image_elems"]), np.float32)
    w0 = time.perf_counter()
    e_steps = max(1, args.steps // 2)
    for _ in range(e_steps):
        fb.invert(h_vis)
    e_ms = (time.perf_counter() - w0) * 1e3 / e_steps
    # the same jobs one at a time through the plain per-call path
    per_group = [d_vis[:, c0:c0 + 2].contiguous() for c0 in groups[:-1]]
    d_uvw = torch.as_tensor(d["uvw"], device=dev)
    d_freq = torch.as_tensor(d["freq"], device=dev)
    gp = {}
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    images_plain = {}
    for gi in range(len(groups) - 1):
        c0 = groups[gi]
        for fi, f in enumerate(facets):
            key = fi
            if key not in gp:
                gp[key] = WGriddingGridder_Simple(f["width"], f["height"], f["width"], f["height"],
                                                  dl, dl, f["l_shift"], f["m_shift"], 1,
                                                  epsilon=eps)
            gg = gp[key]
            gg.InitializeInversion()
            gg.AddInversionDataDevice(n_rows, 2, d_uvw.data_ptr(), d_freq[c0:c0 + 2].data_ptr(),
                                      per_group[gi].data_ptr())
            gg.FinalizeImage(1.0)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - w0
    # accuracy: two jobs against the plain path on the job's plan, one against the DFT
    images = out.cpu().numpy()
    offs = np.cumsum([0] + [f["width"] * f["height"] for f in facets] * (len(groups) - 1))
    checks = {}
    for job in (0, len(facets) * 3 + 5):
        gi, fi = divmod(job, len(facets))
        f, c0 = facets[fi], groups[gi]
        img = images[offs[job]:offs[job + 1]].astype(np.float64)
        gg = WGriddingGridder_Simple(f["width"], f["height"], f["width"], f["height"], dl, dl,
                                     f["l_shift"], f["m_shift"], 1, epsilon=eps)
        gg.pin_plan(fb.job_plan(job))
        gg.InitializeInversion()
        gg.AddInversionDataDevice(n_rows, 2, d_uvw.data_ptr(), d_freq[c0:c0 + 2].data_ptr(),
                                  per_group[gi].data_ptr())
        gg.FinalizeImage(1.0)
        ref = gg.RealImage().astype(np.float64)
        gg.close()
        checks[f"job{job}_vs_plain_rel_l2"] = float(np.linalg.norm(img - ref) / np.linalg.norm(ref))
        if job == 0:
            pix = rng.choice(f["width"] * f["height"], 64, replace=False)
            hv = h_vis[:, c0:c0 + 2]
            dft = oracle.dft_invert(d["uvw"], d["freq"][c0:c0 + 2], hv, f["width"], f["height"],
                                    dl, dl, f["l_shift"], f["m_shift"], pixels=pix,
                                    n_threads=os.cpu_count())
            checks["job0_vs_dft_rel_l2_64px"] = float(np.linalg.norm(img[pix] - dft) /
                                                      np.linalg.norm(dft))
    for gg in gp.values():
        gg.close()
    corrections = None
    if args.facet_corrections:
        # direction-dependent gains: 4-correlation visibilities (XX = YY = V)
        # and a full-Jones solution table per facet (per time step, channel,
        # antenna), one upload per inversion, gains applied per facet on the
        # device (host entry point: uploads inside the timed region)
        n_ant, n_t = d["n_ant"], d["n_t"]
        vis4 = np.zeros((n_rows, n_chan, 4), np.complex64)
        vis4[:, :, 0] = h_vis.reshape(n_rows, n_chan)
        vis4[:, :, 3] = vis4[:, :, 0]
        ant = np.stack([d["ant1"], d["ant2"]], axis=1).astype(np.uint64)
        tof = np.asarray(d["time_index"], np.uint64)
        crng = np.random.default_rng(5)
        sol = np.zeros((len(facets), n_t, n_chan, n_ant, 4), np.complex64)
        sol[..., 0] = 1.0
        sol[..., 3] = 1.0
        sol += (0.05 * (crng.standard_normal(sol.shape) + 1j * crng.standard_normal(sol.shape))
                ).astype(np.complex64)
        fc = FacetBatch(facets, groups, epsilon=eps)
        t0 = time.time()
        fc.bind(d["uvw"], d["freq"], corrected=True)
        cbind_s = time.time() - t0
        fc.invert_corrected(4, vis4, ant, tof, sol, 4, n_t, n_ant)
        w0 = time.perf_counter()
        for _ in range(e_steps):
            cimgs = fc.invert_corrected(4, vis4, ant, tof, sol, 4, n_t, n_ant)
        c_ms = (time.perf_counter() - w0) * 1e3 / e_steps
        # job 0 (facet 0, first group) against the plain batch on the oracle's
        # gain-applied visibilities for facet 0
        cvis = oracle.apply_gains(4, 4, vis4, ant, tof, sol[0], 4, n_ant)
        ref0 = fb.invert(cvis)[0]
        corrections = {
            "ms_per_inversion": c_ms, "gvis_s": job_vis / (c_ms * 1e-3) / 1e9,
            "uncorrected_e2e_ms": e_ms, "bind_s": round(cbind_s, 2),
            "upload_bytes": int(vis4.nbytes + sol.nbytes + ant.nbytes + tof.nbytes),
            "job0_vs_plain_on_oracle_gains_rel_l2": rel_l2(cimgs[0], ref0),
            "note": "full-Jones per-facet solutions (37 tables), 4 correlations, host buffers"}
        fc.close()
    fb.close()
    value = job_vis / (ms * 1e-3) / 1e9
    plain_value = job_vis / plain_s / 1e9
    sides = [f["width"] for f in facets]
    return {
        "metric": "Gvis/s batched facet inversion (job-samples: facets x channel groups)",
        "value": value, "unit": "Gvis/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT["facets"], "n_rows": n_rows, "n_chan": n_chan,
                   "l2": (f"working set larger than L2 ({int(info['n_waves'])} waves of facet "
                          f"planes per step, {n_rows * n_chan * 8 / 1e9:.2f} GB of "
                          "visibilities)"),
                   "facet_sides": [min(sides), max(sides)], "jobs": int(info["n_jobs"]),
                   "waves": int(info["n_waves"]), "support": int(info["support"]),
                   "graph_kernels_per_inversion": int(info["graph_kernels"]),
                   "job_samples": job_vis, "bind_s": round(bind_s, 2),
                   "plain_one_at_a_time_gvis_s": plain_value,
                   "batched_over_plain": value / plain_value,
                   "checks": checks, "datagen_s": round(gen_s, 1),
                   "direction_dependent_corrections": corrections,
                   "step": "one inversion of every facet x channel job (graph replay), device "
                           "visibilities in, device images out"},
        "clocks": clk,
        "e2e": {"value": job_vis / (e_ms * 1e-3) / 1e9, "unit": "Gvis/s",
                "h2d_bytes_per_step": int(h_vis.nbytes),
                "d2h_bytes_per_step": int(h_img.nbytes), "ms_per_step": e_ms},
        "gpu_launches": int(launches),
    }


def run_rowweights(args):
    """Raw-row weighting on the device: the imaging-weight grid (Grid +
    FinishGridding, once) and then, per step, CalculateWeights + ApplyWeights
    + CollapseData over every sample (wgpu_prepare_rows_device, inputs resident
    in HBM); e2e through wgpu_prepare_rows with pinned host buffers; the
    oracle's serial restatement timed on a row sample as the CPU baseline."""
    import ctypes as C
    import torch
    import oracle
    from wsclean_gb300 import _lib, synthetic
    from wsclean_gb300.weights import BRIGGS, ImageWeights, prepare_rows_device, row_weighting
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    d = synthetic.make_workload("wide8192", seed=5, with_model=False, n_t=75,
                                max_rows=args.max_rows)
    uvw, freq = d["uvw"], d["freq"]
    n_rows, n_chan, n_pol = uvw.shape[0], freq.size, 4
    n = n_rows * n_chan
    t_uvw = torch.as_tensor(uvw, device=dev)
    t_freq = torch.as_tensor(freq, device=dev)
    t_w = torch.as_tensor(d["weights"], device=dev)[:, :, None].expand(-1, -1, n_pol).contiguous()
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    t_vis = torch.randn((n_rows, n_chan, n_pol), generator=gen, dtype=torch.complex64,
                        device=dev)
    t_out = torch.empty((n_rows, n_chan), dtype=torch.complex64, device=dev)
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    W, dl = d["width"], d["dl"]
    iw = ImageWeights(BRIGGS, W, W, dl, dl, False, 1.0, 0.0)
    stream = torch.cuda.ExternalStream(iw.stream(), device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iw.grid_device(n_rows, n_chan, n_pol, t_uvw.data_ptr(), t_freq.data_ptr(), t_w.data_ptr())
    iw.FinishGridding()
    e1.record(stream)
    torch.cuda.synchronize()
    grid_ms = e0.elapsed_time(e1)
    settings = dict(polarization=_lib.POL_I)

    def step():
        return prepare_rows_device(iw, n_pol, n_rows, n_chan, t_uvw.data_ptr(), t_freq.data_ptr(),
                                   t_w.data_ptr(), t_out.data_ptr(), d_vis=t_vis.data_ptr(),
                                   **settings)

    for _ in range(args.warmup):
        sums = step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib_launches()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = _lib_launches() - l0
    ms = start.elapsed_time(end) / args.steps
    value = n / (ms * 1e-3) / 1e9

    # e2e: the host entry point with pinned host buffers (inputs up, prepared
    # visibilities down, every step)
    h_uvw = pinned_copy(t_uvw)
    h_w = pinned_copy(t_w)
    h_vis = pinned_copy(t_vis)
    h_out = torch.empty((n_rows, n_chan), dtype=torch.complex64, pin_memory=True)
    rw = row_weighting(**settings)
    hs = _lib.WeightSums()

    def e2e_step():
        _lib.check(_lib.lib().wgpu_prepare_rows(
            iw.handle, C.byref(rw), n_pol, n_rows, n_chan, h_uvw.data_ptr(), freq.ctypes.data,
            h_vis.data_ptr(), h_w.data_ptr(), None, None, h_out.data_ptr(), None, None,
            C.byref(hs)))

    for _ in range(2):
        e2e_step()
    w0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_ms = (time.perf_counter() - w0) * 1e3 / args.steps
    same = bool(torch.equal(h_out.to(dev), t_out))

    # CPU baseline and bit-exactness on a row sample: the oracle's serial
    # restatement with the device's finished grid
    ref = oracle.ImageWeights(BRIGGS, W, W, dl, dl, False, 1.0, 0.0)
    ref.grid[:] = iw.half_grid()
    n_s = min(n_rows, max(1, args.cpu_sample_rows))
    sw = t_w[:n_s].cpu().numpy()
    sv = t_vis[:n_s].cpu().numpy()
    c0 = time.perf_counter()
    ref_out = ref.prepare_rows(uvw[:n_s], freq, sw, sv, None, None, 0, 0.0, 0.0, 0,
                               _lib.POL_I)[0]
    cpu_s = time.perf_counter() - c0
    bit_exact = bool(np.array_equal(ref_out, t_out[:n_s].cpu().numpy()))
    cpu_value = n_s * n_chan / cpu_s / 1e9

    # roofline of prepare_rows_fast_kernel<4, true>: per sample 4 weights (16 B), 4
    # correlations (32 B), the imaging-weight cell (8 B) and the output (8 B),
    # plus 24 B of uvw per row
    alg_bytes = n * (16 + 32 + 8 + 8) + n_rows * 24 + n_chan * 8
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    h2d = h_uvw.numel() * 8 + freq.nbytes + h_w.numel() * 4 + h_vis.numel() * 8
    d2h = h_out.numel() * 8
    grid_bytes = n_rows * 24 + n * n_pol * 4 + n * n_pol * 16
    return {
        "metric": "Gsamples/s raw-row weighting (CalculateWeights + ApplyWeights + collapse)",
        "value": value, "unit": "Gsamples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT["rowweights"], "n_rows": n_rows, "n_chan": n_chan,
                   "n_samples": n, "correlations": n_pol,
                   "l2": (f"inputs larger than L2 ({(t_w.numel() * 4 + t_vis.numel() * 8) / 1e9:.1f}"
                          " GB of weights and visibilities per step)"),
                   "weight_grid": {"ms": grid_ms, "grid": f"{iw.Width()}x{iw.Height() // 2} doubles",
                                   "GB/s_algorithmic": grid_bytes / (grid_ms * 1e-3) / 1e9,
                                   "note": "Grid over every sample (atomic adds) + Briggs "
                                           "FinishGridding, once per weighting"},
                   "bit_exact_vs_oracle": bit_exact, "e2e_matches_device": same,
                   "weight_sums": sums, "datagen_s": round(gen_s, 1)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": _traffic("prepare_rows_fast_kernel")[0],
                     "traffic_unit": "GB per launch",
                     "traffic_source": _traffic("prepare_rows_fast_kernel")[1],
                     "kernel": "prepare_rows_fast_kernel<4, true> + exact pass",
                     "peak_source": peak_src,
                     "bytes_per_sample": 64},
        "cpu_baseline": {"value": cpu_value, "unit": "Gsamples/s", "cores": 1, "kind": "port",
                         "sample": f"first {n_s} rows x {n_chan} channels x 4 correlations, "
                                   "oracle serial restatement"},
        "clocks": clk,
        "e2e": {"value": n / (e2e_ms * 1e-3) / 1e9, "unit": "Gsamples/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
    }


def run_resample(args):
    """The boundary resampler: 8192^2 -> 5120^2 and 5120^2 -> 8192^2 per step,
    device buffers (wgpu_resample_device), the host entry point for e2e, and
    numpy's FFT restatement (the oracle) as the CPU baseline."""
    import torch
    from oracle import resample as ores
    from wsclean_gb300 import _lib
    from wsclean_gb300.resample import resample_device
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    big, small = 8192, 5120
    gen = torch.Generator(device=dev)
    gen.manual_seed(3)
    t_big = torch.randn((big, big), generator=gen, dtype=torch.float32, device=dev)
    t_small = torch.empty((small, small), dtype=torch.float32, device=dev)
    t_back = torch.empty((big, big), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step():
        resample_device(t_big.data_ptr(), big, big, t_small.data_ptr(), small, small, sp)
        resample_device(t_small.data_ptr(), small, small, t_back.data_ptr(), big, big, sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    l0 = _lib_launches()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = _lib_launches() - l0
    ms = start.elapsed_time(end) / args.steps
    # accuracy against the FP64 numpy restatement on this image
    h_big = t_big.cpu().numpy()
    c0 = time.perf_counter()
    ref_small = ores.resample(h_big, small, small)
    cpu_s = time.perf_counter() - c0
    rel_small = float(np.linalg.norm(t_small.cpu().numpy() - ref_small) / np.linalg.norm(ref_small))
    # e2e through the host entry point (pinned host buffers)
    from wsclean_gb300.resample import resample as resample_host
    p_big = pinned_copy(t_big)
    w0 = time.perf_counter()
    out_small = resample_host(p_big.numpy(), small, small)
    e2e_ms = (time.perf_counter() - w0) * 1e3
    same = bool(np.array_equal(out_small, t_small.cpu().numpy()))
    # one read and one write of the complex work image per transform pass
    def fft_bytes(n_elems, n):
        passes = 0
        m = n
        for r in (8, 4, 2, 3, 5, 7):
            while m % r == 0:
                passes += 1
                m //= r
        return passes * n_elems * 16
    def row_bytes(n_elems, n):
        # power-of-two rows of 512 to 8192 are transformed in shared memory:
        # one read and one write of the row for all passes
        if 512 <= n <= 8192 and n & (n - 1) == 0:
            return n_elems * 16
        return fft_bytes(n_elems, n)
    def leg_bytes(iw, ih, ow, oh):
        return (iw * ih * 4 + row_bytes(iw * ih, iw) + fft_bytes(ih * (iw // 2 + 1), ih) +
                fft_bytes(oh * (ow // 2 + 1), oh) + row_bytes(ow * oh, ow) + ow * oh * 4)
    alg = leg_bytes(big, big, small, small) + leg_bytes(small, small, big, big)
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = alg / (ms * 1e-3) / 1e9
    pixels = 2 * big * big + 2 * small * small  # input + output pixels of both legs
    return {
        "metric": "Gpixels/s boundary resampling (FFT method, in + out pixels)",
        "value": pixels / (ms * 1e-3) / 1e9, "unit": "Gpixels/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_TEXT["resample"], "sizes": [big, small],
                   "l2": "work images (512 MB complex) larger than L2",
                   "accuracy": {"rel_l2_vs_fp64_oracle": rel_small},
                   "e2e_matches_device": same},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": _traffic("fft_stage_kernel")[0],
                     "traffic_unit": "GB per radix-8 row pass",
                     "traffic_source": _traffic("fft_stage_kernel")[1],
                     "kernel": "fft_stage_kernel (all passes)",
                     "peak_source": peak_src,
                     "bytes": "one read + one write of the complex work image per pass "
                              "(per transform for rows done in shared memory)"},
        "cpu_baseline": {"value": (big * big + small * small) / cpu_s / 1e9,
                         "unit": "Gpixels/s", "cores": 1, "kind": "port",
                         "sample": "8192^2 -> 5120^2, numpy FFT (FP64) restatement"},
        "clocks": clk,
        "e2e": {"value": (big * big + small * small) / (e2e_ms * 1e-3) / 1e9, "unit": "Gpixels/s",
                "h2d_bytes_per_step": big * big * 4, "d2h_bytes_per_step": small * small * 4,
                "note": "one leg (8192^2 -> 5120^2) through wgpu_resample"},
        "gpu_launches": int(launches),
    }


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summaries
    (profiles/traffic.json), in GB, with where they come from."""
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tpath):
        return None, None
    t = json.load(open(tpath)).get(kernel)
    if not t:
        return None, None
    return float(t["traffic_bytes_per_launch"]) / 1e9, t["how"]


def _lib_launches():
    from wsclean_gb300 import _lib
    return _lib.lib().wgpu_kernel_launch_count()


# ---------------------------------------------------------------- serving ---
def run_serving(args, device_bytes):
    """Mixed-size request stream through the request server (scaled serving
    workload): the plain one-request-at-a-time path, the saturated server and
    Poisson arrivals at 0.8 of the saturated capacity."""
    from wsclean_gb300 import serving
    t0 = time.time()
    pool = serving.make_pool(args.serve_max_vis)
    pool_rows = pool["uvw"].shape[0]
    reqs = serving.make_stream(args.serve_requests, vis_range=(1e5, args.serve_max_vis),
                               side_range=(512, args.serve_max_side), pool_rows=pool_rows,
                               cycles=args.serve_cycles)
    gen_s = time.time() - t0
    keep = tuple(r["id"] for r in reqs[:6])
    planes = device_bytes / (2.0 * args.serve_slots)
    # the one-at-a-time path over the whole stream, or over a seeded sample of
    # it (the rates compare: both are samples of the same request distribution)
    n_plain = args.serve_plain_requests or len(reqs)
    if n_plain < len(reqs):
        pick = np.sort(np.random.default_rng(23).choice(len(reqs), n_plain, replace=False))
        plain_reqs = [reqs[i] for i in pick]
        keep = tuple(r["id"] for r in plain_reqs[:6])
    else:
        plain_reqs = reqs
    plain, kept_plain = serving.one_at_a_time(pool, plain_reqs, device_bytes, planes, keep)
    sat, kept_sat = serving.saturated(pool, reqs, device_bytes, planes, args.serve_slots, keep)
    rate = 0.8 * len(reqs) / sat["wall_s"]
    poi = serving.poisson(pool, reqs, device_bytes, planes, args.serve_slots, rate)
    # served (mixed) against one-at-a-time (alone) results of the same requests:
    # the runs can differ in the plane batch (the memory budget differs) and in
    # the order of the float atomic additions of split uv tiles
    same, same_eps = 0.0, 0.0
    eps_of = {r["id"]: r["eps"] for r in reqs}
    for i in keep:
        a, b = kept_plain[i], kept_sat[i]
        e = float(np.linalg.norm(b - a) / max(np.linalg.norm(a), 1e-30))
        same, same_eps = max(same, e), max(same_eps, e / eps_of[i])
    sides = [r["side"] for r in reqs]
    nvis = [r["rows"] * serving.N_CHAN for r in reqs]
    return {
        "workload": (f"{len(reqs)} requests ({sum(r['kind'] == 'invert' for r in reqs)} grid / "
                     f"{sum(r['kind'] == 'predict' for r in reqs)} degrid), image side log-uniform "
                     f"512-{args.serve_max_side} (drawn {min(sides)}-{max(sides)}), N_vis "
                     f"log-uniform 1e5-{args.serve_max_vis:.0e} (drawn {min(nvis)}-{max(nvis)}) "
                     f"from the 64-antenna 3 km array, eps 1e-4/1e-5, {args.serve_cycles} major "
                     f"cycles per request with state resident"),
        "slots": args.serve_slots, "device_budget_gb": device_bytes / 1e9,
        "one_at_a_time_requests": len(plain_reqs),
        "visibilities": serving.total_vis(reqs),
        "one_at_a_time": plain, "saturated": sat, "poisson": poi,
        "served_over_plain": sat["gvis_s"] / plain["gvis_s"],
        "alone_vs_mixed_max_rel_l2": same, "alone_vs_mixed_max_over_eps": same_eps,
        "alone_vs_mixed_tolerance": "relative L2 <= the request's epsilon",
        "datagen_s": round(gen_s, 1),
    }


# ---------------------------------------------------------- reference arm ---
def run_reference(args):
    """The CPU implementation of the path on the host cores: the reference's own
    w-gridder is ducc0, which is absent from the reference tree and cannot be
    built here, so the oracle's FP64 CPU w-gridder port is timed instead.  This
    arm loads only oracle code: the gridding plan (grid size, support, w
    planes) comes from oracle/plans.json, the planner's choices for this
    workload recorded beside the oracle, not from the product library.  Each
    step is one bounded sample (cpu_sample_step): both directions timed, the
    step's own wall time reported as ms_per_step, the rate extrapolated from
    the sample to the whole workload as value."""
    from oracle import make_plans
    from wsclean_gb300 import synthetic
    if args.workload not in make_plans.WORKLOADS:
        return {"impl": "reference", "unavailable": f"no recorded plan for {args.workload}"}
    d = synthetic.make_workload(args.workload, seed=2, max_rows=args.max_rows, with_model=False)
    n_rows, n_chan = d["uvw"].shape[0], d["freq"].size
    plan = make_plans.load(args.workload)

    def vis_rows(rows):
        # random unit-variance visibilities on the non-flagged samples
        rng = np.random.default_rng(int(rows[0]) + 9)
        w = d["weights"][rows]
        v = rng.standard_normal(w.shape) + 1j * rng.standard_normal(w.shape)
        return np.where(w > 0, v, 0).astype(np.complex64)

    d["n_gridded"] = int(np.count_nonzero(d["weights"]))
    walls, rates, texts = [], [], []
    w_start = time.perf_counter()
    for i in range(args.warmup + args.steps):
        wall, full, text = cpu_sample_step(d, plan, vis_rows, args.ref_baselines,
                                           args.ref_plane_fraction, seed=100 + i)
        if i >= args.warmup:
            walls.append(wall)
            rates.append(n_rows * n_chan / full / 1e9)
            texts.append(text)
    timed_s = float(np.sum(walls))
    v = float(np.median(rates))
    ms = timed_s * 1e3 / args.steps
    cores = os.cpu_count()
    cb = {"value": v, "unit": "Gvis/s", "cores": cores, "kind": "port",
          "sample": (f"per step: {texts[-1]}; value = median over the {args.steps} timed steps "
                     "of the extrapolated rate")}
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gvis/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD_TEXT.get(args.workload, args.workload),
                       "n_vis": n_rows * n_chan, "n_vis_gridded": d["n_gridded"],
                       "plan": {k: plan[k] for k in ("nu", "support", "sigma", "n_planes")},
                       "plan_source": "oracle/plans.json (recorded planner output; the product "
                                      "library is not loaded by this arm)",
                       "timed_region_s": round(timed_s, 2),
                       "arm_wall_s": round(time.perf_counter() - w_start, 2),
                       "note": "ducc0 (the reference's wgridder) is absent from the reference "
                               "tree; the oracle's FP64 CPU w-gridder port is timed instead. "
                               "ms_per_step is the measured time of one sample step; value is "
                               "the workload rate extrapolated from the samples"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Gvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wgpu", choices=["wgpu", "reference"])
    ap.add_argument("--workload", default="wide8192", choices=sorted(WORKLOAD_TEXT))
    ap.add_argument("--max-rows", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-bound", action="store_true",
                    help="skip the major cycles on a bound visibility set")
    ap.add_argument("--tune-bound", action="store_true",
                    help="also run the bound major cycles on a tuning gridder")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the full-data error against the FP64 direct transform")
    ap.add_argument("--cpu-sample-rows", type=int, default=200000,
                    help="rows of the raw-row weighting CPU sample")
    ap.add_argument("--cpu-baselines", type=int, default=200,
                    help="baselines (all time steps) in the CPU baseline's sample")
    ap.add_argument("--cpu-plane-fraction", type=float, default=0.25,
                    help="fraction of one plane pass per direction in the CPU baseline")
    ap.add_argument("--ref-baselines", type=int, default=48,
                    help="baselines per step of the reference arm's CPU sample")
    ap.add_argument("--ref-plane-fraction", type=float, default=1.0 / 16,
                    help="fraction of one plane pass per direction per reference step")
    ap.add_argument("--facet-corrections", action="store_true",
                    help="also time the facet batch with per-facet full-Jones corrections")
    ap.add_argument("--facet-times", type=int, default=6200,
                    help="time steps of the facet workload (6200 in the full workload)")
    ap.add_argument("--facet-resident-times", type=int, default=1000,
                    help="above this many time steps the facet workload binds one "
                         "output-channel group at a time (the jobs' records do not fit)")
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests in the serving stream (0 skips it)")
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-cycles", type=int, default=5)
    ap.add_argument("--serve-max-vis", type=float, default=1e7)
    ap.add_argument("--serve-max-side", type=int, default=4096)
    ap.add_argument("--serve-plain-requests", type=int, default=0,
                    help="requests of the stream timed one at a time (0: all of them)")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the serving stream and print its JSON")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu DRAM bytes per launch of the dominant kernel, if captured")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference" and args.workload in ("rowweights", "resample"):
        print(json.dumps({"impl": "reference", "unavailable": "this workload has no "
                          "reference arm; its CPU baseline is the cpu_baseline key"}), flush=True)
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.workload == "facets":
        print(json.dumps(run_facets(args)), flush=True)
        return
    if args.workload == "fullpol4096":
        print(json.dumps(run_fullpol(args)), flush=True)
        return
    if args.workload == "rowweights":
        print(json.dumps(run_rowweights(args)), flush=True)
        return
    if args.workload == "resample":
        print(json.dumps(run_resample(args)), flush=True)
        return
    if args.serve_only:
        import torch
        torch.cuda.set_device(local)
        free_b, _ = torch.cuda.mem_get_info()
        print(json.dumps(run_serving(args, 0.7 * free_b)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    res = run_gpu(args, rank, world, local)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
