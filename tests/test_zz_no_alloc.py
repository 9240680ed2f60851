"""The allocation-free bucketing entry point (wgpu_bucket_noalloc).

It serves callers that cannot allocate device memory while they call the
library (a host owning all device memory through its own pool, or a pipeline
that must not trigger the synchronisation cudaMalloc/cudaFree can cause): the
caller passes device inputs and outputs and the scratch lives in a static
device array.  Its results must equal those of the allocating bucketing entry
point (wgpu_bucket_debug) bit for bit, on consecutive calls that reuse the
static scratch.  Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import bucket_debug

pytestmark = pytest.mark.gpu
LIGHT = 299792458.0


def _plan(uvw, freq, vis, W, dl):
    wl = (uvw[:, 2:3] * (freq / LIGHT)[None, :])
    if vis is not None:
        wl = wl[vis != 0]
    return _lib.make_plan(width=W, height=W, dl=dl, dm=dl, epsilon=1e-4,
                          w_min=float(wl.min()), w_max=float(wl.max()), n_vis=int(wl.size))


def _noalloc(plan, uvw, freq, vis, skip_zero):
    import torch
    dev = torch.device("cuda", 0)
    n_rows, n_chan = uvw.shape[0], freq.size
    n = n_rows * n_chan
    d_uvw = torch.as_tensor(np.ascontiguousarray(uvw), device=dev)
    d_freq = torch.as_tensor(np.ascontiguousarray(freq), device=dev)
    d_vis = torch.as_tensor(np.ascontiguousarray(vis, np.complex64), device=dev) \
        if vis is not None else None
    n_keys = (plan.nu // plan.tile) * (plan.nv // plan.tile) * 4 * plan.n_planes
    d_rec = torch.zeros((n, 8), dtype=torch.int32, device=dev)
    d_perm = torch.zeros(n, dtype=torch.int32, device=dev)
    d_off = torch.zeros(n_keys + 1, dtype=torch.int32, device=dev)
    n_out = C.c_int64()
    torch.cuda.synchronize()
    _lib.check(_lib.lib().wgpu_bucket_noalloc(
        C.byref(plan), n_rows, n_chan, d_uvw.data_ptr(), d_freq.data_ptr(),
        d_vis.data_ptr() if d_vis is not None else None, 1 if skip_zero else 0,
        d_rec.data_ptr(), d_perm.data_ptr(), d_off.data_ptr(), None, C.byref(n_out)))
    torch.cuda.synchronize()
    k = n_out.value
    rec = d_rec[:k].cpu().numpy()
    f = rec.view(np.float32)
    return dict(perm=d_perm[:k].cpu().numpy().view(np.uint32), fu=f[:, 2], fv=f[:, 3],
                fw=f[:, 4], iu=rec[:, 5], iv=rec[:, 6], ip=rec[:, 7],
                offsets=d_off.cpu().numpy().view(np.uint32))


def test_noalloc_bucketing_matches_allocating_entry_point(wgpu_lib):
    cases = [
        dict(W=256, dl=3e-4, rows=3000, chan=8, w_scale=2.0, zero=0.2, seed=31, inv=True),
        dict(W=192, dl=4e-4, rows=5000, chan=16, w_scale=1.0, zero=0.0, seed=32, inv=False),
    ]
    for case in cases:  # two calls in a row reuse the static scratch
        uvw, freq, vis = synthetic.random_points(case["rows"], case["chan"], case["W"], case["dl"],
                                                 case["seed"], w_scale=case["w_scale"],
                                                 frac_zero=case["zero"])
        v = vis if case["inv"] else None
        plan = _plan(uvw, freq, v, case["W"], case["dl"])
        got = _noalloc(plan, uvw, freq, v, case["inv"])
        ref = bucket_debug(plan, uvw.shape[0], freq.size, uvw, freq, v, case["inv"])
        for k in ("perm", "iu", "iv", "ip", "fu", "fv", "fw", "offsets"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_noalloc_rejects_oversize_requests(wgpu_lib):
    import torch
    n_rows, n_chan = (_lib.NOALLOC_MAX_VISIBILITIES // 4) + 1, 4
    plan = _lib.make_plan(width=64, height=64, dl=1e-3, dm=1e-3, epsilon=1e-4, w_min=0.0,
                          w_max=0.0, n_vis=1)
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    n_out = C.c_int64()
    st = _lib.lib().wgpu_bucket_noalloc(C.byref(plan), n_rows, n_chan, d.data_ptr(),
                                        d.data_ptr(), d.data_ptr(), 0, d.data_ptr(),
                                        d.data_ptr(), d.data_ptr(), None, C.byref(n_out))
    assert st == _lib.WGPU_ERR_INVALID
    assert b"at most" in _lib.lib().wgpu_last_error()
    # sizes whose product wraps around 64 bits are refused before it is formed
    for rows, chans in (((1 << 62) + 1, 4), (1 << 33, 1 << 31), (3, _lib.NOALLOC_MAX_CHANNELS + 1)):
        st = _lib.lib().wgpu_bucket_noalloc(C.byref(plan), rows, chans, d.data_ptr(),
                                            d.data_ptr(), d.data_ptr(), 0, d.data_ptr(),
                                            d.data_ptr(), d.data_ptr(), None, C.byref(n_out))
        assert st == _lib.WGPU_ERR_INVALID
        assert b"at most" in _lib.lib().wgpu_last_error()


def test_noalloc_bucketing_at_the_sample_limit(wgpu_lib):
    """Exactly WGPU_NOALLOC_MAX_VISIBILITIES samples, twice in a row: the
    largest request the static scratch takes."""
    n_chan = 16
    n_rows = _lib.NOALLOC_MAX_VISIBILITIES // n_chan
    uvw, freq, vis = synthetic.random_points(n_rows, n_chan, 512, 1e-4, 33, w_scale=1.5,
                                             frac_zero=0.1)
    assert uvw.shape[0] * freq.size == _lib.NOALLOC_MAX_VISIBILITIES
    plan = _plan(uvw, freq, vis, 512, 1e-4)
    ref = bucket_debug(plan, uvw.shape[0], freq.size, uvw, freq, vis, True)
    for _ in range(2):
        got = _noalloc(plan, uvw, freq, vis, True)
        for k in ("perm", "iu", "iv", "ip", "fu", "fv", "fw", "offsets"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
