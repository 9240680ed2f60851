"""Python mirror of the facet batch (wgpu_facets_* in include/wgpu.h).

One visibility set imaged into many facets for several output-channel groups,
as WSClean's batch inversion with shared reads does
(gridding/msgriddermanager.cpp:118-396), with every wave of jobs gridded in one
persistent launch and the whole inversion replayed from one CUDA graph.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, lib


class FacetBatch:
    """facets: list of dicts (width, height, dl, dm, l_shift, m_shift);
    channel_groups: increasing channel boundaries (n_groups + 1)."""

    def __init__(self, facets, channel_groups, epsilon=1e-4, plane_budget_bytes=0.0):
        arr = (_lib.Facet * len(facets))()
        for a, f in zip(arr, facets):
            a.width, a.height = int(f["width"]), int(f["height"])
            a.pixel_size_x, a.pixel_size_y = float(f["dl"]), float(f.get("dm", f["dl"]))
            a.l_shift, a.m_shift = float(f.get("l_shift", 0.0)), float(f.get("m_shift", 0.0))
        groups = (C.c_size_t * len(channel_groups))(*[int(c) for c in channel_groups])
        h = C.c_void_p()
        check(lib().wgpu_facets_create(arr, len(facets), groups, len(channel_groups) - 1,
                                       float(epsilon), float(plane_budget_bytes), C.byref(h)))
        self._h = h
        self.facets = [dict(f) for f in facets]
        self.n_groups = len(channel_groups) - 1

    def close(self):
        if getattr(self, "_h", None):
            lib().wgpu_facets_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind(self, uvw, freq, corrected=False):
        """Binds the rows; corrected=True keeps one corrected visibility buffer
        per facet for invert_corrected (direction-dependent gains)."""
        self._uvw = np.ascontiguousarray(uvw, dtype=np.float64).reshape(-1, 3)
        self._freq = np.ascontiguousarray(freq, dtype=np.float64)
        fn = lib().wgpu_facets_bind_corrected if corrected else lib().wgpu_facets_bind
        check(fn(self._h, self._uvw.shape[0], self._freq.size, self._uvw.ctypes.data,
                 self._freq.ctypes.data))

    def info(self):
        i = _lib.FacetsInfo()
        check(lib().wgpu_facets_info(self._h, C.byref(i)))
        out = {k: getattr(i, k) for k, _ in i._fields_}
        out["bind_ms"] = list(i.bind_ms)
        return out

    def job_plan(self, job):
        p = _lib.Plan()
        check(lib().wgpu_facets_job_plan(self._h, int(job), C.byref(p)))
        return p

    def invert(self, vis):
        """Dirty images of every job: list indexed group * n_facets + facet,
        each (height, width) float32."""
        vis = np.ascontiguousarray(vis, dtype=np.complex64)
        out = np.empty(int(self.info()["image_elems"]), np.float32)
        check(lib().wgpu_facets_invert(self._h, vis.ctypes.data, out.ctypes.data))
        return self._split(out)

    def invert_corrected(self, mode, vis, antennas, time_offsets, solutions, nparms, n_times,
                         n_antenna, polarization=_lib.POL_I):
        """Dirty images with each facet's conjugated gains applied on the
        device: vis (rows, chans, n_pol) uncorrected, solutions (n_facets,
        n_times, chans, n_antenna, nparms) complex64; bind(corrected=True)
        first."""
        if isinstance(mode, str):
            mode = {"xx": 0, "yy": 1, "trace": 2, "diagonal": 3, "full": 4}[mode]
        vis = np.ascontiguousarray(vis, dtype=np.complex64)
        n_pol = vis.size // (self._uvw.shape[0] * self._freq.size)
        ant = np.ascontiguousarray(antennas, dtype=np.uint64)
        tof = np.ascontiguousarray(time_offsets, dtype=np.uint64)
        sol = np.ascontiguousarray(solutions, dtype=np.complex64)
        assert sol.size == len(self.facets) * n_times * self._freq.size * n_antenna * nparms
        out = np.empty(int(self.info()["image_elems"]), np.float32)
        check(lib().wgpu_facets_invert_corrected(self._h, int(mode), n_pol, vis.ctypes.data,
                                                 ant.ctypes.data, tof.ctypes.data,
                                                 sol.ctypes.data, nparms, n_times, n_antenna,
                                                 int(polarization), out.ctypes.data))
        return self._split(out)

    def _split(self, out):
        images, o = [], 0
        for _ in range(self.n_groups):
            for f in self.facets:
                n = f["width"] * f["height"]
                images.append(out[o:o + n].reshape(f["height"], f["width"]))
                o += n
        return images

    def invert_device(self, d_vis, d_images):
        check(lib().wgpu_facets_invert_device(self._h, int(d_vis), int(d_images)))

    def stream(self):
        return lib().wgpu_facets_stream(self._h)
