"""Python mirror of the request server (wgpu_server_* in include/wgpu.h).

The server replaces GriddingTaskManager / ThreadedScheduler on the gridding
path (scheduling/griddingtaskmanager.cpp:26-103, threadedscheduler.cpp:12-228):
requests are queued, admitted by device memory, run concurrently on worker
slots with their own CUDA streams, and waited for by ticket.  Requests with the
same non-zero session keep their bound visibility set on the device across
major cycles.

The numpy buffers of a request are kept alive by the returned ticket object
until ``wait`` returns.
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, lib


@dataclass
class Ticket:
    id: int
    kind: int
    keep: list = field(default_factory=list)  # buffers the request points into
    out: np.ndarray = None                     # image (inversion) or visibilities
    latency_ms: float = None
    queue_ms: float = None


class GriddingServer:
    """Continuous-batching request loop on one GPU.

    device_bytes caps the device memory of admitted requests plus resident
    sessions; max_active is the number of worker slots (concurrent requests);
    plane_budget_bytes caps each plan's w-plane batch (0 = device_bytes /
    (2 * max_active)).
    """

    def __init__(self, device_bytes, max_active=4, plane_budget_bytes=0.0):
        h = C.c_void_p()
        check(lib().wgpu_server_create(float(device_bytes), int(max_active),
                                       float(plane_budget_bytes), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().wgpu_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _geometry(req, geom):
        (req.width, req.height, req.width_t, req.height_t, req.pixel_size_x,
         req.pixel_size_y, req.l_shift, req.m_shift, req.epsilon) = (
            int(geom["width"]), int(geom["height"]), int(geom.get("width_t", geom["width"])),
            int(geom.get("height_t", geom["height"])), float(geom["dl"]), float(geom["dm"]),
            float(geom.get("l_shift", 0.0)), float(geom.get("m_shift", 0.0)),
            float(geom["epsilon"]))

    def _submit(self, kind, geom, uvw, freq, session, mask, keep):
        req = _lib.Request()
        req.kind = kind
        req.session = int(session)
        self._geometry(req, geom)
        uvw = np.ascontiguousarray(uvw, dtype=np.float64).reshape(-1, 3)
        freq = np.ascontiguousarray(freq, dtype=np.float64)
        req.n_rows, req.n_chan = uvw.shape[0], freq.shape[0]
        req.uvw, req.freq = uvw.ctypes.data, freq.ctypes.data
        keep += [uvw, freq]
        if mask is not None:
            mask = np.ascontiguousarray(mask, dtype=np.uint8)
            req.mask = mask.ctypes.data
            keep.append(mask)
        return req

    @staticmethod
    def _out(out, n, dtype):
        if out is None:
            return np.empty(n, dtype=dtype)
        if out.dtype != dtype or out.size != n or not out.flags.c_contiguous:
            raise ValueError(f"output buffer must be {n} contiguous {np.dtype(dtype).name}")
        return out.reshape(-1)

    def submit_invert(self, geom, uvw, freq, vis, image_factor=1.0, session=0, mask=None,
                      out=None):
        """Queues InitializeInversion + AddInversionData + FinalizeImage + RealImage.
        ``out`` (width * height float32) may be passed to reuse a buffer."""
        keep = []
        req = self._submit(_lib.REQUEST_INVERT, geom, uvw, freq, session, mask, keep)
        vis = np.ascontiguousarray(vis, dtype=np.complex64)
        out = self._out(out, req.width * req.height, np.float32)
        req.vis, req.image_factor, req.image_out = vis.ctypes.data, float(image_factor), \
            out.ctypes.data
        keep += [vis, out]
        return self._enqueue(req, keep, out)

    def submit_predict(self, geom, uvw, freq, model, session=0, mask=None, out=None):
        """Queues InitializePrediction + PredictVisibilities.  ``out`` (n_rows *
        n_chan complex64) may be passed to reuse a buffer."""
        keep = []
        req = self._submit(_lib.REQUEST_PREDICT, geom, uvw, freq, session, mask, keep)
        model = np.ascontiguousarray(model, dtype=np.float32)
        out = self._out(out, req.n_rows * req.n_chan, np.complex64)
        req.model, req.vis_out = model.ctypes.data, out.ctypes.data
        keep += [model, out]
        return self._enqueue(req, keep, out)

    def _enqueue(self, req, keep, out):
        tid = C.c_uint64()
        check(lib().wgpu_server_submit(self._h, C.byref(req), C.byref(tid)))
        return Ticket(tid.value, req.kind, keep, out)

    def wait(self, ticket):
        """Blocks until the request is done; returns its image or visibilities."""
        lat, q = C.c_double(), C.c_double()
        st = lib().wgpu_server_wait(self._h, ticket.id, C.byref(lat), C.byref(q))
        ticket.latency_ms, ticket.queue_ms = lat.value, q.value
        ticket.keep = []
        check(st)
        return ticket.out

    def close_session(self, session):
        check(lib().wgpu_server_close_session(self._h, int(session)))

    def stats(self):
        s = _lib.ServerStats()
        check(lib().wgpu_server_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}
