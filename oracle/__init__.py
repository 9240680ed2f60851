"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this package, as the checker.  See wgpu_oracle.h for what each
function restates and its parity status.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class OraclePlan(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("width", "height", "nu", "nv", "support", "tile",
                                         "n_planes")] + \
               [(n, C.c_double) for n in ("beta", "dl", "dm", "l_shift", "m_shift", "w0", "dw",
                                          "nm1_center")]


_lib = None


REF_FFTSIZE = os.path.join(HERE, "_ref", "libref_fftsize.so")
CUDA_LIB_PATH = os.path.join(HERE, "_build", "liboracle_cuda.so")
# The reference tree, read only to compile its header-only code into
# oracle/_ref (absent on machines that only run the prebuilt files).
REFERENCE_TREE = os.environ.get("WGPU_REFERENCE_TREE", "/root/reference")


def _nvcc():
    import shutil
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build():
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    nvcc = _nvcc()
    if nvcc is not None:
        r = subprocess.run(["make", "-C", HERE, "cuda", f"NVCC={nvcc}"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle CUDA twin build failed:\n" + r.stdout + r.stderr)
    # the reference's own header-only code, where the reference tree exists
    if os.path.isdir(REFERENCE_TREE):
        subprocess.run(["make", "-C", HERE, "ref", f"REFERENCE={REFERENCE_TREE}"],
                       capture_output=True, text=True)
    return LIB_PATH


def ref_calculate_fft_size():
    """The reference's CalculateFFTSize compiled from its own header
    (oracle/_ref), or None where the reference tree was absent at build."""
    if not os.path.exists(REF_FFTSIZE):
        return None
    L = C.CDLL(REF_FFTSIZE)
    L.ref_calculate_fft_size.argtypes = [C.c_size_t, C.c_double, C.c_double,
                                         C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]

    def fn(size, pixel_scale, beam_size):
        mn, opt = C.c_size_t(), C.c_size_t()
        L.ref_calculate_fft_size(size, pixel_scale, beam_size, C.byref(mn), C.byref(opt))
        return mn.value, opt.value
    return fn


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P, SZ, D, I = C.c_void_p, C.c_size_t, C.c_double, C.c_int
        L.oracle_dft_invert.argtypes = [SZ, SZ, P, P, P, SZ, SZ, D, D, D, D, P, SZ, I, P]
        L.oracle_dft_predict.argtypes = [SZ, SZ, P, P, P, SZ, SZ, D, D, D, D, P, SZ, I, P]
        L.oracle_bucket.restype = C.c_int64
        L.oracle_bucket.argtypes = [C.POINTER(OraclePlan), SZ, SZ, P, P, P, I, P, P, P, P, P,
                                    P, P, P, P]
        L.oracle_wgrid_invert.argtypes = [C.POINTER(OraclePlan), SZ, SZ, P, P, P, I, P]
        L.oracle_wgrid_predict.argtypes = [C.POINTER(OraclePlan), SZ, SZ, P, P, P, I, P]
        L.oracle_wgrid_time_parts.restype = D
        L.oracle_wgrid_time_parts.argtypes = [C.POINTER(OraclePlan), SZ, SZ, P, P, P, I, D,
                                              C.POINTER(D)]
        L.oracle_wgrid_time_predict_parts.restype = D
        L.oracle_wgrid_time_predict_parts.argtypes = [C.POINTER(OraclePlan), SZ, SZ, P, P, P,
                                                      I, D, C.POINTER(D)]
        L.oracle_es_kernel.restype = D
        L.oracle_es_kernel.argtypes = [D, D]
        L.oracle_es_fourier.restype = D
        L.oracle_es_fourier.argtypes = [D, I, D]
        L.oracle_apply_gains.restype = I
        L.oracle_apply_gains.argtypes = [I, SZ, SZ, SZ, P, P, P, P, SZ, SZ, I, P]
        L.oracle_forward_gains.restype = I
        L.oracle_forward_gains.argtypes = [I, SZ, SZ, SZ, P, P, P, P, SZ, SZ, I, P]
        L.oracle_apply_conjugated_gain.argtypes = [I, P, P, P]
        L.oracle_correction_matrix_add.argtypes = [P, P, D, P]
        L.oracle_apply_gain.argtypes = [I, P, P, P]
        I64 = C.c_int64
        L.oracle_weights_dims.argtypes = [SZ, SZ, D, C.POINTER(I64), C.POINTER(I64)]
        L.oracle_weights_grid.restype = D
        L.oracle_weights_grid.argtypes = [P, I64, I64, D, D, I, SZ, SZ, SZ, P, P, P]
        L.oracle_weights_finish.argtypes = [P, I64, I64, I, D, D]
        L.oracle_weights_taper.argtypes = [P, I64, I64, D, D, I, D, D]
        L.oracle_weights_mirror.argtypes = [P, I64, I64, P]
        L.oracle_weights_sample.argtypes = [P, I64, I64, D, D, SZ, P, P, P]
        L.oracle_prepare_rows.argtypes = [P, I64, I64, D, D, I, D, D, I, I, I, SZ, SZ, SZ, P, P,
                                          P, P, P, P, P, P, P, P]
        L.oracle_prepare_rows_corrected.argtypes = [P, I64, I64, D, D, I, D, D, I, I, I, SZ, SZ,
                                                    SZ, P, P, P, P, P, P, P, P, P, P, I, P, P, P,
                                                    SZ, SZ, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def to_oracle_plan(plan):
    """From a product plan (wsclean_gb300._lib.Plan or dict) to the oracle's."""
    get = (lambda k: plan[k]) if isinstance(plan, dict) else (lambda k: getattr(plan, k))
    o = OraclePlan()
    for k in ("width", "height", "nu", "nv", "support", "tile", "n_planes"):
        setattr(o, k, int(get(k)))
    for k in ("beta", "dl", "dm", "l_shift", "m_shift", "w0", "dw"):
        setattr(o, k, float(get(k)))
    o.nm1_center = float(get("nm1_center"))
    return o


def dft_invert(uvw, freq, vis, width, height, dl, dm, l_shift=0.0, m_shift=0.0, pixels=None,
               n_threads=0):
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    vis = np.ascontiguousarray(vis, np.complex64)
    if pixels is None:
        pixels = np.arange(width * height, dtype=np.int64)
    pixels = np.ascontiguousarray(pixels, np.int64)
    out = np.zeros(pixels.size, np.float64)
    lib().oracle_dft_invert(uvw.shape[0], freq.size, _p(uvw), _p(freq), _p(vis), width, height,
                            dl, dm, l_shift, m_shift, _p(pixels), pixels.size, n_threads,
                            _p(out))
    return out


def dft_predict(uvw, freq, image, width, height, dl, dm, l_shift=0.0, m_shift=0.0,
                vis_index=None, n_threads=0):
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    image = np.ascontiguousarray(image, np.float64).ravel()
    n = uvw.shape[0] * freq.size
    if vis_index is None:
        vis_index = np.arange(n, dtype=np.int64)
    vis_index = np.ascontiguousarray(vis_index, np.int64)
    out = np.zeros(2 * vis_index.size, np.float64)
    lib().oracle_dft_predict(uvw.shape[0], freq.size, _p(uvw), _p(freq), _p(image), width,
                             height, dl, dm, l_shift, m_shift, _p(vis_index), vis_index.size,
                             n_threads, _p(out))
    return out[0::2] + 1j * out[1::2]


_cuda_lib = None


def cuda_lib():
    """The FP64 direct-transform twin for the GPU (oracle/dft_cuda.cu)."""
    global _cuda_lib
    if _cuda_lib is None:
        if not os.path.exists(CUDA_LIB_PATH):
            build()
        L = C.CDLL(CUDA_LIB_PATH)
        P, SZ, D = C.c_void_p, C.c_size_t, C.c_double
        L.oracle_cuda_last_error.restype = C.c_char_p
        L.oracle_cuda_dft_invert.restype = C.c_int
        L.oracle_cuda_dft_invert.argtypes = [SZ, SZ, P, P, P, SZ, SZ, D, D, D, D, P, SZ, P, P]
        L.oracle_cuda_dft_predict.restype = C.c_int
        L.oracle_cuda_dft_predict.argtypes = [SZ, SZ, P, P, P, SZ, SZ, D, D, D, D, P, P, P, P,
                                              P]
        _cuda_lib = L
    return _cuda_lib


def _ptr(a, dtype=None):
    """Address of a numpy array (made contiguous in `dtype`) or of a torch tensor
    (host or device; used in place).  Returns (address, keep-alive object)."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr(), a
    arr = np.ascontiguousarray(a, dtype) if dtype is not None else np.ascontiguousarray(a)
    return arr.ctypes.data, arr


def _cuda_check(r):
    if r != 0:
        raise RuntimeError("oracle CUDA twin: " + cuda_lib().oracle_cuda_last_error().decode())


def cuda_dft_invert(uvw, freq, vis, width, height, dl, dm, l_shift=0.0, m_shift=0.0,
                    pixels=None, n_rows=None, n_chan=None, stream=0):
    """oracle_dft_invert on the GPU in FP64 (every row, selected pixels).  uvw
    and vis may be numpy arrays or torch tensors (host or device)."""
    freq = np.ascontiguousarray(freq, np.float64)
    n_chan = freq.size if n_chan is None else n_chan
    n_rows = uvw.shape[0] if n_rows is None else n_rows
    if pixels is None:
        pixels = np.arange(width * height, dtype=np.int64)
    pixels = np.ascontiguousarray(pixels, np.int64)
    pu, ku = _ptr(uvw, np.float64)
    pv, kv = _ptr(vis, np.complex64)
    out = np.zeros(pixels.size, np.float64)
    _cuda_check(cuda_lib().oracle_cuda_dft_invert(n_rows, n_chan, pu, _p(freq), pv, width,
                                                  height, dl, dm, l_shift, m_shift, _p(pixels),
                                                  pixels.size, _p(out), stream))
    return out


def cuda_dft_predict(uvw, freq, image, width, height, dl, dm, l_shift=0.0, m_shift=0.0,
                     mask=None, pred=None, want_values=False, n_rows=None, stream=0):
    """oracle_dft_predict on the GPU in FP64 at every sample.  Returns
    (values or None, sum |pred - ref|^2, sum |ref|^2) with the sums over the
    samples where mask != 0 (every sample without a mask).  uvw, mask and pred
    may be numpy arrays or torch tensors (host or device)."""
    freq = np.ascontiguousarray(freq, np.float64)
    image = np.ascontiguousarray(image, np.float64).ravel()
    n_rows = uvw.shape[0] if n_rows is None else n_rows
    pu, ku = _ptr(uvw, np.float64)
    pm, km = _ptr(mask, np.uint8)
    pp, kp = _ptr(pred, np.complex64)
    vals = np.zeros(n_rows * freq.size, np.complex128) if want_values else None
    sums = np.zeros(2, np.float64)
    _cuda_check(cuda_lib().oracle_cuda_dft_predict(n_rows, freq.size, pu, _p(freq), _p(image),
                                                   width, height, dl, dm, l_shift, m_shift, pm,
                                                   pp, None if vals is None else _p(vals),
                                                   _p(sums), stream))
    return vals, float(sums[0]), float(sums[1])


def bucket(plan, uvw, freq, vis, skip_zero):
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    vis = None if vis is None else np.ascontiguousarray(vis, np.complex64)
    op = to_oracle_plan(plan)
    n = uvw.shape[0] * freq.size
    perm = np.zeros(n, np.uint32)
    key = np.zeros(n, np.int64)
    iu, iv, ip = (np.zeros(n, np.int32) for _ in range(3))
    fu, fv, fw = (np.zeros(n, np.float32) for _ in range(3))
    n_keys = (op.nu // op.tile) * (op.nv // op.tile) * 4 * op.n_planes
    off = np.zeros(n_keys + 1, np.int64)
    k = lib().oracle_bucket(C.byref(op), uvw.shape[0], freq.size, _p(uvw), _p(freq), _p(vis),
                            1 if skip_zero else 0, _p(perm), _p(key), _p(iu), _p(iv), _p(ip),
                            _p(fu), _p(fv), _p(fw), _p(off))
    return dict(perm=perm[:k], key=key[:k], iu=iu[:k], iv=iv[:k], ip=ip[:k], fu=fu[:k],
                fv=fv[:k], fw=fw[:k], offsets=off)


def wgrid_invert(plan, uvw, freq, vis, n_threads=0):
    op = to_oracle_plan(plan)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    vis = np.ascontiguousarray(vis, np.complex64)
    out = np.zeros(op.width * op.height, np.float64)
    r = lib().oracle_wgrid_invert(C.byref(op), uvw.shape[0], freq.size, _p(uvw), _p(freq),
                                  _p(vis), n_threads, _p(out))
    if r != 0:
        raise RuntimeError(f"oracle_wgrid_invert failed ({r})")
    return out


def wgrid_predict(plan, uvw, freq, image, n_threads=0):
    op = to_oracle_plan(plan)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    image = np.ascontiguousarray(image, np.float64).ravel()
    out = np.zeros(2 * uvw.shape[0] * freq.size, np.float64)
    r = lib().oracle_wgrid_predict(C.byref(op), uvw.shape[0], freq.size, _p(uvw), _p(freq),
                                   _p(image), n_threads, _p(out))
    if r != 0:
        raise RuntimeError(f"oracle_wgrid_predict failed ({r})")
    return out[0::2] + 1j * out[1::2]


def wgrid_time_parts(plan, uvw, freq, vis, n_threads=0, plane_fraction=1.0):
    """Seconds of the CPU inversion's spreading of the samples with vis != 0
    over all their planes, and of plane_fraction of one plane pass."""
    op = to_oracle_plan(plan)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    vis = np.ascontiguousarray(vis, np.complex64)
    ps = C.c_double()
    t = lib().oracle_wgrid_time_parts(C.byref(op), uvw.shape[0], freq.size, _p(uvw), _p(freq),
                                      _p(vis), n_threads, float(plane_fraction), C.byref(ps))
    return t, ps.value


def wgrid_time_predict_parts(plan, uvw, freq, vis, n_threads=0, plane_fraction=1.0):
    """Seconds of the CPU prediction's interpolation of the samples with
    vis != 0 over all their planes, and of plane_fraction of one plane pass."""
    op = to_oracle_plan(plan)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    vis = np.ascontiguousarray(vis, np.complex64)
    ps = C.c_double()
    t = lib().oracle_wgrid_time_predict_parts(C.byref(op), uvw.shape[0], freq.size, _p(uvw),
                                              _p(freq), _p(vis), n_threads,
                                              float(plane_fraction), C.byref(ps))
    return t, ps.value


def es_kernel(beta, z):
    return lib().oracle_es_kernel(beta, z)


def es_fourier(beta, support, f):
    return lib().oracle_es_fourier(beta, support, f)


def apply_gains(mode, n_pol, vis, antenna_pairs, time_offsets, solutions, nparms, n_ant,
                polarization=0):
    vis = np.ascontiguousarray(vis, np.complex64)
    n_rows, n_chan = vis.shape[0], vis.shape[1]
    ant = np.ascontiguousarray(antenna_pairs, np.uint64)
    tof = np.ascontiguousarray(time_offsets, np.uint64)
    sol = np.ascontiguousarray(solutions, np.complex64)
    out = np.zeros((n_rows, n_chan), np.complex64)
    r = lib().oracle_apply_gains(mode, n_pol, n_rows, n_chan, _p(vis), _p(ant), _p(tof),
                                 _p(sol), nparms, n_ant, polarization, _p(out))
    if r != 0:
        raise ValueError("invalid gain mode / polarisation combination")
    return out


def forward_gains(mode, n_pol, vis, antenna_pairs, time_offsets, solutions, nparms, n_ant,
                  polarization=0):
    """Prediction write-back: predicted [row][chan] values expanded to n_pol
    correlations and multiplied by the forward gains; [row][chan][n_pol]."""
    vis = np.ascontiguousarray(vis, np.complex64)
    n_rows, n_chan = vis.shape[0], vis.shape[1]
    ant = np.ascontiguousarray(antenna_pairs, np.uint64)
    tof = np.ascontiguousarray(time_offsets, np.uint64)
    sol = np.ascontiguousarray(solutions, np.complex64)
    out = np.zeros((n_rows, n_chan, n_pol), np.complex64)
    r = lib().oracle_forward_gains(mode, n_pol, n_rows, n_chan, _p(vis), _p(ant), _p(tof),
                                   _p(sol), nparms, n_ant, polarization, _p(out))
    if r != 0:
        raise ValueError("invalid gain mode / polarisation combination")
    return out


def apply_conjugated_gain(mode, vis, g1, g2):
    v = np.ascontiguousarray(vis, np.complex64).copy()
    a = np.ascontiguousarray(g1, np.complex64)
    b = np.ascontiguousarray(g2, np.complex64)
    lib().oracle_apply_conjugated_gain(mode, _p(v), _p(a), _p(b))
    return v


def correction_matrix_add(g1, g2, weight, total=None):
    """AverageCorrection::Add in matrix form: returns total (4 x 4 complex,
    zero when None) plus 0.5 w (a^H a + b^H b), a = G1 (x) G2, b = G2 (x) G1."""
    a = np.ascontiguousarray(g1, np.complex64)
    b = np.ascontiguousarray(g2, np.complex64)
    s = np.zeros(32, np.float64)
    if total is not None:
        t = np.asarray(total, np.complex128).ravel()
        s[0::2], s[1::2] = t.real, t.imag
    lib().oracle_correction_matrix_add(_p(a), _p(b), float(weight), _p(s))
    return (s[0::2] + 1j * s[1::2]).reshape(4, 4)


def apply_gain(mode, vis, g1, g2):
    v = np.ascontiguousarray(vis, np.complex64).copy()
    a = np.ascontiguousarray(g1, np.complex64)
    b = np.ascontiguousarray(g2, np.complex64)
    lib().oracle_apply_gain(mode, _p(v), _p(a), _p(b))
    return v


class ImageWeights:
    """The oracle's imaging-weight grid (ImageWeights restated in C): the same
    operations as the product's wsclean_gb300.weights.ImageWeights, serially
    and in the reference's order.  grid: (height/2, width) float64."""

    def __init__(self, mode, image_width, image_height, pixel_scale_x, pixel_scale_y,
                 weights_as_taper=False, super_weight=1.0, briggs_robustness=0.0):
        w, h = C.c_int64(), C.c_int64()
        lib().oracle_weights_dims(image_width, image_height, super_weight, C.byref(w),
                                  C.byref(h))
        self.width, self.height = w.value, h.value
        self.mode, self.robustness = int(mode), float(briggs_robustness)
        self.psx, self.psy = float(pixel_scale_x), float(pixel_scale_y)
        self.as_taper = bool(weights_as_taper)
        self.grid = np.zeros((self.height // 2, self.width), np.float64)
        self.total = 0.0

    def grid_rows(self, uvw, freq, weights):
        uvw = np.ascontiguousarray(uvw, np.float64)
        freq = np.ascontiguousarray(freq, np.float64)
        wts = np.ascontiguousarray(weights, np.float32)
        n_rows, n_chan = uvw.shape[0], freq.size
        n_pol = wts.size // (n_rows * n_chan) if n_rows * n_chan else 1
        self.total += lib().oracle_weights_grid(_p(self.grid), self.width, self.height,
                                                self.psx, self.psy, int(self.as_taper), n_rows,
                                                n_chan, n_pol, _p(uvw), _p(freq), _p(wts))

    def finish(self):
        lib().oracle_weights_finish(_p(self.grid), self.width, self.height, self.mode,
                                    self.robustness, self.total)

    def taper(self, kind, a, b=0.0):
        lib().oracle_weights_taper(_p(self.grid), self.width, self.height, self.psx, self.psy,
                                   int(kind), float(a), float(b))

    def mirrored(self):
        out = np.zeros((self.height, self.width), np.float64)
        lib().oracle_weights_mirror(_p(self.grid), self.width, self.height, _p(out))
        return out

    def sample(self, u, v):
        u = np.ascontiguousarray(u, np.float64).ravel()
        v = np.ascontiguousarray(v, np.float64).ravel()
        out = np.zeros(u.size, np.float64)
        lib().oracle_weights_sample(_p(self.grid), self.width, self.height, self.psx, self.psy,
                                    u.size, _p(u), _p(v), _p(out))
        return out

    def prepare_rows(self, uvw, freq, weights, vis=None, model=None, selected=None,
                     psf_mode=0, psf_dl=0.0, psf_dm=0.0, visibility_weighting=0,
                     polarization=0, gains=None):
        """CalculateWeights + ApplyWeights + CollapseData over [row][chan][pol]
        inputs; returns (vis_out [row, chan], weights_out [row, chan, pol],
        imaging weights [row, chan], sums [vws, max, total, count]).  gains =
        (mode, antenna_pairs, time_offsets, solutions, nparms, n_ant) applies
        the conjugated gains before ApplyWeights; the TRACE correction sum is
        then sums[4]."""
        uvw = np.ascontiguousarray(uvw, np.float64)
        freq = np.ascontiguousarray(freq, np.float64)
        wts = np.ascontiguousarray(weights, np.float32)
        n_rows, n_chan, n_pol = wts.shape
        vis_a = None if vis is None else np.ascontiguousarray(vis, np.complex64)
        mod_a = None if model is None else np.ascontiguousarray(model, np.complex64)
        sel_a = None if selected is None else np.ascontiguousarray(selected, np.uint8)
        vis_out = np.zeros((n_rows, n_chan), np.complex64)
        w_out = np.zeros((n_rows, n_chan, n_pol), np.float32)
        iw_out = np.zeros((n_rows, n_chan), np.float32)
        sums = np.zeros(5, np.float64)
        args = (_p(self.grid), self.width, self.height, self.psx, self.psy, int(psf_mode),
                float(psf_dl), float(psf_dm), int(mod_a is not None), int(visibility_weighting),
                int(polarization), n_pol, n_rows, n_chan, _p(uvw), _p(freq),
                None if vis_a is None else _p(vis_a), _p(wts),
                None if mod_a is None else _p(mod_a), None if sel_a is None else _p(sel_a),
                _p(vis_out), _p(w_out), _p(iw_out), _p(sums))
        if gains is None:
            lib().oracle_prepare_rows(*args)
            return vis_out, w_out, iw_out, sums[:4]
        mode, ant, tof, sol, nparms, n_ant = gains
        ant = np.ascontiguousarray(ant, np.uint64)
        tof = np.ascontiguousarray(tof, np.uint64)
        sol = np.ascontiguousarray(sol, np.complex64)
        corr = np.zeros(33, np.float64)
        lib().oracle_prepare_rows_corrected(*args, int(mode), _p(ant), _p(tof), _p(sol), nparms,
                                            n_ant, _p(corr))
        sums[4] = corr[0]
        self.correction_matrix = (corr[1::2] + 1j * corr[2::2]).reshape(4, 4)
        return vis_out, w_out, iw_out, sums
