"""Derives the exponential-of-semicircle (ES) gridding-kernel table used by the GPU w-gridder.

The reference delegates kernel selection to ducc0's built-in tables (called from
wgridder/gridder_simple.h:217-225); those tables are not part of the reference tree.
This script derives an equivalent table from the published method (Barnett et al. 2019,
"A parallel non-uniform fast Fourier transform library based on an exponential of
semicircle kernel"; Arras et al. 2021, "Efficient wide-field radio interferometry
response"), by numerically evaluating the aliasing error of the kernel

    phi(z) = exp(beta * (sqrt(1 - z^2) - 1)),   |z| <= 1,

spread over W grid cells (t = z * W / 2) on a grid oversampled by sigma.

For every (W, sigma) it picks the beta that minimises the RMS relative aliasing error

    e(f) = sqrt(sum_{m != 0} psihat(f + m)^2) / psihat(f),   |f| <= 1 / (2 sigma)

(psihat is the continuous Fourier transform of the kernel in cycles per cell), and
records both the RMS and the maximum of e over the band.  The three gridded
dimensions (u, v and w) each contribute such an error; the planner combines them.

Run ``python -m wsclean_gb300.kernel_table`` to regenerate csrc/es_table.h.
"""
import os

import numpy as np

W_RANGE = list(range(4, 17))
SIGMAS = [1.10, 1.15, 1.20, 1.25, 1.30, 1.35, 1.40, 1.50, 1.60, 1.75, 2.00]


def _gl(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


_X, _WT = _gl(600)


def psihat(f, W, beta):
    """Continuous FT of the kernel in cell units at frequencies f (cycles/cell)."""
    phi = np.exp(beta * (np.sqrt(1.0 - _X * _X) - 1.0))
    f = np.atleast_1d(f)
    return (W / 2.0) * (np.cos(np.pi * np.outer(f, _X) * W) @ (_WT * phi))


def alias_error(W, beta, sigma, nf=64, nalias=6):
    f = np.linspace(0.0, 0.5 / sigma, nf)
    main = psihat(f, W, beta)
    tail = np.zeros_like(f)
    for m in range(1, nalias + 1):
        tail += psihat(f + m, W, beta) ** 2 + psihat(f - m, W, beta) ** 2
    e = np.sqrt(tail) / np.abs(main)
    return float(np.sqrt(np.mean(e * e))), float(e.max())


def best_beta(W, sigma):
    # beta ~ gamma * pi * W * (1 - 1/(2 sigma)); scan gamma then refine.
    base = np.pi * W * (1.0 - 0.5 / sigma)
    gammas = np.linspace(0.80, 1.05, 26)
    errs = [alias_error(W, g * base, sigma)[0] for g in gammas]
    i = int(np.argmin(errs))
    lo = gammas[max(i - 1, 0)]
    hi = gammas[min(i + 1, len(gammas) - 1)]
    for _ in range(20):
        a = lo + (hi - lo) / 3
        b = hi - (hi - lo) / 3
        if alias_error(W, a * base, sigma)[0] < alias_error(W, b * base, sigma)[0]:
            hi = b
        else:
            lo = a
    g = 0.5 * (lo + hi)
    rms, mx = alias_error(W, g * base, sigma)
    return g * base, rms, mx, amplification(W, g * base, sigma)


def amplification(W, beta, sigma, nf=200):
    """RMS over the band |f| <= 1/(2 sigma) of psihat(0) / psihat(f): the factor
    by which the grid correction magnifies white round-off noise of the grid
    and of the FFT.  In FP32 this, raised to the number of corrected
    dimensions, sets the noise floor of the result."""
    f = np.linspace(0.0, 0.5 / sigma, nf)
    a = psihat(0.0, W, beta)[0] / psihat(f, W, beta)
    return float(np.sqrt(np.mean(a * a)))


def build_table():
    rows = []
    for W in W_RANGE:
        for s in SIGMAS:
            beta, rms, mx, amp = best_beta(W, s)
            rows.append((W, s, beta, rms, mx, amp))
    return rows


def write_header(rows, path):
    with open(path, "w") as fh:
        fh.write("// Generated by wsclean_gb300/kernel_table.py: ES kernel parameters.\n")
        fh.write("// Columns: support W (cells), oversampling sigma, beta, RMS and max\n")
        fh.write("// one-dimensional relative aliasing error over |f| <= 1/(2 sigma), and the\n")
        fh.write("// RMS correction amplification psihat(0)/psihat(f) over the same band.\n")
        fh.write("#pragma once\n\nnamespace wgpu {\n\n")
        fh.write("struct EsKernelEntry { int support; double sigma; double beta;"
                 " double err_rms; double err_max; double amp_rms; };\n\n")
        fh.write("static const EsKernelEntry kEsKernelTable[] = {\n")
        for W, s, beta, rms, mx, amp in rows:
            fh.write(f"    {{{W}, {s:.2f}, {beta:.10f}, {rms:.6e}, {mx:.6e}, {amp:.6e}}},\n")
        fh.write("};\n\n")
        fh.write(f"static const int kEsKernelTableSize = {len(rows)};\n\n}}  // namespace wgpu\n")


if __name__ == "__main__":
    rows = build_table()
    for r in rows:
        print("W=%2d sigma=%.2f beta=%8.4f rms=%.3e max=%.3e amp=%.3e" % r)
    here = os.path.dirname(os.path.abspath(__file__))
    write_header(rows, os.path.join(here, "csrc", "es_table.h"))
