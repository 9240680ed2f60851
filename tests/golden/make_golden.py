"""Generates the committed golden fixtures in tests/golden/.

gains_kat.json
    The known-answer cases of the reference's gain tests
    (tests/gridding/tvisibilitymodifier.cpp:13-28 constants; expectations of
    apply_h5parm :107-115 and apply_conjugate_h5parm :117-139, including the
    latter's correction-sum elements), evaluated in complex64 / float exactly
    as the test states them.
dft_small.npz
    A 64 x 64 direct-FT inversion and prediction of a seeded random case,
    computed by the oracle (FP64).  Pins the oracle across host architectures.
bucket_small.npz
    The oracle's bucketing of a seeded random case for a fixed plan (keys,
    permutation, footprint corners and fractions).  The GPU pass must match it
    bit for bit.

Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# tests/gridding/tvisibilitymodifier.cpp:13-20
A1_PARM_X = np.complex64(0.25 - 0.25j)
A2_PARM_X = np.complex64(5.0 - 1.0j)
A1_PARM_Y = np.complex64(3.0 - 0.5j)
A2_PARM_Y = np.complex64(-1.0 + 7.0j)


def c2l(z):
    z = np.asarray(z, np.complex64).ravel()
    return [[float(v.real), float(v.imag)] for v in z]


def gains_kat():
    g1 = np.array([A1_PARM_X, 0, 0, A1_PARM_Y], np.complex64)
    g2 = np.array([A2_PARM_X, 0, 0, A2_PARM_Y], np.complex64)
    cases = []
    # apply_h5parm: ApplyParmResponse<k2VisDiagonal> on {7, 8}
    xx, yy = np.complex64(7.0), np.complex64(8.0)
    cases.append(dict(name="apply_h5parm", direction="forward", mode=3, vis=c2l([xx, yy]),
                      g1=c2l(g1), g2=c2l(g2),
                      expected=c2l([xx * A1_PARM_X * np.conj(A2_PARM_X),
                                    yy * A1_PARM_Y * np.conj(A2_PARM_Y)])))
    # apply_conjugate_h5parm: ApplyConjugatedParmResponse<kApplyAndSum, k2VisDiagonal> on {-1, 2}
    xx, yy = np.complex64(-1.0), np.complex64(2.0)
    # and its correction sum (:128-136): elements 0, 5, 10, 15 of the 4 x 4
    # matrix (row-major), unit visibility and imaging weights
    nx = np.float32(abs(A1_PARM_X) ** 2 * abs(A2_PARM_X) ** 2)
    ny = np.float32(abs(A1_PARM_Y) ** 2 * abs(A2_PARM_Y) ** 2)
    nxy = np.float32(0.5 * (abs(A1_PARM_X * np.conj(A2_PARM_Y)) ** 2 +
                            abs(A2_PARM_X * np.conj(A1_PARM_Y)) ** 2))
    cases.append(dict(name="apply_conjugate_h5parm", direction="conjugated", mode=3,
                      vis=c2l([xx, yy]), g1=c2l(g1), g2=c2l(g2),
                      expected=c2l([xx * np.conj(A1_PARM_X) * A2_PARM_X,
                                    yy * np.conj(A1_PARM_Y) * A2_PARM_Y]),
                      correction_sum={"0": float(nx), "5": float(nxy), "10": float(nxy),
                                      "15": float(ny)}))
    return dict(tolerance=1e-5, source="tests/gridding/tvisibilitymodifier.cpp", cases=cases)


def main():
    import oracle
    from wsclean_gb300 import synthetic

    with open(os.path.join(HERE, "gains_kat.json"), "w") as fh:
        json.dump(gains_kat(), fh, indent=1)

    W, dl = 64, 1e-3
    uvw, freq, vis = synthetic.random_points(200, 4, W, dl, seed=11, w_scale=2.0, frac_zero=0.1)
    img = oracle.dft_invert(uvw, freq, vis, W, W, dl, dl, 0.003, -0.002)
    model = np.zeros(W * W)
    model[[100, 2000, 3333]] = [1.0, -0.5, 0.25]
    pred = oracle.dft_predict(uvw, freq, model, W, W, dl, dl, 0.003, -0.002)
    np.savez_compressed(os.path.join(HERE, "dft_small.npz"), uvw=uvw, freq=freq, vis=vis,
                        width=W, dl=dl, l_shift=0.003, m_shift=-0.002, image=img, model=model,
                        pred=pred)

    plan = dict(width=96, height=96, nu=128, nv=128, support=7, tile=16, n_planes=11,
                beta=14.2414, dl=1e-3, dm=1e-3, l_shift=0.0, m_shift=0.0, w0=-900.0, dw=180.0,
                nm1_center=-0.002)
    uvw, freq, vis = synthetic.random_points(500, 6, 96, 1e-3, seed=5, w_scale=0.5,
                                             frac_zero=0.2)
    # keep w inside the plan's plane range
    uvw[:, 2] = np.clip(uvw[:, 2], -150.0, 150.0)
    b = oracle.bucket(plan, uvw, freq, vis, True)
    np.savez_compressed(os.path.join(HERE, "bucket_small.npz"), uvw=uvw, freq=freq, vis=vis,
                        plan=json.dumps(plan), **{k: v for k, v in b.items()})
    print("golden fixtures written")


if __name__ == "__main__":
    main()
