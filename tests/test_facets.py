"""Facet batch (many jobs, one gridding launch per wave, one CUDA graph).

Each job's image must equal the plain gridder run on the same plan with the
job's channel range (within 2e-6 relative L2: the batch accumulates in a
different order) and be within epsilon of the FP64 direct FT at the facet's
phase-centre shift; splitting the batch into more waves must not change it.
"""
import numpy as np
import pytest

from wsclean_gb300 import _lib, synthetic
from wsclean_gb300.gridder import WGriddingGridder_Simple

C = 299792458.0


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


FACETS = [dict(width=64, height=64, dl=8e-4, l_shift=0.0, m_shift=0.0),
          dict(width=96, height=64, dl=8e-4, l_shift=0.03, m_shift=-0.02),
          dict(width=128, height=128, dl=6e-4, l_shift=-0.025, m_shift=0.035)]
GROUPS = [0, 2, 5]


def _data():
    uvw, freq, vis = synthetic.random_points(700, 5, 128, 8e-4, seed=81, w_scale=2.0,
                                             frac_zero=0.05)
    return uvw, freq, vis


@pytest.mark.gpu
def test_facet_jobs_match_single_gridders_and_dft(wgpu_lib, oracle_lib):
    from wsclean_gb300.facets import FacetBatch
    uvw, freq, vis = _data()
    eps = 1e-4
    fb = FacetBatch(FACETS, GROUPS, epsilon=eps)
    fb.bind(uvw, freq)
    info = fb.info()
    assert info["n_jobs"] == len(FACETS) * (len(GROUPS) - 1)
    images = fb.invert(vis)
    for job, img in enumerate(images):
        gi, fi = divmod(job, len(FACETS))
        f = FACETS[fi]
        c0, c1 = GROUPS[gi], GROUPS[gi + 1]
        plan = fb.job_plan(job)
        assert plan.support == info["support"]  # one width for the whole batch
        g = WGriddingGridder_Simple(f["width"], f["height"], f["width"], f["height"], f["dl"],
                                    f["dl"], f["l_shift"], f["m_shift"], 1, epsilon=eps)
        g.pin_plan(plan)
        g.InitializeInversion()
        g.AddInversionData(uvw.shape[0], c1 - c0, uvw, freq[c0:c1],
                           np.ascontiguousarray(vis[:, c0:c1]))
        g.FinalizeImage(1.0)
        single = g.RealImage().reshape(f["height"], f["width"]).astype(np.float64)
        g.close()
        assert rel(img, single) <= 2e-6, job
        dft = oracle_lib.dft_invert(uvw, freq[c0:c1], np.ascontiguousarray(vis[:, c0:c1]),
                                    f["width"], f["height"], f["dl"], f["dl"], f["l_shift"],
                                    f["m_shift"]).reshape(f["height"], f["width"])
        assert rel(img, dft) <= eps, job
    # replaying the graph gives the same images
    again = fb.invert(vis)
    for a, b in zip(images, again):
        assert rel(b, a) <= 2e-6
    fb.close()


@pytest.mark.gpu
def test_facet_waves_do_not_change_images(wgpu_lib):
    from wsclean_gb300.facets import FacetBatch
    uvw, freq, vis = _data()
    one = FacetBatch(FACETS, GROUPS, epsilon=1e-4)
    one.bind(uvw, freq)
    many = FacetBatch(FACETS, GROUPS, epsilon=1e-4, plane_budget_bytes=1.0)  # a wave per batch
    many.bind(uvw, freq)
    assert one.info()["n_waves"] == 1
    assert many.info()["n_waves"] >= one.info()["n_jobs"]
    for a, b in zip(one.invert(vis), many.invert(vis)):
        assert rel(b, a) <= 2e-6
    one.close()
    many.close()


def test_facet_batch_validates_arguments(wgpu_lib):
    from wsclean_gb300.facets import FacetBatch
    with pytest.raises(_lib.WgpuError) as e:
        FacetBatch([dict(width=63, height=64, dl=1e-3)], [0, 1])
    assert e.value.status == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError) as e:
        FacetBatch([dict(width=64, height=64, dl=1e-3)], [0, 2, 2])
    assert e.value.status == _lib.WGPU_ERR_INVALID
    with pytest.raises(_lib.WgpuError) as e:
        FacetBatch([dict(width=64, height=64, dl=1e-3)], [0, 2], epsilon=0.0)
    assert e.value.status == _lib.WGPU_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("mode,n_pol,nparms", [(4, 4, 4), (3, 2, 2), (2, 1, 4)])
def test_facet_corrections_match_oracle_gains(wgpu_lib, oracle_lib, mode, n_pol, nparms):
    """Direction-dependent gains: each facet's jobs see its own conjugated gains
    (applied on the device from one upload of the uncorrected visibilities and
    all facets' solution tables).  A facet's images equal the plain batch run
    on the oracle's gain-applied, collapsed visibilities for that facet (FP32
    gains with fused multiply-adds: 1e-5), and are within epsilon of the FP64
    direct FT of those visibilities."""
    from wsclean_gb300.facets import FacetBatch
    uvw, freq, vis1 = _data()
    rng = np.random.default_rng(90 + mode)
    n_rows, n_chan, n_ant, n_t = uvw.shape[0], freq.size, 6, 2
    vis = (np.repeat(vis1[:, :, None], n_pol, axis=2) *
           (1.0 + 0.2 * rng.standard_normal((n_rows, n_chan, n_pol)))).astype(np.complex64)
    ant = np.stack([rng.integers(0, n_ant, n_rows), rng.integers(0, n_ant, n_rows)], axis=1)
    tof = rng.integers(0, n_t, n_rows).astype(np.uint64)
    sol = (1.0 + 0.3 * (rng.standard_normal((len(FACETS), n_t, n_chan, n_ant, nparms)) +
                        1j * rng.standard_normal((len(FACETS), n_t, n_chan, n_ant, nparms)))
           ).astype(np.complex64)
    eps = 1e-4
    fb = FacetBatch(FACETS, GROUPS, epsilon=eps)
    fb.bind(uvw, freq, corrected=True)
    images = fb.invert_corrected(mode, vis, ant, tof, sol, nparms, n_t, n_ant)
    with pytest.raises(_lib.WgpuError):
        fb.invert(vis1)  # a corrected binding needs the corrected inversion
    plain = FacetBatch(FACETS, GROUPS, epsilon=eps)
    plain.bind(uvw, freq)
    for fi, f in enumerate(FACETS):
        corrected = oracle_lib.apply_gains(mode, n_pol, vis, ant, tof, sol[fi], nparms, n_ant)
        ref_images = plain.invert(corrected)
        for gi in range(len(GROUPS) - 1):
            job = gi * len(FACETS) + fi
            assert rel(images[job], ref_images[job]) <= 1e-5, job
            c0, c1 = GROUPS[gi], GROUPS[gi + 1]
            dft = oracle_lib.dft_invert(uvw, freq[c0:c1], np.ascontiguousarray(corrected[:, c0:c1]),
                                        f["width"], f["height"], f["dl"], f["dl"], f["l_shift"],
                                        f["m_shift"]).reshape(f["height"], f["width"])
            assert rel(images[job], dft) <= eps, job
    bad = ant.copy()
    bad[0, 1] = n_ant
    with pytest.raises(_lib.WgpuError):
        fb.invert_corrected(mode, vis, bad, tof, sol, nparms, n_t, n_ant)
    fb.close()
    plain.close()


@pytest.mark.gpu
def test_rebinding_one_batch_matches_fresh_batches(wgpu_lib):
    """A batch re-bound to other rows (here each channel group in turn, as the
    full-size workload streams them) reuses its device memory: every bind's
    images equal those of a batch created for that bind alone."""
    from wsclean_gb300.facets import FacetBatch
    uvw, freq, vis = _data()
    fb = FacetBatch(FACETS, [0, 2], epsilon=1e-4)
    for c0, c1 in ((0, 2), (2, 4), (3, 5), (0, 2)):
        sub = np.ascontiguousarray(vis[:, c0:c1])
        fb.bind(uvw, freq[c0:c1])
        got = fb.invert(sub)
        fresh = FacetBatch(FACETS, [0, 2], epsilon=1e-4)
        fresh.bind(uvw, freq[c0:c1])
        ref = fresh.invert(sub)
        fresh.close()
        for a, b in zip(got, ref):
            assert rel(a, b) <= 2e-6, (c0, c1)
    fb.close()
