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
