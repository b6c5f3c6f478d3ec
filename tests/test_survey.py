"""CPU tests of the seeded benchmark workloads: shapes, seeds and the stability
condition of toolbox/base.py:42, 58-59 (dt < sqrt(3/8) dx / vmax)."""
import numpy as np
import pytest

from swit_gb300 import survey


@pytest.mark.parametrize("idx,shape,ns,ng,nt", [(0, (201, 101), 5, 201, 2000), (1, (481, 141), 49, 481, 4000),
                                                (2, (501, 171), 51, 501, 5000)])
def test_config_shapes_and_stability(idx, shape, ns, ng, nt):
    s = survey.config(idx)
    assert s.vp_true.shape == shape and s.vp_init.shape == shape
    assert s.ns == ns and s.ng == ng and s.nt == nt and s.npml == 40
    for vp in (s.vp_true, s.vp_init):
        assert np.isfinite(vp).all() and vp.min() >= 1000
        assert s.dt < np.sqrt(3.0 / 8.0) * s.dx / vp.max()
    src = s.source()
    assert src.shape == (ns, nt) and src.dtype == np.float32


def test_configs_are_seeded():
    a, b = survey.config(1), survey.config(1)
    np.testing.assert_array_equal(a.vp_true, b.vp_true)
    assert survey.config(1).vp_true[:, :12].max() == 1500.0  # water layer


def test_source_is_the_integrated_reference_ricker():
    w = survey.ricker(4000, 0.002, 5.0)
    assert abs(np.argmax(w) * 0.002 - 1.2 / 5.0) < 0.002
    s = survey.integrated_source(w)
    np.testing.assert_allclose(s[1:], np.cumsum(0.5 * (w[1:] + w[:-1])).astype(np.float32), rtol=1e-5, atol=1e-7)


def test_thrust_fold_model():
    """501x171 at 20 m: 25 layers from 2000 to 6000 m/s, increasing with depth on
    average, folded (layer boundaries not flat) and seeded."""
    s = survey.config(2)
    vp = s.vp_true
    assert np.unique(vp).size == 25 and vp.min() == 2000.0 and vp.max() == 6000.0
    mean_z = vp.mean(axis=0)
    assert mean_z[-1] > mean_z[0] + 2500
    top_layer_depth = (vp <= vp.min()).sum(axis=1)
    assert top_layer_depth.max() - top_layer_depth.min() >= 5  # the anticline bends the layers
    np.testing.assert_array_equal(vp, survey.config(2).vp_true)
    assert s.dt == 0.0015 and s.dx == 20.0
