"""Device misfits against golden vectors made by the reference's own
toolbox/misfit.py (tests/golden/make_misfit_golden.py).  Runs on CPU tensors
here; the same torch code runs on the GPU."""
import os

import numpy as np
import pytest
import torch

from swit_gb300 import misfit as M

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "misfit_golden.npz"))


@pytest.mark.parametrize("name", ["waveform", "envelope", "traveltime", "globalcorrelation"])
def test_adjoint_source_and_value_match_reference(name):
    syn = torch.from_numpy(G["syn"])
    obs = torch.from_numpy(G["obs"])
    dt = float(G["dt"])
    val, adj = M.adjoint_source(syn, obs, dt, name)
    ref = G["adj_" + name]
    scale = np.abs(ref).max()
    assert np.abs(adj.numpy() - ref).max() <= 1e-5 * scale, name
    mref = float(G["mis_" + name][0])
    assert abs(float(val) - mref) <= 1e-5 * abs(mref) + 1e-12, (name, float(val), mref)
    # the dead synthetic trace contributes nothing
    assert not np.any(adj.numpy()[3])


def test_cross_correlation_lag_matches_reference():
    cc = M.cross_correlate_max(torch.from_numpy(G["obs"]), torch.from_numpy(G["syn"]))
    np.testing.assert_array_equal(cc.numpy(), G["ccmax"])


def test_batched_shapes_give_the_same_adjoint():
    syn = torch.from_numpy(np.stack([G["syn"], G["syn"][::-1].copy()]))
    obs = torch.from_numpy(np.stack([G["obs"], G["obs"][::-1].copy()]))
    _, adj = M.adjoint_source(syn, obs, float(G["dt"]), "Globalcorrelation")
    ref = G["adj_globalcorrelation"]
    np.testing.assert_allclose(adj[0].numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    _, one = M.adjoint_source(syn[0], obs[0], float(G["dt"]), "Globalcorrelation")
    np.testing.assert_array_equal(adj[0].numpy(), one.numpy())
