"""Device misfits against golden vectors made by the reference's own
toolbox/misfit.py (tests/golden/make_misfit_golden.py), on CPU tensors and
(marked gpu) on CUDA tensors."""
import os

import numpy as np
import pytest
import torch

from swit_gb300 import misfit as M

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "misfit_golden.npz"))
DEVICES = [pytest.param("cpu", id="cpu"), pytest.param("cuda", id="cuda", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("device", DEVICES)
@pytest.mark.parametrize("name", ["waveform", "envelope", "traveltime", "globalcorrelation"])
def test_adjoint_source_and_value_match_reference(name, device):
    syn = torch.from_numpy(G["syn"]).to(device)
    obs = torch.from_numpy(G["obs"]).to(device)
    dt = float(G["dt"])
    val, adj = M.adjoint_source(syn, obs, dt, name)
    assert adj.device.type == device
    adj = adj.cpu()
    ref = G["adj_" + name]
    scale = np.abs(ref).max()
    assert np.abs(adj.numpy() - ref).max() <= 1e-5 * scale, name
    mref = float(G["mis_" + name][0])
    assert abs(float(val) - mref) <= 1e-5 * abs(mref) + 1e-12, (name, float(val), mref)
    # the dead synthetic trace contributes nothing
    assert not np.any(adj.numpy()[3])


@pytest.mark.parametrize("device", DEVICES)
def test_cross_correlation_lag_matches_reference(device):
    cc = M.cross_correlate_max(torch.from_numpy(G["obs"]).to(device), torch.from_numpy(G["syn"]).to(device))
    np.testing.assert_array_equal(cc.cpu().numpy(), G["ccmax"])


def test_batched_shapes_give_the_same_adjoint():
    syn = torch.from_numpy(np.stack([G["syn"], G["syn"][::-1].copy()]))
    obs = torch.from_numpy(np.stack([G["obs"], G["obs"][::-1].copy()]))
    _, adj = M.adjoint_source(syn, obs, float(G["dt"]), "Globalcorrelation")
    ref = G["adj_globalcorrelation"]
    np.testing.assert_allclose(adj[0].numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    _, one = M.adjoint_source(syn[0], obs[0], float(G["dt"]), "Globalcorrelation")
    np.testing.assert_array_equal(adj[0].numpy(), one.numpy())
