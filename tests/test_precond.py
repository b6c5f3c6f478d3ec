"""Device gradient preconditioning against golden vectors made by the
reference's own toolbox/postprocess.py (tests/golden/make_precond_golden.py),
on CPU tensors and (marked gpu) on CUDA tensors."""
import os

import numpy as np
import pytest
import torch

from swit_gb300 import precond as P

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "precond_golden.npz"))
NX, NZ = int(G["nx"]), int(G["nz"])
DEVICES = [pytest.param("cpu", id="cpu"), pytest.param("cuda", id="cuda", marks=pytest.mark.gpu)]


@pytest.mark.parametrize("device", DEVICES)
def test_smooth2d_matches_reference(device):
    got = P.smooth2d(torch.from_numpy(G["forw"].reshape(NX, NZ)).to(device), span=7).cpu().numpy()
    np.testing.assert_allclose(got, G["smooth_7"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("device", DEVICES)
def test_land_taper_matches_reference(device):
    got = P.grad_taper(NX, NZ, tapersize=6, thred=0.001, marine_or_land="Land", device=device).cpu().numpy()
    np.testing.assert_allclose(got, G["taper_land_6"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("name,opts", [
    ("marine", dict(marine_or_land="Marine", grad_mute=5, grad_thred=0.0, grad_smooth=3, grad_mask=None)),
    ("land", dict(marine_or_land="Land", grad_mute=6, grad_thred=0.001, grad_smooth=2, grad_mask=None)),
    ("land_nosmooth_mask", dict(marine_or_land="Land", grad_mute=0, grad_thred=0.001, grad_smooth=0,
                                grad_mask="mask")),
])
@pytest.mark.parametrize("device", DEVICES)
def test_grad_precond_matches_reference(name, opts, device):
    if opts["grad_mask"] == "mask":
        opts = dict(opts, grad_mask=G["mask"])
    got = P.grad_precond(torch.from_numpy(G["grad"]).to(device), G["forw"], G["back"], NX, NZ, 4500.0, **opts)
    assert got.device.type == device
    got = got.cpu().numpy()
    np.testing.assert_allclose(got, G["out_" + name], rtol=1e-10, atol=1e-9)
