"""Generates tests/golden/precond_golden.npz from the reference's own gradient
preconditioning (toolbox/postprocess.py:20-111, toolbox/tools.py:237-275).

The reference modules import obspy (toolbox/tools.py:19-21) and matplotlib
(toolbox/plot.py), neither installed here; minimal stand-ins are injected (the
plotting call is a no-op, obspy is never used by these functions).  scipy 1.18
dropped the scipy.signal.hamming alias that grad_taper calls for land surveys;
it is pointed at scipy.signal.windows.hamming, the same function.  Inputs are
seeded (numpy default_rng(7)).

    python tests/golden/make_precond_golden.py [/path/to/reference/toolbox]
"""
import os
import sys
import types

import numpy as np


def _stubs():
    ob = types.ModuleType("obspy")
    core = types.ModuleType("obspy.core")
    core.UTCDateTime = object
    ob.core = core
    sys.modules["obspy"] = ob
    sys.modules["obspy.core"] = core
    plot = types.ModuleType("plot")
    plot.plot_model2D = lambda *a, **k: None
    sys.modules["plot"] = plot
    import scipy.signal
    import scipy.signal.windows
    if not hasattr(scipy.signal, "hamming"):
        scipy.signal.hamming = scipy.signal.windows.hamming


def cases():
    rng = np.random.default_rng(7)
    nx, nz = 60, 32
    grad = rng.standard_normal(nx * nz)
    forw = np.abs(rng.standard_normal(nx * nz)) * 3 + 0.1
    back = np.abs(rng.standard_normal(nx * nz)) + 0.05
    mask = (rng.uniform(size=(nx, nz)) > 0.2).astype(np.float64)
    return nx, nz, grad, forw, back, mask, [
        ("marine", dict(marine_or_land="Marine", grad_mute=5, grad_thred=0.0, grad_smooth=3, grad_mask=None)),
        ("land", dict(marine_or_land="Land", grad_mute=6, grad_thred=0.001, grad_smooth=2, grad_mask=None)),
        ("land_nosmooth_mask", dict(marine_or_land="Land", grad_mute=0, grad_thred=0.001, grad_smooth=0,
                                    grad_mask=mask)),
    ]


def main():
    toolbox = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SWIT_REFERENCE_TOOLBOX")
    if not toolbox:
        sys.exit("usage: %s <reference toolbox directory> (or set SWIT_REFERENCE_TOOLBOX)" % sys.argv[0])
    _stubs()
    sys.path.insert(0, toolbox)
    import postprocess as P  # the reference's toolbox/postprocess.py
    import tools as T
    nx, nz, grad, forw, back, mask, cs = cases()
    out = dict(grad=grad, forw=forw, back=back, mask=mask, nx=nx, nz=nz)
    for name, o in cs:
        simu = types.SimpleNamespace(model=types.SimpleNamespace(nx=nx, nz=nz))
        optim = types.SimpleNamespace(vpmax=4500.0, iter=1, **o)
        out["out_" + name] = P.grad_precond(simu, optim, grad.copy(), forw.copy(), back.copy())
    out["smooth_7"] = T.smooth2d(forw.reshape(nx, nz), span=7)
    out["taper_land_6"] = P.grad_taper(nx, nz, tapersize=6, thred=0.001, marine_or_land="Land")
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "precond_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, sorted(out))


if __name__ == "__main__":
    main()
