"""Generates tests/golden/misfit_golden.npz from the reference's own misfit code.

Imports toolbox/misfit.py of the reference (directory given on the command line
or in SWIT_REFERENCE_TOOLBOX) with a minimal stand-in for obspy, which the
reference imports at module level (toolbox/tools.py:19-21) but is not installed
here: a trace list whose items carry ``.data`` and ``.stats.sampling_rate``,
the only attributes misfit.py and tools.get_su_parameter / su2array read.
Inputs are seeded (numpy default_rng(2024)); outputs are the reference's
adjoint sources and misfit values for Waveform, Envelope, Traveltime and
Globalcorrelation.

    python tests/golden/make_misfit_golden.py [/path/to/reference/toolbox]
"""
import os
import sys
import types

import numpy as np


class _Stats:
    def __init__(self, dt):
        self.sampling_rate = 1.0 / dt
        self.delta = dt


class _Trace:
    def __init__(self, data, dt):
        self.data = np.asarray(data, np.float32)
        self.stats = _Stats(dt)

    def __len__(self):
        return len(self.data)


def _stub_obspy():
    ob = types.ModuleType("obspy")
    core = types.ModuleType("obspy.core")
    core.UTCDateTime = object
    ob.core = core
    ob.Trace = _Trace
    ob.Stream = list
    ob.read = None
    sys.modules["obspy"] = ob
    sys.modules["obspy.core"] = core


def inputs():
    rng = np.random.default_rng(2024)
    ntr, nt, dt = 6, 256, 0.004
    t = np.arange(nt) * dt
    obs = np.zeros((ntr, nt), np.float32)
    syn = np.zeros((ntr, nt), np.float32)
    for i in range(ntr):
        f = rng.uniform(4, 12)
        t0 = rng.uniform(0.3, 0.6)
        shift = rng.uniform(-0.05, 0.05)
        amp = rng.uniform(0.5, 2.0)
        w = lambda tt: (1 - 2 * (np.pi * f * tt) ** 2) * np.exp(-(np.pi * f * tt) ** 2)
        obs[i] = w(t - t0)
        syn[i] = amp * w(t - t0 - shift) + 0.01 * rng.standard_normal(nt)
    syn[3] = 0.0  # a dead synthetic trace
    return obs, syn, dt


def main():
    toolbox = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SWIT_REFERENCE_TOOLBOX")
    if not toolbox:
        sys.exit("usage: %s <reference toolbox directory> (or set SWIT_REFERENCE_TOOLBOX)" % sys.argv[0])
    _stub_obspy()
    sys.path.insert(0, toolbox)
    import misfit as M  # the reference's toolbox/misfit.py

    obs, syn, dt = inputs()
    so = [_Trace(x, dt) for x in obs]
    ss = [_Trace(x, dt) for x in syn]
    out = dict(obs=obs, syn=syn, dt=np.float64(dt))
    out["adj_waveform"] = M.adjoint_source_waveform(so, ss)
    out["adj_envelope"] = M.adjoint_source_envelope(so, ss)
    out["adj_traveltime"] = M.adjoint_source_traveltime(so, ss)
    out["adj_globalcorrelation"] = M.adjoint_source_global_correlation(so, ss)
    out["mis_waveform"] = M.misfit_waveform(so, ss)
    out["mis_envelope"] = M.misfit_envelope(so, ss)
    out["mis_traveltime"] = M.misfit_traveltime(so, ss)
    out["mis_globalcorrelation"] = M.misfit_global_correlation(so, ss)
    out["ccmax"] = M.cross_correlate_max(so, ss)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "misfit_golden.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: np.asarray(v).shape for k, v in out.items()})


if __name__ == "__main__":
    main()
