"""Generates tests/golden/optim_golden.npz from the reference's own search
directions (toolbox/inversion.py:111-271, NLCG and LBFGS).

toolbox/inversion.py imports matplotlib (via plot) and obspy, neither installed
here: minimal stand-ins are injected; none of their functions is called.  The
directions are followed for four iterations on a seeded quadratic problem
(numpy default_rng(11)), accepting a fixed step each time; LBFGS keeps its S, Y
memmaps in ./outputs/LBFGS_memory/ (inversion.py:212-223), so the generator runs
in a temporary directory.

    python tests/golden/make_optim_golden.py [/path/to/reference/toolbox]
"""
import os
import sys
import tempfile
import types

import numpy as np


def _stubs():
    ob = types.ModuleType("obspy")
    core = types.ModuleType("obspy.core")
    core.UTCDateTime = object
    ob.core = core
    ob.Stream = list
    ob.Trace = object
    sys.modules["obspy"] = ob
    sys.modules["obspy.core"] = core
    plot = types.ModuleType("plot")
    for name in ("plot_inv_scheme", "plot_wavelet", "plot_trace", "plot_rtm", "plot_model2D"):
        setattr(plot, name, lambda *a, **k: None)
    sys.modules["plot"] = plot


def problem():
    rng = np.random.default_rng(11)
    n = 200
    Q = rng.standard_normal((n, n))
    A = Q @ Q.T / n + np.eye(n)
    b = rng.standard_normal(n)
    v0 = rng.standard_normal(n)
    return A, b, v0


def run(mod, scheme, steps=(0.5, 0.5, 0.5, 0.5)):
    A, b, v0 = problem()
    n = v0.size
    simu = types.SimpleNamespace(model=types.SimpleNamespace(nx=n, nz=1))
    optim = types.SimpleNamespace(scheme=scheme)
    st = mod.optimize_init(simu, optim)
    st["v_now"] = v0.copy()
    st["v_old"] = v0.copy()
    ds = []
    for step in steps:
        st["g_now"] = A @ st["v_now"] - b
        st = mod.NLCG(st) if scheme == "NLCG" else mod.LBFGS(st)
        ds.append(np.array(st["d_now"], np.float64))
        if scheme == "NLCG":
            st["g_old"], st["d_old"] = st["g_now"], st["d_now"]
            st["v_now"] = st["v_now"] + step * st["d_now"]
        else:
            st["g_old"], st["v_old"] = st["g_now"], st["v_now"]
            st["v_now"] = st["v_now"] + step * st["d_now"]
    return np.stack(ds)


def main():
    toolbox = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SWIT_REFERENCE_TOOLBOX")
    if not toolbox:
        sys.exit("usage: %s <reference toolbox directory> (or set SWIT_REFERENCE_TOOLBOX)" % sys.argv[0])
    _stubs()
    sys.path.insert(0, toolbox)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "optim_golden.npz")
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "outputs", "LBFGS_memory"))
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            import inversion as M  # the reference's toolbox/inversion.py
            out = dict(d_lbfgs=run(M, "LBFGS"), d_nlcg=run(M, "NLCG"))
        finally:
            os.chdir(cwd)
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
