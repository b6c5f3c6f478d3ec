"""Misfits of SWIT's toolbox/misfit.py on device, in torch, with the reference's
adjoint sources as their autograd gradients.

Each function takes synthetics and observations shaped (..., ng, nt) and
returns the reference's misfit value; calling .backward() on it yields, as the
gradient w.r.t. the synthetics, exactly the reference's adjoint source
(times the upstream gradient).  Traces where either the observed or the
synthetic trace is all zero contribute nothing, as in the reference.

    waveform            misfit.py:263-282  (value)   128-148 (adjoint: syn - obs)
    envelope            misfit.py:285-309            151-184 (power p = 2)
    traveltime          misfit.py:312-334, 359-373   188-215 (cross-correlation lag)
    global_correlation  misfit.py:338-355            219-242

All arithmetic is float64, like numpy in the reference.
"""
import torch


def _live(syn, obs):
    return (torch.linalg.vector_norm(obs, dim=-1) > 0) & (torch.linalg.vector_norm(syn, dim=-1) > 0)


def hilbert_imag(x):
    """Imaginary part of scipy.signal.hilbert(x) along the last axis."""
    n = x.shape[-1]
    X = torch.fft.fft(x.to(torch.float64), dim=-1)
    h = torch.zeros(n, dtype=torch.float64, device=x.device)
    if n % 2 == 0:
        h[0] = h[n // 2] = 1.0
        h[1:n // 2] = 2.0
    else:
        h[0] = 1.0
        h[1:(n + 1) // 2] = 2.0
    return torch.fft.ifft(X * h, dim=-1).imag


def cross_correlate_max(obs, syn):
    """misfit.py:359-373: lag index of the cross-correlation maximum, shifted into [nt//2, nt + nt//2)."""
    nt = obs.shape[-1]
    a = torch.fft.fft(obs.to(torch.float64), dim=-1)
    b = -torch.conj(torch.fft.fft(syn.to(torch.float64), dim=-1))
    cc = torch.argmax(torch.abs(torch.fft.ifft(a * b, dim=-1)), dim=-1) - 1
    return torch.where(cc < nt // 2, cc + nt, cc)


class _Waveform(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs, dt):
        s, o = syn.to(torch.float64), obs.to(torch.float64)
        live = _live(s, o)
        r = (syn - obs).to(torch.float64)  # float32 difference, as numpy on float32 traces
        val = torch.where(live, torch.sqrt(torch.sum(r * r * dt, dim=-1)), torch.zeros_like(r[..., 0])).sum()
        ctx.save_for_backward(torch.where(live[..., None], r, torch.zeros_like(r)))
        ctx.dtype = syn.dtype
        return val

    @staticmethod
    def backward(ctx, g):
        (adj,) = ctx.saved_tensors
        return (g * adj).to(ctx.dtype), None, None


class _Envelope(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs, dt):
        p = 2.0
        s, o = syn.to(torch.float64), obs.to(torch.float64)
        live = _live(s, o)
        sh, oh = hilbert_imag(s), hilbert_imag(o)
        es = s ** 2 + sh ** 2
        eo = o ** 2 + oh ** 2
        rsd = es ** (p / 2) - eo ** (p / 2)
        d = p * es ** (p / 2 - 1)
        adj = d * s * rsd - hilbert_imag(d * sh * rsd)
        adj = torch.where(live[..., None], adj, torch.zeros_like(adj))
        val = torch.where(live, torch.sum(rsd * rsd, dim=-1), torch.zeros_like(rsd[..., 0])).sum() * dt
        ctx.save_for_backward(adj)
        ctx.dtype = syn.dtype
        return val

    @staticmethod
    def backward(ctx, g):
        (adj,) = ctx.saved_tensors
        return (g * adj).to(ctx.dtype), None, None


class _Traveltime(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs, dt):
        nt = syn.shape[-1]
        s, o = syn.to(torch.float64), obs.to(torch.float64)
        live = _live(s, o)
        cc = cross_correlate_max(o, s).to(torch.float64)
        adj = torch.zeros_like(s)
        adj[..., 1:-1] = (syn[..., 2:] - syn[..., :-2]).to(torch.float64) / (2.0 * dt)
        ok = live & (torch.sum(torch.abs(adj), dim=-1) > 0)
        norm = torch.sum(adj * adj, dim=-1) * dt
        scale = torch.where(ok, (cc - nt + 1) * dt / torch.where(ok, norm, torch.ones_like(norm)),
                            torch.zeros_like(norm))
        adj = adj * scale[..., None]
        val = torch.where(ok, 0.5 * (cc - nt + 1) ** 2 * dt, torch.zeros_like(norm)).sum()
        ctx.save_for_backward(adj)
        ctx.dtype = syn.dtype
        return val

    @staticmethod
    def backward(ctx, g):
        (adj,) = ctx.saved_tensors
        return (g * adj).to(ctx.dtype), None, None


class _GlobalCorrelation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs, dt):
        s, o = syn.to(torch.float64), obs.to(torch.float64)
        live = _live(s, o)
        sn = torch.linalg.vector_norm(s, dim=-1, keepdim=True)
        on = torch.linalg.vector_norm(o, dim=-1, keepdim=True)
        one = torch.ones_like(sn)
        shat = s / torch.where(sn > 0, sn, one)
        ohat = o / torch.where(on > 0, on, one)
        a = shat - shat.mean(dim=-1, keepdim=True)
        b = ohat - ohat.mean(dim=-1, keepdim=True)
        corr = (a * b).sum(-1) / torch.sqrt((a * a).sum(-1) * (b * b).sum(-1)).clamp_min(1e-300)
        adj = (shat * corr[..., None] - ohat) / torch.where(sn > 0, sn, one)
        adj = torch.where(live[..., None], adj, torch.zeros_like(adj))
        val = torch.where(live, -corr, torch.zeros_like(corr)).sum()
        ctx.save_for_backward(adj)
        ctx.dtype = syn.dtype
        return val

    @staticmethod
    def backward(ctx, g):
        (adj,) = ctx.saved_tensors
        return (g * adj).to(ctx.dtype), None, None


def waveform(syn, obs, dt):
    """L2 waveform misfit; gradient = syn - obs (misfit.py:128-148, 263-282)."""
    return _Waveform.apply(syn, obs, float(dt))


def envelope(syn, obs, dt):
    """Envelope misfit with its adjoint source (misfit.py:151-184, 285-309)."""
    return _Envelope.apply(syn, obs, float(dt))


def traveltime(syn, obs, dt):
    """Cross-correlation traveltime misfit (misfit.py:188-215, 312-334, 359-373)."""
    return _Traveltime.apply(syn, obs, float(dt))


def global_correlation(syn, obs, dt):
    """Normalised global-correlation misfit (misfit.py:219-242, 338-355)."""
    return _GlobalCorrelation.apply(syn, obs, float(dt))


MISFITS = {"waveform": waveform, "envelope": envelope, "traveltime": traveltime,
           "globalcorrelation": global_correlation}


def adjoint_source(syn, obs, dt, misfit_type):
    """(misfit value, adjoint source) of misfit_type ('Waveform', 'Envelope',
    'Traveltime', 'Globalcorrelation'), like toolbox/misfit.py:74-125 for one shot or a batch."""
    f = MISFITS[misfit_type.lower()]
    s = syn.detach().clone().requires_grad_(True)
    val = f(s, obs, dt)
    (g,) = torch.autograd.grad(val, s)
    return val.detach(), g
