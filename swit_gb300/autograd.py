"""torch.autograd wrapper: seismograms = F(vp) with the engine's reverse loop as
the backward, so misfits written in torch get their adjoint sources from autograd.

    seis = propagate(engine, vp, rho, src)      # (ns, ng_max, nt), CUDA tensor
    loss = misfit(seis, obs); loss.backward()   # vp.grad filled by the engine

Backward feeds dL/dseis to the reverse loop as the adjoint source (what
toolbox/solver.py:72-75 writes to parfile/adjoint_source) and returns the
reference's vp kernel g = -2/c sum_t p_f (p_b(t+1) - p_b(t))
(fd2dmpi/solver.f90:237, 270) divided by dt.  The reference's adjoint injects
dt * r (fdcore.f90:351-356), so g/dt approximates dL/dvp; it is the
continuous-adjoint imaging gradient of fd2dmpi, not the exact transpose of the
discrete forward map (its agreement with central finite differences is
measured by tests/test_gpu_solver.py and tests/test_gpu_correlation.py).

With an engine created with adjoint="exact" the backward is the exact
transpose of the discrete forward map instead (swit_backward_exact): vp.grad
is dL/dvp with the damping profile held fixed (it follows vp only through
vmin), and src.grad is dL/dsrc; torch.autograd.gradcheck holds with the FP64
build (tests/test_gpu_exact.py).

If the engine ran another forward between this forward and its backward, the
boundary strips (or, for the exact adjoint, the stored divergence terms) are
recomputed first.
"""
import torch


class _Propagate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vp, rho, src, engine):
        engine.set_model(vp.detach().contiguous().float(), rho.detach().contiguous().float())
        seis = engine.forward(src.detach().contiguous().float(), save_boundary=True)
        engine._generation = getattr(engine, "_generation", 0) + 1
        ctx.engine = engine
        ctx.generation = engine._generation
        ctx.save_for_backward(vp, rho, src)
        return seis

    @staticmethod
    def backward(ctx, grad_seis):
        engine = ctx.engine
        vp, rho, src = ctx.saved_tensors
        if engine._generation != ctx.generation:
            engine.set_model(vp.detach().contiguous().float(), rho.detach().contiguous().float())
            engine.forward(src.detach().contiguous().float(), save_boundary=True)
            engine._generation += 1
        adj = grad_seis.detach().contiguous().float()
        if getattr(engine, "adjoint", "fd2dmpi") == "exact":
            g, gs = engine.backward_exact(adj)
            return g.to(vp.dtype), None, (gs.to(src.dtype) if ctx.needs_input_grad[2] else None), None
        g, _, _ = engine.backward(adj)
        g = g / engine.dt
        return g.to(vp.dtype), None, None, None


def propagate(engine, vp, rho, src):
    """Differentiable forward modeling of every shot: gradients w.r.t. vp, and
    w.r.t. src for exact-adjoint engines."""
    return _Propagate.apply(vp, rho, src, engine)
