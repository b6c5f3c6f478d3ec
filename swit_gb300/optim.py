"""SWIT's optimiser loop on device (torch, float64 state vectors).

Restates toolbox/inversion.py:
    nlcg_direction      NLCG            111-171  (Polak-Ribiere, periodic restart after 6)
    lbfgs_direction     LBFGS           174-271  (memory 5; S, Y kept on the device instead
                                                   of the disk memmap of :212-223)
    backtrack           backtrack       274-350  (halving steps, at most 6 trials, safeguard
                                                   step for L-BFGS)
    decide              desicion_make   410-459
    model_update        model_update    474-482
    pollak_ribere, check_descent        485-506
and runs it with the engine's gradient (`fwi`): misfit and preconditioned
gradient from a callable, every vector staying on the GPU.
"""
import copy

import torch


def pollak_ribere(g_now, g_old):
    """Polak-Ribiere beta (inversion.py:485-492)."""
    return torch.dot(g_now, g_now - g_old) / torch.dot(g_old, g_old)


def check_descent(d_now, g_now):
    """<d, g> / <g, g>: positive when d is not a descent direction (inversion.py:501-505)."""
    return torch.dot(d_now, g_now) / torch.dot(g_now, g_now)


def model_update(vp, update, vpmax, vpmin):
    """vp + update clipped to [vpmin, vpmax] (inversion.py:474-482)."""
    return torch.clamp(vp + update, min=vpmin, max=vpmax)


def init_state(scheme, n, device="cuda", memory=5):
    """optimize_init (inversion.py:353-407)."""
    z = torch.zeros(n, dtype=torch.float64, device=device)
    st = dict(scheme=scheme, g_now=z, g_old=z, d_now=z, d_old=z, v_old=z, v_now=z, v_try=z, f_old=0.0, f_now=0.0,
              f_try=0.0, ls_iter=0, ls_status=0, ls_step=0.0, log=[])
    if scheme == "NLCG":
        st["cg_it"] = 0
    elif scheme == "LBFGS":
        st.update(memory=memory, memory_used=0, lbfgs_it=0,
                  S=torch.zeros((memory, n), dtype=torch.float64, device=device),
                  Y=torch.zeros((memory, n), dtype=torch.float64, device=device))
    else:
        raise ValueError("not supported inversion scheme: %s" % scheme)
    return st


def nlcg_direction(st, cg_itmax=6):
    """NLCG search direction with restarts (inversion.py:111-171)."""
    g_now, g_old, d_old = st["g_now"], st["g_old"], st["d_old"]
    st["cg_it"] += 1
    if st["cg_it"] == 1:
        d_now, status = -g_now, 0
    elif st["cg_it"] > cg_itmax:
        d_now, status = -g_now, 1
        st["log"].append("restarting NLCG... [periodic restart]")
    else:
        beta = float(pollak_ribere(g_now, g_old))
        if beta <= 0.0:
            beta, status = 0.0, 1
            st["log"].append("restarting NLCG... [negative beta]")
        else:
            status = 0
        d_now = -g_now + beta * d_old
    if float(check_descent(d_now, g_now)) > 0.0:
        d_now, status = -g_now, 1
        st["log"].append("restarting NLCG... [not a descent direction]")
    if status:
        st["cg_it"] = 0
    st["d_now"] = d_now
    return st


def lbfgs_direction(st):
    """L-BFGS two-loop direction with memory 5 and restarts (inversion.py:174-271)."""
    g_now, g_old, v_now, v_old = st["g_now"], st["g_old"], st["v_now"], st["v_old"]
    S, Y = st["S"], st["Y"]
    st["lbfgs_it"] += 1
    if st["lbfgs_it"] == 1:
        d_now, status = -g_now, 0
    else:
        s, y = v_now - v_old, g_now - g_old
        if st["memory_used"] == 0:
            S[0], Y[0] = s, y
            st["memory_used"] = 1
        else:
            S[1:] = S[:-1].clone()
            Y[1:] = Y[:-1].clone()
            S[0], Y[0] = s, y
            if st["memory_used"] < st["memory"]:
                st["memory_used"] += 1
        k = st["memory_used"]
        rho, alpha = [0.0] * k, [0.0] * k
        q = g_now
        for i in range(k):
            rho[i] = 1.0 / torch.dot(Y[i], S[i])
            alpha[i] = rho[i] * torch.dot(S[i], q)
            q = q - alpha[i] * Y[i]
        z = (torch.dot(Y[0], S[0]) / torch.dot(Y[0], Y[0])) * q
        for i in range(k - 1, -1, -1):
            beta = rho[i] * torch.dot(Y[i], z)
            z = z + (alpha[i] - beta) * S[i]
        if float(check_descent(-z, g_now)) > 0:
            d_now, status = -g_now, 1
            st["log"].append("restarting LBFGS... [not a descent direction]")
        else:
            d_now, status = -z, 0
    if status:
        st["lbfgs_it"] = 1
        st["memory_used"] = 0
        S.zero_()
        Y.zero_()
    st["d_now"] = d_now
    return st


def backtrack_steps(st, step_length, vpmax, vpmin, dec=0.5, search_max=6, vmax_thresh=300.0, vmin_thresh=20.0):
    """inversion.py:274-350 as a generator: yields each trial model vector, is sent
    its misfit, and returns the updated state (StopIteration.value)."""
    v_now, d_now, f_now = st["v_now"], st["d_now"], st["f_now"]
    if st["scheme"] == "LBFGS" and st["lbfgs_it"] != 1:
        dmax = float(d_now.abs().max())
        step = vmax_thresh / dmax if dmax > vmax_thresh else (vmin_thresh / dmax if dmax < vmin_thresh else 1.0)
    else:
        step = step_length
    ls_iter = 0
    while True:
        ls_iter += 1
        v_try = model_update(v_now, d_now * step, vpmax, vpmin)
        f_try = float((yield v_try))
        if f_try < f_now:
            st.update(ls_status=0, ls_iter=ls_iter, ls_step=step, f_try=f_try, v_try=v_try)
            st["log"].append("line search: step = %.4f, f_now = %.4e, f_try = %.4e. Succeed." % (step, f_now, f_try))
            return st
        st["log"].append("line search: step = %.4f, f_now = %.4e, f_try = %.4e. Not decrease." % (step, f_now, f_try))
        if ls_iter >= search_max:
            st.update(ls_status=-1, ls_iter=ls_iter, ls_step=step, f_try=f_try, v_try=v_try)
            st["log"].append("line search fails: exceed the iteration of linesearch.")
            return st
        step = step * dec


def backtrack(st, misfit_of, step_length, vpmax, vpmin, dec=0.5, search_max=6, vmax_thresh=300.0,
              vmin_thresh=20.0):
    """inversion.py:274-350; misfit_of(v) evaluates the misfit of a trial model vector."""
    gen = backtrack_steps(st, step_length, vpmax, vpmin, dec, search_max, vmax_thresh, vmin_thresh)
    v = next(gen)
    while True:
        try:
            v = gen.send(misfit_of(v))
        except StopIteration as done:
            return done.value


def decide(st):
    """desicion_make (inversion.py:410-459): accept the trial model or restart."""
    if st["scheme"] == "NLCG":
        if st["ls_status"] == -1 and st["cg_it"] > 1:
            st["cg_it"] = 0
            st["g_old"] = st["g_old"] * 0.0
            st["d_old"] = st["d_old"] * 0.0
        else:
            st["g_old"], st["d_old"] = st["g_now"], st["d_now"]
            st["f_old"], st["f_now"] = st["f_now"], st["f_try"]
            st["v_now"] = st["v_try"]
    else:
        if st["ls_status"] == -1:
            old = st
            st = init_state("LBFGS", old["v_now"].numel(), device=old["v_now"].device, memory=old["memory"])
            st.update(v_old=old["v_now"], v_now=old["v_now"], f_now=old["f_now"], g_now=old["g_now"],
                      d_now=old["d_now"], log=old["log"])
        else:
            st["g_old"], st["v_old"], st["v_now"] = st["g_now"], st["v_now"], st["v_try"]
            st["f_old"], st["f_now"] = st["f_now"], st["f_try"]
    return st


def fwi(v0, objective, misfit_of, scheme="LBFGS", maxiter=5, step_length=0.02, vpmax=5000.0, vpmin=1000.0):
    """The inversion loop of inversion.py:30-80 on device.

    objective(v) -> (misfit, preconditioned gradient vector) of model vector v;
    misfit_of(v) -> misfit only (line-search trials).  Returns (final state, history).
    """
    v0 = torch.as_tensor(v0, dtype=torch.float64)
    st = init_state(scheme, v0.numel(), device=v0.device)
    st["v_now"] = v0.clone()
    st["v_old"] = v0.clone()
    hist = []
    for it in range(1, maxiter + 1):
        f, g = objective(st["v_now"])
        st["f_now"], st["g_now"] = float(f), torch.as_tensor(g, dtype=torch.float64, device=v0.device)
        st = nlcg_direction(st) if scheme == "NLCG" else lbfgs_direction(st)
        st = backtrack(st, misfit_of, step_length, vpmax, vpmin)
        st = decide(st)
        hist.append(dict(iteration=it, f=st["f_now"], step=st["ls_step"], ls_status=st["ls_status"]))
    return st, hist


def fwi_lockstep(v0s, objective_all, misfit_all, scheme="LBFGS", maxiter=5, step_length=0.02, vpmax=5000.0,
                 vpmin=1000.0):
    """fwi for many independent problems at once: each iteration evaluates every
    problem's objective in one call, then runs the problems' line searches in
    lockstep rounds, one misfit_all call per round.  objective_all(vs) ->
    [(f, g)]; misfit_all(vs, active) -> [f], where only the problems with
    active[i] true are still searching (the others' values are not used).  Every problem follows the same iterates as fwi()
    would give it alone.  Returns (states, histories)."""
    sts, hists = [], []
    for v0 in v0s:
        v0 = torch.as_tensor(v0, dtype=torch.float64)
        st = init_state(scheme, v0.numel(), device=v0.device)
        st["v_now"] = v0.clone()
        st["v_old"] = v0.clone()
        sts.append(st)
        hists.append([])
    for it in range(1, maxiter + 1):
        fg = objective_all([st["v_now"] for st in sts])
        gens, trials, active = [], [], []
        for st, (f, g) in zip(sts, fg):
            st["f_now"], st["g_now"] = float(f), torch.as_tensor(g, dtype=torch.float64, device=st["v_now"].device)
            st = nlcg_direction(st) if scheme == "NLCG" else lbfgs_direction(st)
            gen = backtrack_steps(st, step_length, vpmax, vpmin)
            gens.append(gen)
            trials.append(next(gen))
            active.append(True)
        while any(active):
            fs = misfit_all(trials, list(active))
            for i in range(len(sts)):
                if not active[i]:
                    continue
                try:
                    trials[i] = gens[i].send(fs[i])
                except StopIteration as done:
                    sts[i] = done.value
                    active[i] = False
        for i in range(len(sts)):
            sts[i] = decide(sts[i])
            hists[i].append(dict(iteration=it, f=sts[i]["f_now"], step=sts[i]["ls_step"],
                                 ls_status=sts[i]["ls_status"]))
    return sts, hists
