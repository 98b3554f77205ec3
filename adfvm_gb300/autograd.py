"""The time-stepped solver as a differentiable torch operation.

``solve(solver, rho, rhoU, rhoE, S, nSteps, dt, checkpoint_every)`` runs ``nSteps`` SSP-RK3
steps on the GPU and returns the final state and the per-step objective (evaluated on the
stage-1 primitives, adFVM/density.py:412-413). Its backward pass is the reference's
checkpointed adjoint sweep (apps/adjoint.py:176-404): the forward keeps only every k-th state;
the backward recomputes the k states of a segment from its checkpoint, keeping each step's RK
stage states and, when a segment's tapes fit in 32 GB, its tape, then runs the
hand-written adjoint kernels (``afvm_adjoint_step``) through the segment in reverse, with the
objective seed of step n equal to the incoming gradient of objective n. dt is held fixed per
step (a fixed-step run, or the dt series recorded by the forward of an adaptive run), as in
the reference's adjoint. Gradients flow to the initial state and to the source terms.
"""
import torch


class _Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rho, rhoU, rhoE, S_rho, S_rhoU, S_rhoE, solver, nSteps, dt, k):
        S = (S_rho, S_rhoU, S_rhoE)
        x = (rho.detach().clone(), rhoU.detach().clone(), rhoE.detach().clone())
        dts = []
        objs = torch.zeros(nSteps, dtype=torch.float64, device=rho.device)
        checkpoints = {}
        cur_dt = float(dt)
        for n in range(nSteps):
            if n % k == 0:
                checkpoints[n] = tuple(t.clone() for t in x)
            out = (torch.empty_like(x[0]), torch.empty_like(x[1]), torch.empty_like(x[2]))
            r = solver.step(x[0], x[1], x[2], cur_dt, S=S, out=out)
            objs[n] = r[4]
            dts.append(cur_dt)
            x = out
            if not solver.fixedTimeStep:
                cur_dt = min(2 * solver.CFL / r[3], cur_dt * solver.stepFactor)
        ctx.solver, ctx.nSteps, ctx.k, ctx.dts = solver, nSteps, k, dts
        ctx.checkpoints = checkpoints
        ctx.save_for_backward(S_rho, S_rhoU, S_rhoE)
        return x[0], x[1], x[2], objs

    @staticmethod
    def backward(ctx, g_rho, g_rhoU, g_rhoE, g_obj):
        solver, nSteps, k, dts = ctx.solver, ctx.nSteps, ctx.k, ctx.dts
        S = ctx.saved_tensors
        a = [g if g is not None else torch.zeros_like(s) for g, s in zip((g_rho, g_rhoU, g_rhoE), S)]
        a = [t.contiguous().clone() for t in a]
        g_obj = torch.zeros(nSteps, dtype=torch.float64) if g_obj is None else g_obj.detach().double().cpu()
        Sbar = [torch.zeros_like(s) for s in S]
        starts = sorted(ctx.checkpoints)
        stages = [solver.stage_buffer() for _ in range(k)]
        taped = k * solver.tape_bytes <= 32e9
        tapes = [solver.tape_buffer() for _ in range(k)] if taped else [None] * k
        for s0 in reversed(starts):
            s1 = min(s0 + k, nSteps)
            # recompute the segment's input states, keeping each step's stages (and tape)
            states = [ctx.checkpoints[s0]]
            for n in range(s0, s1):
                x = states[-1]
                r = solver.step(x[0], x[1], x[2], dts[n], S=S, want_scalars=False, stages=stages[n - s0],
                                tape=tapes[n - s0])
                states.append(r[:3])
            for n in range(s1 - 1, s0 - 1, -1):
                x = states[n - s0]
                r = solver.adjoint_step(x[0], x[1], x[2], dts[n], a, obja=float(g_obj[n]), S=S, out=a,
                                        stages=stages[n - s0], tape=tapes[n - s0])
                for sb, g in zip(Sbar, r[3]):
                    sb += g
        return a[0], a[1], a[2], Sbar[0], Sbar[1], Sbar[2], None, None, None, None


def solve(solver, rho, rhoU, rhoE, S=None, nSteps=1, dt=None, checkpoint_every=20):
    """Differentiable nSteps of ``solver`` (an adfvm_gb300.solver.RCF on the GPU).

    Returns (rho, rhoU, rhoE, obj) with obj the (nSteps,) per-step objective."""
    if S is None:
        S = (torch.zeros_like(rho), torch.zeros_like(rhoU), torch.zeros_like(rhoE))
    return _Solve.apply(rho, rhoU, rhoE, S[0], S[1], S[2], solver, int(nSteps), float(dt), int(checkpoint_every))
