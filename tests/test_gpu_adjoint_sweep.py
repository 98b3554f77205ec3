"""The adjoint configuration of the workloads: periodic jittered 64^3 box, 400 FP64 steps,
objective the time average of the volume-integrated kinetic energy over the last 200 steps,
gradient with respect to the initial state by the checkpointed adjoint (checkpoints every 20
steps), checked against central finite differences (step 1e-6 relative to each field's
magnitude) on 16 seeded random directions and one along the gradient.

Random directions in a 1.3-million-dimensional state are nearly orthogonal to the gradient
(|<g,v>| ~ 1e-4 |g| |v|), so their finite differences are dominated by the round-off of J;
the error is therefore measured against |g| |v| (the Cauchy-Schwarz scale of <g, v>) there,
and relative to <g, v> itself on the direction along the gradient."""
import numpy as np
import pytest
import torch

from adfvm_gb300 import cases
from adfvm_gb300.autograd import solve
from adfvm_gb300.solver import RCF

pytestmark = pytest.mark.gpu


def test_box64_400_steps_adjoint_vs_central_differences():
    case = cases.box(64, objective='kinetic_energy')
    mesh = case.build_mesh()
    rcf = RCF(mesh, case.bc, objective=case.objective, **case.config)
    x0 = [torch.as_tensor(a).cuda() for a in cases.conservative(case)]
    nSteps, avg = 400, 200
    w = torch.zeros(nSteps, dtype=torch.float64, device='cuda')
    w[avg:] = 1.0 / (nSteps - avg)

    def J_of(x):
        with torch.no_grad():
            y = list(x)
            acc = 0.0
            for n in range(nSteps):
                y0, y1, y2, dtc, obj = rcf.step(y[0], y[1], y[2], case.dt)
                y = [y0, y1, y2]
                if n >= avg:
                    acc += obj / (nSteps - avg)
            return acc

    xs = [t.clone().requires_grad_(True) for t in x0]
    r = solve(rcf, xs[0], xs[1], xs[2], None, nSteps=nSteps, dt=case.dt, checkpoint_every=20)
    J = (r[3] * w).sum()
    g = torch.autograd.grad(J, xs)
    assert abs(float(J.detach()) - J_of(x0)) <= 1e-12 * abs(float(J.detach()))
    rng = np.random.default_rng(3)
    scale = [float(t.abs().max()) for t in x0]
    # gradient norm in the same scaled space as the directions
    gnorm = float(torch.sqrt(sum((gi * s).pow(2).sum() for gi, s in zip(g, scale))))
    h = 1e-6

    def check(v):
        fd = (J_of([t + h * vi for t, vi in zip(x0, v)]) - J_of([t - h * vi for t, vi in zip(x0, v)])) / (2 * h)
        ad = sum(float((gi * vi).sum()) for gi, vi in zip(g, v))
        return fd, ad

    errs = []
    for k in range(16):
        v = [torch.as_tensor(rng.standard_normal(tuple(t.shape))).cuda() * s for t, s in zip(x0, scale)]
        norm = float(torch.sqrt(sum((vi / s).pow(2).sum() for vi, s in zip(v, scale))))
        v = [vi / norm for vi in v]
        fd, ad = check(v)
        errs.append(abs(fd - ad) / gnorm)
    assert max(errs) < 1e-6, errs
    # along the gradient: <g, v> = |g|, relative error of the finite difference itself
    v = [gi * s * s / gnorm for gi, s in zip(g, scale)]
    fd, ad = check(v)
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
