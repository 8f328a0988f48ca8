"""Gradient harness for the adjoint of the SR step (pic_srpic_gradient).

`EnergyAfterSteps` is a torch.autograd.Function whose forward runs the
product step `nsteps` times from (momenta, weights, E/B) and returns the final
E-field energy, and whose backward returns the adjoint computed by the C ABI
(checkpoint-and-recompute). Torch only chains the gradient to whatever
parameters built those initial arrays, e.g. the two-stream set-up below
(drift velocity -> momenta, perturbation amplitude -> weights and the initial
Gauss field). Every step and every adjoint step runs in libentity_pic.so.

The two-stream set-up follows the reference's pgens/streaming/twostream
problem: two cold beams at +-beta along x1 with weights 1 + amp cos(k x1),
k = 2 pi / L, on an immobile neutralising background, and the initial E1
that solves the discrete Gauss law of the scheme, D^- E1 = kappa (rho -
mean rho) with kappa = q0 / (B0 V0) (the constant for which the deposit's
continuity equation keeps D^- E - kappa rho fixed).
"""
import math

import torch

from .inputs import GridSpec, SpeciesArrays, empty_field
from .sim import Context, SpeciesAdjoint, step_params


def quiet_beam(g: GridSpec, ppc: int, beta: torch.Tensor, weights, *, charge=-1.0, index=1,
               device="cuda"):
    """`ppc` (a square) particles per cell on a regular in-cell lattice, all
    with u1 = gamma beta, in cell order. `weights(x1)` gives each weight from
    the particle's x1 coordinate (cells)."""
    m = int(round(math.sqrt(ppc)))
    assert m * m == ppc and g.dim == 2
    n1, n2 = g.n[0], g.n[1]
    ncell = n1 * n2
    cell = torch.arange(ncell, device=device, dtype=torch.int64).repeat_interleave(ppc)
    sub = torch.arange(ppc, device=device, dtype=torch.int64).repeat(ncell)
    i1 = (cell // n2).to(torch.int32)
    i2 = (cell % n2).to(torch.int32)
    dx1 = ((sub // m).to(torch.float64) + 0.5) / m
    dx2 = ((sub % m).to(torch.float64) + 0.5) / m
    dx1, dx2 = dx1.to(torch.float32), dx2.to(torch.float32)
    npart = ncell * ppc
    x1 = i1.to(torch.float64) + dx1.to(torch.float64)
    w = weights(x1).to(g.real)
    gamma_beta = beta / torch.sqrt(1.0 - beta * beta)
    u1 = (torch.ones(npart, dtype=torch.float64, device=device) * gamma_beta).to(g.real)
    z = lambda dt: torch.zeros(npart, dtype=dt, device=device)
    return SpeciesArrays([i1, i2, z(torch.int32)], [dx1, dx2, z(torch.float32)], [None] * 3,
                         [None] * 3, [u1, z(g.real), z(g.real)], w,
                         torch.ones(npart, dtype=torch.int16, device=device), 1.0, charge, 1,
                         npart, index)


def gauss_field(ctx: Context, g: GridSpec, species, kappa: float):
    """E1 solving D^- E1 = kappa (rho - mean rho) for a density uniform in x2
    (as the quiet beams make it); E2 = E3 = 0, B = 0."""
    rho = empty_field(g, 3, "cuda")
    ctx.charge_density(species, rho)
    ctx.sync_currents(rho)
    ng = g.ng
    r = rho[0, 0, ng:-ng, ng:-ng].double().mean(dim=0)   # along x1
    r = r - r.mean()
    E1 = kappa * torch.cumsum(r, 0)
    E1 = E1 - E1.mean()
    EB = empty_field(g, 6, "cuda")
    EB[0, 0, ng:-ng, ng:-ng] = E1.to(g.real).unsqueeze(0)
    ctx.fill_ghosts(EB, True, 0, 6)
    return EB


class EnergyAfterSteps(torch.autograd.Function):
    """L = E-field energy after `nsteps` steps of the species (positions fixed
    inputs) from momenta U (nspecies x 3 x npart), weights W (nspecies x
    npart) and fields EB0; backward through pic_srpic_gradient."""

    @staticmethod
    def forward(fctx, U, W, EB0, run):
        ctx, g, species, prm, nsteps, every = run
        sp = [s.clone() for s in species]
        for k, s in enumerate(sp):
            for c in range(3):
                s.u[c].copy_(U[k, c].detach())
            s.w.copy_(W[k].detach())
        EB = EB0.detach().clone()
        J, buff = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
        lam = torch.zeros_like(EB)
        adj = [SpeciesAdjoint(g, s.npart) for s in sp]
        loss = ctx.gradient(sp, adj, EB, J, buff, prm, nsteps, every, lam)
        fctx.save_for_backward(
            torch.stack([torch.stack(a.lu) for a in adj]), torch.stack([a.lw for a in adj]), lam)
        return torch.tensor(loss, dtype=torch.float64, device=U.device)

    @staticmethod
    def backward(fctx, gL):
        LU, LW, lam = fctx.saved_tensors
        s = gL.to(LU.dtype)
        return LU * s, LW * s, lam * s, None


def two_stream(n=(256, 256), ppc_per_beam=16, order=2, real=torch.float32, skindepth0=10.0,
               cfl=0.45):
    """Grid, step parameters and the fixed (position) part of the two-stream
    set-up; the momenta, weights and field come from `build`."""
    g = GridSpec(dim=2, n=(n[0], n[1], 1), order=order, real=real)
    prm = step_params(g, cfl=cfl, ppc0=2.0 * ppc_per_beam, skindepth0=skindepth0,
                      larmor0=skindepth0, nfilter=0, sort_interval=0, write_prev=False)
    kappa = float(prm.q0) / (float(prm.B0) * float(prm.V0))
    k = 2.0 * math.pi / n[0]
    return g, prm, kappa, k


def build(g, kappa, k, beta, amp, ppc_per_beam=16, ctx=None):
    """Differentiable initial state of the two-stream problem: beta and amp
    are 0-d tensors (requires_grad allowed). Returns (species, U, W, EB0)."""
    ctx = ctx or Context(g)
    b = beta.detach()
    sp = [quiet_beam(g, ppc_per_beam, b, lambda x: 1.0 + 0.0 * x, index=1),
          quiet_beam(g, ppc_per_beam, -b, lambda x: 1.0 + 0.0 * x, index=2)]
    x1 = sp[0].i[0].double() + sp[0].dx[0].double()
    cosk = torch.cos(k * x1)
    # E for unit amplitude: weights cos(k x1) on both beams
    unit = [s.clone() for s in sp]
    for s in unit:
        s.w.copy_(cosk.to(g.real))
    Ehat = gauss_field(ctx, g, unit, kappa)
    gb = (beta / torch.sqrt(1.0 - beta * beta)).to(torch.float64)
    n = sp[0].npart
    ones = torch.ones(n, dtype=torch.float64, device="cuda")
    zero = torch.zeros(n, dtype=torch.float64, device="cuda")
    U = torch.stack([torch.stack([gb * ones, zero, zero]),
                     torch.stack([-gb * ones, zero, zero])])
    W = (1.0 + amp * cosk).unsqueeze(0).expand(2, -1)
    EB0 = amp * Ehat.double()
    return sp, U.to(g.real), W.to(g.real), EB0.to(g.real)


def energy(ctx, g, prm, species, U, W, EB0, nsteps, every):
    return EnergyAfterSteps.apply(U, W, EB0, (ctx, g, species, prm, nsteps, every))


def forward_energy(ctx, g, prm, species, U, W, EB0, nsteps):
    """The plain forward (no adjoint) for finite differences and timing."""
    sp = [s.clone() for s in species]
    for k, s in enumerate(sp):
        for c in range(3):
            s.u[c].copy_(U[k, c].detach())
        s.w.copy_(W[k].detach())
    EB = EB0.detach().clone()
    J, buff = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    for n in range(nsteps):
        ctx.step(sp, EB, J, buff, prm, n)
    return ctx.field_energy(EB, g.dx)[0]
