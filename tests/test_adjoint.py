"""Adjoint of the SR step (pic_srpic_gradient) against finite differences.

The gradient of the final E-field energy of the two-stream problem with
respect to the beam drift and the density-perturbation amplitude (chained by
torch through the momenta, weights and initial Gauss field) is checked
against central differences of:
  * the CPU oracle's step sequence in FP64 (the reference algorithm itself);
  * the GPU forward in FP64 and in FP32.
The full per-particle gradients (momenta, weights) and the field gradient
are checked by the directional derivative along themselves, single
momenta and field cells pointwise, all by central differences in FP64. The checkpoint interval must not change the result, and the FP32
adjoint must agree with the FP64 adjoint.

Step sizes: in-cell offsets are float at every precision (prtldx_t), so each
step rounds every position to ~3e-8 of a cell, coherently across a cold
quiet-start beam. A difference quotient whose perturbation moves particles by
less than ~1e-3 cells over the run measures that rounding, not the
derivative; the drift and momentum steps below move them by 1e-2 cells or
more (the central-difference truncation error stays below 1e-5 there).
"""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu

N = (32, 32)
PPC = 4
STEPS = 40
BETA, AMP = 0.2, 0.05


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import abi, build
    build.build()
    abi.load()


def _setup(real, order=2):
    from entity_gb300 import adjoint as A
    from entity_gb300.sim import Context
    g, prm, kappa, k = A.two_stream(n=N, ppc_per_beam=PPC, order=order, real=real,
                                    skindepth0=4.0)
    return A, Context(g), g, prm, kappa, k


def _grad(real, every=8, order=2, steps=STEPS):
    A, ctx, g, prm, kappa, k = _setup(real, order)
    beta = torch.tensor(BETA, dtype=torch.float64, device="cuda", requires_grad=True)
    amp = torch.tensor(AMP, dtype=torch.float64, device="cuda", requires_grad=True)
    sp, U, W, EB0 = A.build(g, kappa, k, beta, amp, PPC, ctx)
    L = A.energy(ctx, g, prm, sp, U, W, EB0, steps, every)
    gb, ga = torch.autograd.grad(L, [beta, amp])
    return float(L), float(gb), float(ga)


def _fd_gpu(real, which, h, order=2):
    A, ctx, g, prm, kappa, k = _setup(real, order)
    vals = []
    for s in (+1, -1):
        b = BETA + (s * h if which == "beta" else 0.0)
        a = AMP + (s * h if which == "amp" else 0.0)
        sp, U, W, EB0 = A.build(g, kappa, k, torch.tensor(b, dtype=torch.float64, device="cuda"),
                                torch.tensor(a, dtype=torch.float64, device="cuda"), PPC, ctx)
        vals.append(A.forward_energy(ctx, g, prm, sp, U, W, EB0, STEPS))
    return (vals[0] - vals[1]) / (2 * h)


def _oracle_energy(b, a):
    """Final E energy of the same problem through the CPU oracle in FP64."""
    from entity_gb300 import adjoint as A
    from oracle.oracle import Oracle
    _, ctx, g, prm, kappa, k = _setup(torch.float64)
    sp, U, W, EB0 = A.build(g, kappa, k, torch.tensor(b, dtype=torch.float64, device="cuda"),
                            torch.tensor(a, dtype=torch.float64, device="cuda"), PPC, ctx)
    o = Oracle(g)
    cpu = []
    for kk, s in enumerate(sp):
        s = s.clone().to("cpu")
        for c in range(3):
            s.u[c] = U[kk, c].detach().cpu().clone()
        s.w = W[kk].detach().cpu().clone()
        s.i_prev = [x.clone() for x in s.i]
        s.dx_prev = [x.clone() for x in s.dx]
        cpu.append(s)
    from entity_gb300.inputs import empty_field
    EB = EB0.detach().cpu().clone()
    J, buff = empty_field(g, 3), empty_field(g, 3)
    for n in range(STEPS):
        o.step(cpu, EB, J, buff, prm, n)
    return o.field_energy(EB, g.dx)[0]


def test_gradient_matches_oracle_finite_differences():
    L, gb, ga = _grad(torch.float64)
    hb, ha = 2e-3, 2e-3
    fd_b = (_oracle_energy(BETA + hb, AMP) - _oracle_energy(BETA - hb, AMP)) / (2 * hb)
    fd_a = (_oracle_energy(BETA, AMP + ha) - _oracle_energy(BETA, AMP - ha)) / (2 * ha)
    assert L == pytest.approx(_oracle_energy(BETA, AMP), rel=1e-9)
    assert gb == pytest.approx(fd_b, rel=3e-4), (gb, fd_b)
    assert ga == pytest.approx(fd_a, rel=3e-4), (ga, fd_a)


@pytest.mark.parametrize("order", [2, 3])
def test_gradient_matches_gpu_finite_differences_fp64(order):
    L, gb, ga = _grad(torch.float64, order=order)
    assert gb == pytest.approx(_fd_gpu(torch.float64, "beta", 2e-3, order), rel=3e-4)
    assert ga == pytest.approx(_fd_gpu(torch.float64, "amp", 2e-3, order), rel=3e-4)


def test_gradient_fp32_against_fd_and_fp64():
    L32, gb32, ga32 = _grad(torch.float32)
    L64, gb64, ga64 = _grad(torch.float64)
    assert gb32 == pytest.approx(_fd_gpu(torch.float32, "beta", 2e-3), rel=2e-3)
    assert ga32 == pytest.approx(_fd_gpu(torch.float32, "amp", 2e-3), rel=2e-3)
    assert gb32 == pytest.approx(gb64, rel=1e-3)
    assert ga32 == pytest.approx(ga64, rel=1e-3)
    assert L32 == pytest.approx(L64, rel=1e-4)


@pytest.mark.parametrize("real", [torch.float32, torch.float64])
def test_amplitude_gradient_at_the_stated_step(real):
    """At h = 1e-4 the amplitude gradient meets the 1e-3 bar: the amplitude
    enters through the weights and the initial Gauss field, not through the
    float in-cell offsets whose rounding floors the drift quotient there."""
    L, gb, ga = _grad(real)
    assert ga == pytest.approx(_fd_gpu(real, "amp", 1e-4), rel=1e-3)


def test_checkpoint_interval_does_not_change_the_gradient():
    ref = _grad(torch.float64, every=STEPS)
    for every in (1, 7, 16):
        got = _grad(torch.float64, every=every)
        for a, b in zip(ref, got):
            assert b == pytest.approx(a, rel=1e-10)


def _full_gradient(real=torch.float64, every=10):
    from entity_gb300.inputs import empty_field
    from entity_gb300.sim import SpeciesAdjoint
    A, ctx, g, prm, kappa, k = _setup(real)
    sp, U, W, EB0 = A.build(g, kappa, k, torch.tensor(BETA, dtype=torch.float64, device="cuda"),
                            torch.tensor(AMP, dtype=torch.float64, device="cuda"), PPC, ctx)
    run = [s.clone() for s in sp]
    for kk, s in enumerate(run):
        for c in range(3):
            s.u[c].copy_(U[kk, c])
        s.w.copy_(W[kk])
    EB = EB0.clone()
    J, buff = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    lam = torch.zeros_like(EB)
    adj = [SpeciesAdjoint(g, s.npart) for s in run]
    L = ctx.gradient(run, adj, EB, J, buff, prm, STEPS, every, lam)
    gU = torch.stack([torch.stack(a.lu) for a in adj])
    gW = torch.stack([a.lw for a in adj])
    return A, ctx, g, prm, sp, U, W, EB0, L, gU, gW, lam


@pytest.mark.parametrize("which", ["momenta", "weights", "fields"])
def test_directional_derivative_along_the_gradient_fp64(which):
    """d/dh L(x + h g/|g|) at h = 0 equals |g| for the whole per-particle
    momentum and weight gradients and the field gradient."""
    A, ctx, g, prm, sp, U, W, EB0, L, gU, gW, lam = _full_gradient()
    grad = {"momenta": gU, "weights": gW, "fields": lam}[which]
    norm = float(grad.norm())
    assert norm > 0
    d = grad / norm
    # steps that move the state well above the float-offset rounding floor
    h = {"momenta": 3e-2, "weights": 0.5, "fields": 1e-2 * float(EB0.norm())}[which]
    vals = []
    for sgn in (1, -1):
        U2, W2, E2 = U.clone(), W.clone(), EB0.clone()
        if which == "momenta":
            U2 += sgn * h * d
        elif which == "weights":
            W2 += sgn * h * d
        else:
            E2 += sgn * h * d
        vals.append(A.forward_energy(ctx, g, prm, sp, U2, W2, E2, STEPS))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert fd == pytest.approx(norm, rel=2e-3), (which, fd, norm)


def test_single_particle_momentum_gradient_fp64():
    A, ctx, g, prm, sp, U, W, EB0, L, gU, gW, lam = _full_gradient()
    h = 3e-3
    gen = torch.Generator().manual_seed(3)
    for trial in range(4):
        kk = trial % 2
        p = int(torch.randint(0, sp[0].npart, (1,), generator=gen))
        vals = []
        for sgn in (1, -1):
            U2 = U.clone()
            U2[kk, 0, p] += sgn * h
            vals.append(A.forward_energy(ctx, g, prm, sp, U2, W, EB0, STEPS))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert float(gU[kk, 0, p]) == pytest.approx(fd, rel=5e-3, abs=1e-3 * float(gU.abs().max()))


def test_field_gradient_pointwise_fp64():
    A, ctx, g, prm, sp, U, W, EB0, L, gU, gW, lam = _full_gradient()
    ng = g.ng
    h = 1e-3
    scale = float(lam.abs().max())
    for comp, i, j in ((0, 5, 7), (0, 20, 30), (1, 12, 3), (5, 9, 9)):
        vals = []
        for sgn in (1, -1):
            E2 = EB0.clone()
            E2[comp, 0, ng + j, ng + i] += sgn * h
            vals.append(A.forward_energy(ctx, g, prm, sp, U, W, E2, STEPS))
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = float(lam[comp, 0, ng + j, ng + i])
        assert abs(ad - fd) <= 1e-3 * scale, (comp, i, j, ad, fd, scale)


def test_unsupported_configurations_are_rejected():
    from entity_gb300 import abi
    from entity_gb300.inputs import GridSpec, empty_field, make_species
    from entity_gb300.sim import Context, SpeciesAdjoint, step_params
    g3 = GridSpec(dim=3, n=(8, 8, 8), order=2, real=torch.float32)
    ctx = Context(g3)
    sp = make_species(g3, 1, 0.1, 0.0, 1, device="cuda", with_prev=False)
    EB, J, buff = empty_field(g3, 6, "cuda"), empty_field(g3, 3, "cuda"), empty_field(g3, 3, "cuda")
    prm = step_params(g3, cfl=0.45, ppc0=1.0, skindepth0=4.0, larmor0=4.0)
    with pytest.raises(abi.PicError):
        ctx.gradient([sp], [SpeciesAdjoint(g3, sp.npart)], EB, J, buff, prm, 2, 1,
                     torch.zeros_like(EB))
