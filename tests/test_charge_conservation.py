"""Charge conservation of the deposit and of the whole step.

Esirkepov's weights (currents_deposit.hpp:406-754) satisfy the discrete
continuity equation
    (rho_after - rho_before) / dt + D^- J = 0
node by node, with rho the unstaggered order-O shape density and D^- the
backward difference of J's staggered components; the zigzag fluxes
(currents_deposit.hpp:108-405) satisfy it for the linear density with the
caveats of `tol`. Ampere's update E += c curl B + jcoeff J changes D^- E only
through J, because the discrete divergence of the Yee curl vanishes, so over
N steps
    D^- (E_N - E_0) + jcoeff / dt * (rho_N - rho_0) = 0
at round-off (jcoeff = -dt q0 / (B0 V0), the coefficient CurrentsAmpere
applies to J). The 3D single-precision weights carry THIRD = 0.333333f
(numeric.h:41), so there the residual is ~1e-6 of the charge change instead
of pure round-off; the tolerances below say so.

The CPU tests pin the oracle; the GPU tests check the CUDA path (per-particle
and tiled deposits, and the engine step with the cell sort) with the same bar.
"""
import pytest
import torch

from entity_gb300.inputs import GridSpec, empty_field, make_species
from tests.helpers import active, random_fields

REALS = [torch.float32, torch.float64]
# residual / max|charge change / dt|: FP32 round-off of the weights, of the
# charge density's atomic sums (order-dependent) and of the difference of two
# densities; 2D order 3 has reached 5.0e-6, so the FP32 2D bar is 1e-5
TOL = {(torch.float32, 2): 1e-5, (torch.float32, 3): 2e-5,
       (torch.float64, 2): 1e-12, (torch.float64, 3): 1e-12}


def tol(real, dim, order):
    """The zigzag deposit (order 0) forms its relay point in the float offset
    type at every precision (currents_deposit.hpp:175-192), so it conserves
    charge to float round-off only; in 3D its transverse weights are midpoint
    products (currents_deposit.hpp:270-404), which omit the dy dz / 12 term of
    the exact trilinear flux: conservation there is second order in the step,
    a property of the scheme."""
    if order == 0:
        return 1e-2 if dim == 3 else 5e-6
    return TOL[(real, dim)]


def _grid(dim, order, real):
    n = (32, 24, 1) if dim == 2 else (12, 10, 8)
    return GridSpec(dim=dim, n=n, order=order, real=real)


def backward_div(g, F):
    """D^- of the three staggered components of F (ghost-inclusive), on the
    active nodes, in FP64."""
    F = F.double()
    d = (F[0] - torch.roll(F[0], 1, dims=-1)) + (F[1] - torch.roll(F[1], 1, dims=-2))
    if g.dim == 3:
        d = d + (F[2] - torch.roll(F[2], 1, dims=-3))
    return active(g, d.unsqueeze(0))[0]


def continuity_residual(g, J, rho0, rho1, dt):
    drho = active(g, (rho1[:1].double() - rho0[:1].double()))[0] / dt
    res = backward_div(g, J) + drho
    return float(res.abs().max()), float(drho.abs().max())


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_deposit_conserves_charge(dim, order, real):
    from oracle.oracle import Oracle
    g = _grid(dim, order, real)
    o = Oracle(g)
    sp = [make_species(g, 3, 0.3, 0.2, 41, charge=-1.0),
          make_species(g, 3, 0.3, -0.2, 42, charge=1.0, index=2)]
    EB = random_fields(g, 5, amp=0.2)
    dt = 0.45 / dim ** 0.5
    rho0, rho1 = empty_field(g, 3), empty_field(g, 3)
    J, buff = empty_field(g, 3), empty_field(g, 3)
    o.charge_density(sp, rho0)
    for s in sp:
        o.push(s, EB, dt, 0.1, g.dx)
    o.deposit(sp, J, dt, g.dx)
    o.charge_density(sp, rho1)
    for f in (J, rho0, rho1):
        o.sync_currents(f, buff)
        o.fill_ghosts(f, False, 0, 3)
    res, scale = continuity_residual(g, J, rho0, rho1, dt)
    assert scale > 0
    assert res <= tol(real, dim, order) * scale, (res, scale)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_charge_density_sums_to_total_charge(dim, real):
    from oracle.oracle import Oracle
    g = _grid(dim, 2, real)
    o = Oracle(g)
    sp = make_species(g, 2, 0.1, 0.0, 7, charge=-1.0)
    rho, buff = empty_field(g, 3), empty_field(g, 3)
    o.charge_density([sp], rho)
    o.sync_currents(rho, buff)
    o.fill_ghosts(rho, False, 0, 3)
    tot = float(active(g, rho[:1].double()).sum())
    assert tot == pytest.approx(-float(sp.npart), rel=1e-5 if real == torch.float32 else 1e-12)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import abi, build
    build.build()
    abi.load()


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("tiled", [False, True])
def test_gpu_deposit_conserves_charge(_lib, dim, order, real, tiled):
    from entity_gb300 import abi
    from entity_gb300.sim import Context
    g = _grid(dim, order, real)
    ctx = Context(g)
    sp = [make_species(g, 3, 0.3, 0.2, 41, charge=-1.0, device="cuda", with_prev=False),
          make_species(g, 3, 0.3, -0.2, 42, charge=1.0, index=2, device="cuda", with_prev=False)]
    if tiled:
        for s in sp:
            ctx.sort(s, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED | abi.PIC_SORT_SKIP_PREV)
    EB = random_fields(g, 5, amp=0.2, device="cuda")
    dt = 0.45 / dim ** 0.5
    rho0, rho1 = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    J, buff = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    ctx.charge_density(sp, rho0)
    ctx.push_deposit(sp, EB, J, dt, 0.1, g.dx)
    ctx.charge_density(sp, rho1)
    for f in (J, rho0, rho1):
        ctx.sync_currents(f, buff)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    res, scale = continuity_residual(g, J.cpu(), rho0.cpu(), rho1.cpu(), dt)
    assert scale > 0
    assert res <= tol(real, dim, order) * scale, (res, scale)


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_charge_density_matches_oracle(_lib, dim, order, real):
    from oracle.oracle import Oracle
    from entity_gb300.sim import Context
    g = _grid(dim, order, real)
    sp = make_species(g, 3, 0.3, 0.2, 43, charge=-1.0)
    rho_o = empty_field(g, 3)
    Oracle(g).charge_density([sp], rho_o)
    rho_g = empty_field(g, 3, "cuda")
    Context(g).charge_density([sp.clone().to("cuda")], rho_g)
    scale = float(rho_o.abs().max())
    diff = float((rho_o.double() - rho_g.cpu().double()).abs().max())
    assert diff <= (4e-6 if real == torch.float32 else 1e-13) * scale


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_particle_moments_match_oracle(_lib, dim, real):
    from oracle.oracle import Oracle
    from entity_gb300.sim import Context
    g = _grid(dim, 2, real)
    sp = [make_species(g, 4, 0.5, 0.3, 44, charge=-1.0),
          make_species(g, 4, 0.5, -0.3, 45, charge=1.0, index=2, mass=2.0)]
    sp[0].tag[::7] = 0
    mo = Oracle(g).particle_moments(sp)
    mg = Context(g).particle_moments([s.clone().to("cuda") for s in sp])
    for a, b in zip(mo, mg):
        assert b == pytest.approx(a, rel=1e-12, abs=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_gauss_law_over_steps(_lib, dim, order, real):
    """div E - jcoeff/dt * rho stays constant over engine steps (no filter),
    with the tiled deposit and a cell sort every 2 steps."""
    from entity_gb300.inputs import turbulent_field
    from entity_gb300.sim import Context, step_params
    g = _grid(dim, order, real)
    ctx = Context(g)
    sp = [make_species(g, 4, 0.2, 0.1, 51, charge=-1.0, device="cuda", with_prev=False),
          make_species(g, 4, 0.2, -0.1, 52, charge=1.0, index=2, device="cuda",
                       with_prev=False)]
    EB = turbulent_field(g, 0.1, 1.0, 4, seed=3, device="cuda")
    J, buff = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    prm = step_params(g, cfl=0.45, ppc0=8.0, skindepth0=5.0, larmor0=5.0, nfilter=0,
                      sort_interval=2, write_prev=False, sort_tiled=True)
    jc = -float(prm.dt) * float(prm.q0) / (float(prm.B0) * float(prm.V0))
    rho0 = empty_field(g, 3, "cuda")
    ctx.fill_ghosts(EB, True, 0, 6)
    ctx.charge_density(sp, rho0)
    ctx.sync_currents(rho0, buff)
    E0 = EB[:3].clone()
    nsteps = 8
    for k in range(nsteps):
        ctx.step(sp, EB, J, buff, prm, k)
    ctx.fill_ghosts(EB, True, 0, 6)
    rho1 = empty_field(g, 3, "cuda")
    ctx.charge_density(sp, rho1)
    ctx.sync_currents(rho1, buff)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    dE = backward_div(g, (EB[:3].double() - E0.double()).cpu())
    drho = active(g, (rho1[:1].double() - rho0[:1].double()).cpu())[0] * (jc / float(prm.dt))
    scale = float(drho.abs().max())
    res = float((dE + drho).abs().max())
    assert scale > 0
    # per step: the deposit's residual, plus one rounding of every E
    # component in the field precision (a few ulp of |E| per node in D^-)
    eps = 6e-8 if real == torch.float32 else 1.2e-16
    emax = float(EB[:3].abs().max())
    tol = nsteps * (TOL[(real, dim)] * scale + 16 * eps * emax)
    assert res <= tol, (res, scale, emax)
