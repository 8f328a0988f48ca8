"""SR field boundaries on non-periodic sides (srpic::FieldBoundaries,
src/engines/srpic/fields_bcs.h:622-672): the perfect conductor
(ConductorBoundaries_kernel, src/kernels/fields_bcs.hpp:522-800) with the
digital filter's wall stencils (digital_filter.hpp:99-379), and MATCH
(MatchBoundaries_kernel's SRPIC branch, fields_bcs.hpp:42-520).

The oracle is pinned by the conductor's defining properties: tangential E
and normal B vanish on the wall, the ghosts mirror the active cells, the
wall stencils' weights act on a uniform current as the reference writes
them, and a vacuum cavity mode keeps its field energy. The GPU matches the oracle bit for bit for the
conductor and the filter (copies, sign flips and the same sums in the same
order) and to the last bits of tanh for MATCH; whole engine steps with
conductor walls and reflecting particles track the oracle like the periodic
steps do.
"""
import pytest
import torch

from entity_gb300.inputs import GridSpec, empty_field, make_species
from entity_gb300.sim import step_params
from oracle.oracle import Oracle
from tests.helpers import random_currents, random_fields

PER, NONE, COND, MATCH = 0, 1, 2, 3
REALS = [torch.float32, torch.float64]


def _grid(dim, real, per, order=1, n=None):
    n = n or ((24, 20, 1) if dim == 2 else (12, 10, 8))
    prtl = tuple((0, 0) if per[d] else (2, 2) for d in range(3))
    return GridSpec(dim=dim, n=n, order=order, real=real, periodic=per, prtl_bc=prtl)


def _kinds(g, cond_sides):
    """kinds per side: PER on periodic axes, COND on the listed (axis, side)
    pairs, NONE elsewhere."""
    return tuple(tuple(PER if g.periodic[d] else (COND if (d, h) in cond_sides else NONE)
                       for h in range(2)) for d in range(3))


# ---------------------------------------------------------------------------
# the oracle against the conductor's properties
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dim", [2, 3])
def test_conductor_wall_and_mirror(dim):
    g = _grid(dim, torch.float64, (0, 1, 1))
    o = Oracle(g)
    o.set_field_bcs(_kinds(g, {(0, 0), (0, 1)}))
    EB = random_fields(g, 3)
    o.field_boundaries(EB, 1, 1)
    ng, n = g.ng, g.n[0]
    F = EB[:, 0] if dim == 2 else EB
    sl = (lambda c, i: F[c, :, i]) if dim == 2 else (lambda c, i: F[c, :, :, i])
    for edge, sgn in ((ng, -1), (n + ng, 1)):
        for c in (1, 2, 3):      # E2, E3 and B1 vanish on the wall
            assert torch.all(sl(c, edge) == 0)
    for k in range(1, ng + 1):
        # lower wall: normal E even across the face, tangential E odd, B the other way
        assert torch.equal(sl(0, ng - k), sl(0, ng + k - 1))
        assert torch.equal(sl(1, ng - k), -sl(1, ng + k))
        assert torch.equal(sl(3, ng - k), -sl(3, ng + k))
        assert torch.equal(sl(4, ng - k), sl(4, ng + k - 1))
    for k in range(1, ng):
        assert torch.equal(sl(1, n + ng + k), -sl(1, n + ng - k))
        assert torch.equal(sl(4, n + ng + k - 1), sl(4, n + ng - k))


@pytest.mark.parametrize("dim", [2, 3])
def test_wall_filter_weights(dim):
    """The wall stencils on a uniform current, conductors at both x1 walls:
    the wall-normal component keeps weights summing to one everywhere; the
    tangential ones, one cell inside a wall, keep 1/2 + 1/4 (the reference
    drops the image term across the wall); the wall cells' tangential
    components are left as they were."""
    g = _grid(dim, torch.float64, (0, 1, 1))
    o = Oracle(g)
    o.set_field_bcs(_kinds(g, {(0, 0), (0, 1)}))
    J, buff = empty_field(g, 3), empty_field(g, 3)
    J.fill_(1.0)
    o.filter_pass(J, buff)
    ng, n = g.ng, g.n[0]
    act = J[:, 0, ng:-ng, ng:-ng] if dim == 2 else J[:, ng:-ng, ng:-ng, ng:-ng]
    assert torch.all(act[0] == 1.0)
    for c in (1, 2):
        want = torch.ones(n, dtype=torch.float64)
        want[1] = want[n - 2] = 0.75
        assert torch.all(act[c] == want), c


def test_conductor_cavity_keeps_its_energy():
    """The lowest TM mode of a 2D box with conductor walls on all four
    sides (E3 = sin(pi x / Lx) sin(pi y / Ly), B = 0): over 400 steps (about
    five periods) the field energy only oscillates, with the leapfrog's
    half-step stagger, and E tangential to the walls stays zero. A wrong
    mirror sign makes the wall cells grow instead."""
    import math
    g = _grid(2, torch.float64, (0, 0, 1), n=(32, 24, 1))
    o = Oracle(g)
    o.set_field_bcs(_kinds(g, {(0, 0), (0, 1), (1, 0), (1, 1)}))
    prm = step_params(g, cfl=0.45, ppc0=4.0, skindepth0=3.0, larmor0=2.0, deposit=False)
    ng, (n1, n2) = g.ng, g.n[:2]
    EB = empty_field(g, 6)
    x = torch.arange(n1 + 2 * ng, dtype=torch.float64) - ng
    y = torch.arange(n2 + 2 * ng, dtype=torch.float64) - ng
    EB[2, 0] = torch.sin(math.pi * y / n2)[:, None] * torch.sin(math.pi * x / n1)[None, :]
    o.field_boundaries(EB, 1, 1)
    J, buff = empty_field(g, 3), empty_field(g, 3)
    energy = lambda: float((EB[:, 0, ng:-ng, ng:-ng].double() ** 2).sum())
    e0 = energy()
    es = []
    for step in range(400):
        o.step([], EB, J, buff, prm, step)
        es.append(energy())
    assert max(abs(e / e0 - 1.0) for e in es) < 0.1
    assert abs(max(es[200:]) / max(es[:200]) - 1.0) < 0.01
    assert torch.all(EB[1, 0, :, ng] == 0) and torch.all(EB[0, 0, ng, :] == 0)


# ---------------------------------------------------------------------------
# GPU against the oracle
# ---------------------------------------------------------------------------
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import abi, build
    build.build()
    abi.load()


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("sides", ["lo", "hi", "both", "two_axes"])
@pytest.mark.parametrize("tags", [(1, 1), (1, 0), (0, 1)])
def test_conductor_matches_oracle(real, dim, sides, tags):
    _gpu()
    from entity_gb300.sim import Context
    per = (0, 0, 1) if sides == "two_axes" else (0, 1, 1)
    if dim == 3 and sides == "two_axes":
        per = (0, 1, 0)
    g = _grid(dim, real, per)
    cs = {"lo": {(0, 0)}, "hi": {(0, 1)}, "both": {(0, 0), (0, 1)},
          "two_axes": {(0, 0), (0, 1), (1 if dim == 2 else 2, 0), (1 if dim == 2 else 2, 1)}}[sides]
    kinds = _kinds(g, cs)
    o, ctx = Oracle(g), Context(g)
    o.set_field_bcs(kinds)
    ctx.set_field_bcs(kinds)
    EB = random_fields(g, 7)
    EBg = EB.cuda()
    o.field_boundaries(EB, *tags)
    ctx.field_boundaries(EBg, *tags)
    torch.cuda.synchronize()
    assert torch.equal(EB, EBg.cpu())


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
def test_match_matches_oracle(real, dim):
    _gpu()
    from entity_gb300.sim import Context
    per = (0, 0, 1) if dim == 2 else (0, 1, 0)
    g = _grid(dim, real, per)
    last = 1 if dim == 2 else 2
    kinds = tuple(tuple(PER if g.periodic[d] else (MATCH if (d, h) in {(0, 1), (last, 0)} else NONE)
                        for h in range(2)) for d in range(3))
    ds = ((0.0, 4.5), (3.0, 0.0), (2.5, 0.0)) if dim == 2 else ((0.0, 4.5), (0.0, 0.0), (2.5, 0.0))
    x_min, dx = (-3.0, 1.0, 0.5), 0.75
    T = random_fields(g, 11)
    EB = random_fields(g, 12)
    o, ctx = Oracle(g), Context(g)
    o.set_field_bcs(kinds, x_min, dx, ds, T)
    Tg = T.cuda()
    ctx.set_field_bcs(kinds, x_min, dx, ds, Tg)
    EBg = EB.cuda()
    o.field_boundaries(EB, 1, 1)
    ctx.field_boundaries(EBg, 1, 1)
    torch.cuda.synchronize()
    tol = 3e-6 if real == torch.float32 else 1e-13
    assert float((EB.double() - EBg.cpu().double()).abs().max()) <= tol
    # only the layers change
    assert not torch.equal(EB, random_fields(g, 12))


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("npasses", [1, 3])
def test_filter_with_conductor_walls_bitexact(real, dim, npasses):
    _gpu()
    from entity_gb300.sim import Context
    per = (0, 0, 1) if dim == 2 else (0, 1, 0)
    g = _grid(dim, real, per)
    cs = {(0, 0), (0, 1), (1, 0), (1, 1)} if dim == 2 else {(0, 0), (0, 1), (2, 1)}
    kinds = _kinds(g, cs)
    o, ctx = Oracle(g), Context(g)
    o.set_field_bcs(kinds)
    ctx.set_field_bcs(kinds)
    J = random_currents(g, 21)
    Jg, Bg = J.cuda(), empty_field(g, 3, "cuda")
    B = empty_field(g, 3)
    for _ in range(npasses):
        o.filter_pass(J, B)
        o.fill_ghosts(J, False, 0, 3)
    ctx.filter_currents(Jg, Bg, npasses)
    torch.cuda.synchronize()
    assert torch.equal(J, Jg.cpu())


@pytest.mark.gpu
@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim,order,nfilter", [(2, 1, 2), (3, 2, 2)])
def test_engine_steps_with_conductor_walls(dim, order, nfilter, real):
    """pic_srpic_step between conductor walls at x1 (particles reflect
    there), periodic elsewhere, against the oracle's step."""
    _gpu()
    from entity_gb300.sim import Context
    g = _grid(dim, real, (0, 1, 1), order=order)
    kinds = _kinds(g, {(0, 0), (0, 1)})
    prm = step_params(g, cfl=0.45, ppc0=8.0, skindepth0=3.0, larmor0=2.0, nfilter=nfilter,
                      sort_interval=3, write_prev=True)
    EB = random_fields(g, 31, amp=0.05)
    spe = make_species(g, 4, 0.2, 0.3, 32, charge=-1.0)
    spp = make_species(g, 4, 0.2, -0.3, 33, charge=1.0, index=2)
    o, ctx = Oracle(g), Context(g)
    o.set_field_bcs(kinds)
    ctx.set_field_bcs(kinds)
    o.field_boundaries(EB, 1, 1)
    EBo, Jo, Bo = EB.clone(), empty_field(g, 3), empty_field(g, 3)
    EBg, Jg, Bg = EB.cuda(), empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    so = [spe.clone(), spp.clone()]
    sg = [spe.clone().to("cuda"), spp.clone().to("cuda")]
    for step in range(6):
        o.step(so, EBo, Jo, Bo, prm, step)
        ctx.step(sg, EBg, Jg, Bg, prm, step)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    tol = 2e-4 if real == torch.float32 else 1e-10
    for a, b in zip(so, sg):
        assert a.npart == b.npart
        for d in range(3):
            du = float((a.u[d].double() - b.u[d].cpu().double()).abs().max())
            assert du <= tol * max(1.0, float(a.u[d].abs().max()))
    scale = float(EBo.abs().max())
    assert float((EBo.double() - EBg.cpu().double()).abs().max()) <= tol * scale
    ng = g.ng
    wall = EBg[1, 0, :, ng] if dim == 2 else EBg[1, :, :, ng]
    assert torch.all(wall == 0)
