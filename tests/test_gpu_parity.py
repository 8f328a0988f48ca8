"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars:
  * particle push (cells, offsets, momenta, prev arrays, tags): bit-exact;
  * field kernels, ghost exchange, filter, current fold: bit-exact;
  * sort permutation and permuted arrays: bit-exact;
  * currents: the GPU adds contributions in a different order than the
    oracle, so J agrees to |dJ| <= 4e-6 * max|J| (float) / 1e-13 (double)
    with each particle's contribution computed bit-identically.
"""
import math

import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, make_species
from entity_gb300.sim import Context, step_params
from tests.helpers import random_currents, random_fields, species_from_lists

pytestmark = pytest.mark.gpu

REALS = [torch.float32, torch.float64]
J_TOL = {torch.float32: 4e-6, torch.float64: 1e-13}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _grid(dim, order, real, **kw):
    n = (32, 24, 1) if dim == 2 else (12, 10, 8)
    return GridSpec(dim=dim, n=n, order=order, real=real, **kw)


def _oracle(g):
    from oracle.oracle import Oracle
    return Oracle(g)


def _species_pair(g, seed, temp=0.2, beta=0.3, ppc=4, **kw):
    sp = make_species(g, ppc, temp, beta, seed, **kw)
    return sp, sp.clone().to("cuda")


def _assert_particles_equal(a, b, dim, prev=True):
    for d in range(dim):
        assert torch.equal(a.i[d], b.i[d].cpu()), f"i{d + 1}"
        assert torch.equal(a.dx[d], b.dx[d].cpu()), f"dx{d + 1}"
        if prev:
            assert torch.equal(a.i_prev[d], b.i_prev[d].cpu()), f"i{d + 1}_prev"
            assert torch.equal(a.dx_prev[d], b.dx_prev[d].cpu()), f"dx{d + 1}_prev"
    for d in range(3):
        assert torch.equal(a.u[d], b.u[d].cpu()), f"u{d + 1}"
    assert torch.equal(a.tag, b.tag.cpu())


def _assert_J_close(Jo, Jg, real):
    scale = max(float(Jo.abs().max()), 1e-30)
    diff = float((Jo.double() - Jg.cpu().double()).abs().max())
    assert diff <= J_TOL[real] * scale, (diff, scale)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("pusher", [abi.PIC_PUSHER_BORIS, abi.PIC_PUSHER_VAY])
def test_push_bitexact(dim, order, real, pusher):
    g = _grid(dim, order, real)
    EB = random_fields(g, 11 + dim * 10 + order)
    sp, spg = _species_pair(g, 100 + order, temp=0.5, beta=0.3, pusher=pusher)
    o = _oracle(g)
    dt, om, dx = 0.45, 0.7, g.dx
    assert o.push(sp, EB, dt, om, dx) == 0
    ctx = Context(g)
    ctx.push(spg, EB.cuda(), dt, om, dx)
    torch.cuda.synchronize()
    _assert_particles_equal(sp, spg, dim)
    assert ctx.device_errors()[0] == 0


@pytest.mark.parametrize("bc", [abi.PIC_BC_ABSORB, abi.PIC_BC_REFLECT])
@pytest.mark.parametrize("real", REALS)
def test_push_boundaries_bitexact(bc, real):
    g = GridSpec(dim=2, n=(16, 16, 1), order=1, real=real, periodic=(0, 1, 1),
                 prtl_bc=((bc, bc), (0, 0), (0, 0)))
    EB = random_fields(g, 5)
    sp, spg = _species_pair(g, 9, temp=1.0, beta=0.0, ppc=8)
    o = _oracle(g)
    o.push(sp, EB, 0.6, 0.5, g.dx)
    ctx = Context(g)
    ctx.push(spg, EB.cuda(), 0.6, 0.5, g.dx)
    torch.cuda.synchronize()
    _assert_particles_equal(sp, spg, 2)
    if bc == abi.PIC_BC_ABSORB:
        assert int((sp.tag == 0).sum()) > 0


@pytest.mark.parametrize("real", REALS)
def test_photon_push_bitexact(real):
    g = _grid(3, 2, real)
    EB = random_fields(g, 3)
    sp, spg = _species_pair(g, 4, temp=1.0, beta=0.0, pusher=abi.PIC_PUSHER_PHOTON,
                            mass=0.0, charge=0.0)
    o = _oracle(g)
    o.push(sp, EB, 0.4, 1.0, g.dx)
    ctx = Context(g)
    ctx.push(spg, EB.cuda(), 0.4, 1.0, g.dx)
    torch.cuda.synchronize()
    _assert_particles_equal(sp, spg, 3)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
def test_deposit_matches_oracle(dim, order, real):
    g = _grid(dim, order, real)
    EB = random_fields(g, 21)
    sp, _ = _species_pair(g, 200 + order, temp=0.5, beta=0.3)
    o = _oracle(g)
    o.push(sp, EB, 0.45, 0.7, g.dx)           # sets prev arrays
    spg = sp.clone().to("cuda")
    Jo = empty_field(g, 3)
    o.deposit([sp], Jo, 0.45, g.dx)
    ctx = Context(g)
    Jg = empty_field(g, 3, "cuda")
    Jg.fill_(123.0)                            # deposit zeroes J first
    ctx.deposit([spg], Jg, 0.45, g.dx)
    torch.cuda.synchronize()
    _assert_J_close(Jo, Jg, real)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
def test_fused_push_deposit(dim, order, real):
    g = _grid(dim, order, real)
    EB = random_fields(g, 31)
    e_sp, e_spg = _species_pair(g, 300, temp=0.3, beta=0.3, charge=-1.0)
    p_sp, p_spg = _species_pair(g, 301, temp=0.3, beta=-0.3, charge=1.0, index=2)
    o = _oracle(g)
    Jo = empty_field(g, 3)
    for s in (e_sp, p_sp):
        o.push(s, EB, 0.45, 0.7, g.dx)
    o.deposit([e_sp, p_sp], Jo, 0.45, g.dx)
    ctx = Context(g)
    Jg = empty_field(g, 3, "cuda")
    ctx.push_deposit([e_spg, p_spg], EB.cuda(), Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
    torch.cuda.synchronize()
    _assert_particles_equal(e_sp, e_spg, dim)
    _assert_particles_equal(p_sp, p_spg, dim)
    _assert_J_close(Jo, Jg, real)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
def test_deposit_known_answer_gpu(real, order):
    # the single-particle scenario of tests/kernels/deposit.cpp on the GPU
    g = GridSpec(dim=2, n=(50, 50, 1), order=order, real=real, extent=55.0)
    sp = species_from_lists(g, [(24, 20)], [(0.99, 0.80)], [(0.0, 0.0, 2.5)],
                            prev_cells=[(25, 21)], prev_offsets=[(0.65, 0.65)], charge=1.0,
                            pad_to=10)
    Jo = empty_field(g, 3)
    _oracle(g).deposit([sp], Jo, 1.0, g.dx)
    ctx = Context(g)
    Jg = empty_field(g, 3, "cuda")
    ctx.deposit([sp.clone().to("cuda")], Jg, 1.0, g.dx)
    torch.cuda.synchronize()
    # a single particle: every J cell receives one contribution -> exact
    assert torch.equal(Jo, Jg.cpu())


STENCIL = (0.01, 0.02, 0.015, 0.005, 0.012, 0.004, 0.006, 0.003, 0.007)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("stencil", [None, STENCIL])
def test_faraday_bitexact(dim, real, stencil):
    g = _grid(dim, 2, real)
    EB = random_fields(g, 41)
    o = _oracle(g)
    c1, c2 = 0.31, 0.22
    EBo = EB.clone()
    o.faraday(EBo, c1, c2, stencil)
    o.fill_ghosts(EBo, True, 3, 6)
    ctx = Context(g)
    EBg = EB.cuda()
    ctx.faraday(EBg, c1, c2, stencil)
    torch.cuda.synchronize()
    assert torch.equal(EBo, EBg.cpu())


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
def test_ampere_and_currents_bitexact(dim, real):
    g = _grid(dim, 1, real)
    EB = random_fields(g, 51)
    J = random_currents(g, 52)
    o = _oracle(g)
    ctx = Context(g)
    # separate calls
    EBo, Jo = EB.clone(), J.clone()
    o.ampere(EBo, 0.3, 0.2)
    o.currents_ampere(EBo, Jo, -0.05, 16.0)
    o.fill_ghosts(EBo, True, 0, 3)
    o.fill_ghosts(Jo, False, 0, 3)
    EBg, Jg = EB.cuda(), J.cuda()
    ctx.ampere(EBg, 0.3, 0.2)
    ctx.currents_ampere(EBg, Jg, -0.05, 16.0)
    torch.cuda.synchronize()
    assert torch.equal(EBo, EBg.cpu())
    assert torch.equal(Jo, Jg.cpu())
    # fused Ampere + J -> E + exchange
    EBg2, Jg2 = EB.cuda(), J.cuda()
    ctx.ampere_currents(EBg2, Jg2, 0.3, 0.2, -0.05, 16.0)
    torch.cuda.synchronize()
    assert torch.equal(EBo, EBg2.cpu())
    assert torch.equal(Jo, Jg2.cpu())


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
def test_sync_currents_bitexact(dim, real):
    g = _grid(dim, 2, real)
    J = random_currents(g, 61)
    buff = empty_field(g, 3)
    o = _oracle(g)
    Jo = J.clone()
    o.sync_currents(Jo, buff)
    o.fill_ghosts(Jo, False, 0, 3)
    ctx = Context(g)
    Jg = J.cuda()
    ctx.sync_currents(Jg, empty_field(g, 3, "cuda"))
    torch.cuda.synchronize()
    assert torch.equal(Jo, Jg.cpu())


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("npasses", [1, 2, 4])
def test_filter_bitexact(dim, real, npasses):
    g = _grid(dim, 2, real)
    J = random_currents(g, 71)
    o = _oracle(g)
    Jo = J.clone()
    o.fill_ghosts(Jo, False, 0, 3)
    buff = empty_field(g, 3)
    for _ in range(npasses):
        o.filter_pass(Jo, buff)
        o.fill_ghosts(Jo, False, 0, 3)
    ctx = Context(g)
    Jg = J.cuda()
    ctx.fill_ghosts(Jg, False, 0, 3)
    ctx.filter_currents(Jg, empty_field(g, 3, "cuda"), npasses)
    torch.cuda.synchronize()
    assert torch.equal(Jo, Jg.cpu())


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("flags", [abi.PIC_SORT_SPATIAL,
                                   abi.PIC_SORT_SPATIAL | abi.PIC_SORT_REMOVE_DEAD,
                                   abi.PIC_SORT_REMOVE_DEAD])
def test_sort_bitexact(dim, flags):
    g = _grid(dim, 1, torch.float32)
    sp = make_species(g, 6, 0.2, 0.0, 81)
    gen = torch.Generator()
    gen.manual_seed(3)
    dead = torch.rand(sp.npart, generator=gen) < 0.15
    sp.tag[dead] = 0
    spg = sp.clone().to("cuda")
    o = _oracle(g)
    if flags & abi.PIC_SORT_REMOVE_DEAD:
        o.remove_dead(sp)
    if flags & abi.PIC_SORT_SPATIAL:
        o.sort(sp)
    ctx = Context(g)
    st = ctx.sort(spg, flags)
    assert st == abi.PIC_OK
    assert spg.npart == sp.npart
    _assert_particles_equal(sp, spg, dim)
    assert torch.equal(sp.w, spg.w.cpu())


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("flags", [abi.PIC_SORT_SPATIAL,
                                   abi.PIC_SORT_SPATIAL | abi.PIC_SORT_REMOVE_DEAD,
                                   abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED])
def test_sort_carries_phi_and_payloads(flags, real):
    # Particles::SortSpatially and RemoveDead move phi and every payload column
    # with the particle (particles_sort.cpp:169-177, 245-251): payloads in the
    # reference's device layout (column-major, pld(p, k) at p + k * maxnpart)
    # for the real ones and row-major for the integer ones; pld_i[:, 0] holds
    # each particle's original index
    g = _grid(3, 2, real)
    sp = make_species(g, 5, 0.2, 0.0, 44)
    n = sp.npart
    gen = torch.Generator()
    gen.manual_seed(9)
    sp.tag[torch.rand(n, generator=gen) < 0.1] = 0
    sp.phi = torch.rand(n, generator=gen, dtype=torch.float64).to(real)
    sp.pld_r = torch.rand(3, n, generator=gen, dtype=torch.float64).to(real).t()  # strides (1, n)
    sp.pld_i = torch.stack([torch.arange(n, dtype=torch.int32),
                            torch.randint(-(1 << 31), 1 << 31, (n,), generator=gen,
                                          dtype=torch.int32)], dim=1)
    assert sp.pld_r.stride() == (1, n) and sp.pld_i.stride() == (2, 1)
    ref = sp.clone()
    spg = sp.clone().to("cuda")
    assert spg.pld_r.stride() == (1, n)
    ctx = Context(g)
    assert ctx.sort(spg, flags) == abi.PIC_OK
    torch.cuda.synchronize()
    m = spg.npart
    orig = spg.pld_i[:m, 0].cpu().long()
    # a permutation of the original particles (the alive ones after removal)
    assert torch.equal(orig.sort().values,
                       (torch.nonzero(ref.tag == 1).flatten() if flags & abi.PIC_SORT_REMOVE_DEAD
                        else torch.arange(n)))
    for d in range(3):
        assert torch.equal(spg.i[d][:m].cpu(), ref.i[d][orig])
        assert torch.equal(spg.u[d][:m].cpu(), ref.u[d][orig])
    assert torch.equal(spg.phi[:m].cpu(), ref.phi[orig])
    assert torch.equal(spg.pld_r[:m].cpu(), ref.pld_r[orig])
    assert torch.equal(spg.pld_i[:m].cpu(), ref.pld_i[orig])
    # and the order is the oracle's
    o = _oracle(g)
    if flags & abi.PIC_SORT_REMOVE_DEAD:
        o.remove_dead(sp)
    if flags & abi.PIC_SORT_TILED:
        o.sort_tiled(sp, ctx.tile_shape())
    else:
        o.sort(sp)
    _assert_particles_equal(sp, spg, 3)


def test_sort_large_cells_and_many_dead():
    # bins over 32 entries take the block-per-bin path; the dead bin is large
    g = GridSpec(dim=2, n=(4, 4, 1), order=1, real=torch.float32)
    sp = make_species(g, 300, 0.1, 0.0, 5)
    sp.tag[::3] = 0
    spg = sp.clone().to("cuda")
    o = _oracle(g)
    o.remove_dead(sp)
    o.sort(sp)
    ctx = Context(g)
    assert ctx.sort(spg, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_REMOVE_DEAD) == abi.PIC_OK
    _assert_particles_equal(sp, spg, 2)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim,order,nfilter", [(2, 1, 0), (2, 0, 1), (3, 2, 4), (3, 3, 2)])
def test_engine_steps_track_oracle(dim, order, nfilter, real):
    # the whole SR step (srpic.hpp:65-188) through pic_srpic_step vs the
    # oracle's step sequence: after 1 step cells and tags are exact (J enters
    # E only after the push); over 6 steps everything agrees to round-off.
    g = _grid(dim, order, real)
    prm = step_params(g, cfl=0.45, ppc0=8.0, skindepth0=3.0, larmor0=2.0, nfilter=nfilter,
                      sort_interval=3, write_prev=True)
    EB = random_fields(g, 91, amp=0.05)
    spe = make_species(g, 4, 0.2, 0.3, 92, charge=-1.0)
    spp = make_species(g, 4, 0.2, -0.3, 93, charge=1.0, index=2)
    o = _oracle(g)
    ctx = Context(g)
    EBo, Jo, Bo = EB.clone(), empty_field(g, 3), empty_field(g, 3)
    EBg, Jg, Bg = EB.cuda(), empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    so = [spe.clone(), spp.clone()]
    sg = [spe.clone().to("cuda"), spp.clone().to("cuda")]
    for step in range(6):
        o.step(so, EBo, Jo, Bo, prm, step)
        ctx.step(sg, EBg, Jg, Bg, prm, step)
        torch.cuda.synchronize()
        if step == 0:
            for a, b in zip(so, sg):
                _assert_particles_equal(a, b, dim)
    tol = 2e-4 if real == torch.float32 else 1e-10
    for a, b in zip(so, sg):
        assert a.npart == b.npart
        for d in range(3):
            du = float((a.u[d].double() - b.u[d].cpu().double()).abs().max())
            assert du <= tol * max(1.0, float(a.u[d].abs().max()))
        same = sum(bool(torch.equal(a.i[d], b.i[d].cpu())) for d in range(dim))
        assert same == dim
    scale = float(EBo.abs().max())
    assert float((EBo.double() - EBg.cpu().double()).abs().max()) <= tol * scale


def test_device_errors_and_host_checks():
    g = _grid(3, 2, torch.float32)
    EB = random_fields(g, 1).cuda()
    sp = make_species(g, 2, 0.1, 0.0, 1).to("cuda")
    sp.tag[5] = 7      # neither alive nor dead: counted, not pushed
    ctx = Context(g)
    ctx.push(sp, EB, 0.3, 1.0, g.dx)
    assert ctx.device_errors(reset=True)[0] == 1
    assert ctx.device_errors()[0] == 0
    # npart beyond maxnpart is rejected on the host
    from entity_gb300.sim import make_species as mk
    ps = mk(sp, 3)
    ps.maxnpart = ps.npart - 1
    import ctypes as C
    st = abi.load().pic_push(ctx.h, C.byref(ps), C.c_void_p(EB.data_ptr()), 0.3, 1.0, 1.0, None)
    assert st == abi.PIC_ERR_ARG
    # a particle outside the grid is reported by the sort, the GPU stays usable
    sp.tag[5] = 1
    sp.i[0][3] = 10_000
    assert ctx.sort(sp, abi.PIC_SORT_SPATIAL) == abi.PIC_ERR_DEVICE
    torch.cuda.synchronize()
    assert ctx.device_errors(reset=True)[1] == 1
    x = torch.ones(10, device="cuda").sum()
    assert float(x) == 10.0


@pytest.mark.parametrize("real", REALS)
def test_field_energy_fp64(real):
    g = _grid(3, 2, real)
    EB = random_fields(g, 17)
    eo = _oracle(g).field_energy(EB, g.dx)
    eg = Context(g).field_energy(EB.cuda(), g.dx)
    assert eg[0] == pytest.approx(eo[0], rel=1e-12)
    assert eg[1] == pytest.approx(eo[1], rel=1e-12)
