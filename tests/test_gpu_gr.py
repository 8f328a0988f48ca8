"""Parity of the GR CUDA path with the GR oracle, through the C ABI.

The GR metric is evaluated with transcendental functions whose last bits
differ between the GPU and the host C library, so parity here is by
tolerance (not bit-exact): FP32 within a few 1e-5 relative of the field or
state scale, FP64 within 1e-10. Positions are compared as continuous code
coordinates X = i + dx (a cell boundary crossed by one side and not the
other by 1 ulp counts as a match).
"""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu

REALS = [torch.float32, torch.float64]
TOL = {torch.float32: 3e-5, torch.float64: 1e-10}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import abi, build
    build.build()
    abi.load()


def _setup(real, order=2, n=(48, 32), a=0.95, r_max=20.0, h=0.0):
    from entity_gb300.gr import GRContext, GRSpec, gr_grid
    from oracle.oracle import GROracle
    g = gr_grid(n[0], n[1], order=order, real=real)
    spec = GRSpec(a=a, r_max=r_max, h=h)
    ctx = GRContext(g, spec)
    m = spec.metric()
    o = GROracle(g, a=a, r_min=m.x1min, r_max=m.x1max, th_min=m.x2min, th_max=m.x2max, h=h)
    return g, spec, ctx, o


def _rand_fields(g, seed, amp=0.05):
    from tests.helpers import random_fields
    return random_fields(g, seed, amp=amp)


def _particles(g, n, seed, umax=0.3, charge=-1.0, pusher=1, margin=2):
    from entity_gb300.inputs import SpeciesArrays
    gen = torch.Generator().manual_seed(seed)
    i1 = torch.randint(margin, g.n[0] - margin, (n,), generator=gen, dtype=torch.int32)
    i2 = torch.randint(1, g.n[1] - 1, (n,), generator=gen, dtype=torch.int32)
    d1 = torch.rand(n, generator=gen, dtype=torch.float32)
    d2 = torch.rand(n, generator=gen, dtype=torch.float32)
    u = [((torch.rand(n, generator=gen, dtype=torch.float64) * 2 - 1) * umax).to(g.real)
         for _ in range(3)]
    z32 = torch.zeros(n, dtype=torch.int32)
    zf = torch.zeros(n, dtype=torch.float32)
    return SpeciesArrays([i1, i2, z32.clone()], [d1, d2, zf.clone()],
                         [i1.clone(), i2.clone(), z32.clone()], [d1.clone(), d2.clone(), zf.clone()],
                         u, torch.ones(n, dtype=g.real), torch.ones(n, dtype=torch.int16), 1.0,
                         charge, pusher, n, 1)


def _X(sp, d):
    return sp.i[d].double().cpu() + sp.dx[d].double().cpu()


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("h", [0.0, 0.25])
def test_gr_metric_matches_oracle(real, h):
    g, spec, ctx, o = _setup(real, h=h)
    gen = torch.Generator().manual_seed(3)
    x = torch.stack([torch.rand(500, generator=gen, dtype=torch.float64) * g.n[0],
                     1.0 + torch.rand(500, generator=gen, dtype=torch.float64) * (g.n[1] - 2)], 1)
    mg = ctx.metric_eval(x).cpu()
    mo = o.metric(x)
    from oracle.oracle import GR_NAMES
    for j, k in enumerate(GR_NAMES):
        a, b = mg[:, j], mo[k]
        scale = float(b.abs().max()) + 1e-300
        err = float((a - b).abs().max()) / scale
        assert err <= (2e-5 if real == torch.float32 else 1e-12), (k, err)


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("pusher", [1, 3])
@pytest.mark.parametrize("h", [0.0, 0.25])
def test_gr_push_matches_oracle(real, order, pusher, h):
    g, spec, ctx, o = _setup(real, order=order, h=h)
    em, em0 = _rand_fields(g, 1), _rand_fields(g, 2)
    sp = _particles(g, 4000, 5, pusher=pusher)
    dt, omegaB0 = 0.05, 2.0
    # a band away from both ends, so particles lie below, in and above it
    island = (g.n[0] // 6, g.n[0] // 3)
    spg = sp.clone().to("cuda")
    o.gr_push(sp, em, em0, dt, omegaB0, 10, island=island)
    ctx.gr_push(spg, em.cuda(), em0.cuda(), dt, omegaB0, 10, island=island)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    assert torch.equal(sp.tag, spg.tag.cpu())
    alive = sp.tag == 1
    tol = TOL[real]
    for d in range(2):
        diff = (_X(sp, d) - _X(spg, d))[alive].abs().max()
        assert float(diff) <= tol * 50, (d, float(diff))
        assert torch.equal(sp.i_prev[d], spg.i_prev[d].cpu())
    for c in range(3):
        a, b = sp.u[c].double(), spg.u[c].cpu().double()
        scale = float(a.abs().max()) + 1e-30
        assert float((a - b)[alive].abs().max()) <= tol * 10 * scale, c


@pytest.mark.parametrize("real", REALS)
def test_gr_particle_push_all_species(real):
    """pic_gr_particle_push over three species (electrons, positrons,
    photons; the islands run on their own streams) against the oracle's
    push of each species."""
    g, spec, ctx, o = _setup(real, order=2)
    em, em0 = _rand_fields(g, 1), _rand_fields(g, 2)
    sps = [_particles(g, 3000, 21, charge=-1.0), _particles(g, 2500, 22, charge=1.0),
           _particles(g, 2000, 23, pusher=3)]
    island = (g.n[0] // 6, g.n[0] // 3)
    gpu = [s.clone().to("cuda") for s in sps]
    for s in sps:
        o.gr_push(s, em, em0, 0.05, 2.0, 10, island=island)
    ctx.gr_particle_push(gpu, em.cuda(), em0.cuda(), 0.05, 2.0, 10, island=island)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    tol = TOL[real]
    for s, sg in zip(sps, gpu):
        assert torch.equal(s.tag, sg.tag.cpu())
        alive = s.tag == 1
        for d in range(2):
            assert float((_X(s, d) - _X(sg, d))[alive].abs().max()) <= tol * 50
        for c in range(3):
            a, b = s.u[c].double(), sg.u[c].cpu().double()
            scale = float(a.abs().max()) + 1e-30
            assert float((a - b)[alive].abs().max()) <= tol * 10 * scale, c


@pytest.mark.parametrize("band", [(0, 48), (8, 9), (30, 10)])
def test_gr_push_island_bands(band):
    """FP32 with the island band covering every cell (many more 32-particle
    chunks than the island kernel has warps, so warps take several each),
    one cell, and an empty band (hi < lo: everything in FP32)."""
    g, spec, ctx, o = _setup(torch.float32, order=2)
    em, em0 = _rand_fields(g, 1), _rand_fields(g, 2)
    sp = _particles(g, 120000 if band == (0, 48) else 20000, 11)
    spg = sp.clone().to("cuda")
    o.gr_push(sp, em, em0, 0.05, 2.0, 10, island=band)
    ctx.gr_push(spg, em.cuda(), em0.cuda(), 0.05, 2.0, 10, island=band)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    assert torch.equal(sp.tag, spg.tag.cpu())
    alive = sp.tag == 1
    for d in range(2):
        assert float((_X(sp, d) - _X(spg, d))[alive].abs().max()) <= TOL[torch.float32] * 50
    for c in range(3):
        a, b = sp.u[c].double(), spg.u[c].cpu().double()
        scale = float(a.abs().max()) + 1e-30
        assert float((a - b)[alive].abs().max()) <= TOL[torch.float32] * 10 * scale, c


@pytest.mark.parametrize("real", REALS)
def test_gr_deposit_matches_oracle(real):
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2)
    em, em0 = _rand_fields(g, 1, amp=0.02), _rand_fields(g, 2, amp=0.02)
    sp = _particles(g, 4000, 7)
    dt = 0.05
    island = (g.n[0] // 6, g.n[0] // 3)
    o.gr_push(sp, em, em0, dt, 2.0, 10, island=island)   # sets the prev arrays
    J = empty_field(g, 3)
    o.gr_deposit([sp], J, dt, island=island)
    Jg = empty_field(g, 3, "cuda")
    ctx.gr_deposit([sp.clone().to("cuda")], Jg, dt, island=island)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    scale = float(J.abs().max())
    assert scale > 0
    assert float((J.double() - Jg.cpu().double()).abs().max()) <= TOL[real] * scale


@pytest.mark.parametrize("real", REALS)
def test_gr_field_kernels_match_oracle(real):
    from entity_gb300.inputs import empty_field
    from tests.helpers import random_currents
    g, spec, ctx, o = _setup(real, order=2)
    A, B, C = _rand_fields(g, 11), _rand_fields(g, 12), _rand_fields(g, 13)
    J = random_currents(g, 14)
    tol = TOL[real] * 10

    def check(name, cpu, gpu):
        scale = float(cpu.abs().max()) + 1e-30
        err = float((cpu.double() - gpu.cpu().double()).abs().max()) / scale
        assert err <= tol, (name, err)

    def run(op_cpu, op_gpu, outs):
        cpu = [t.clone() for t in (A, B, C, J)]
        gpu = [t.clone().cuda() for t in (A, B, C, J)]
        op_cpu(*cpu)
        op_gpu(*gpu)
        torch.cuda.synchronize()
        return cpu, gpu

    cases = {
        "faraday_aux": (lambda a, b, c, j: o.gr_faraday(b, b, c, 0.3),
                        lambda a, b, c, j: ctx.gr_faraday(b, b, c, 0.3)),
        "faraday_main": (lambda a, b, c, j: o.gr_faraday(a, b, c, 0.3),
                         lambda a, b, c, j: ctx.gr_faraday(a, b, c, 0.3)),
        "ampere_alias": (lambda a, b, c, j: o.gr_ampere(b, b, c, 0.3),
                         lambda a, b, c, j: ctx.gr_ampere(b, b, c, 0.3)),
        "ampere_main": (lambda a, b, c, j: o.gr_ampere(a, b, c, 0.3),
                        lambda a, b, c, j: ctx.gr_ampere(a, b, c, 0.3)),
        "currents": (lambda a, b, c, j: o.gr_currents_ampere(b, j, -0.2),
                     lambda a, b, c, j: ctx.gr_currents_ampere(b, j, -0.2)),
        "aux_e": (lambda a, b, c, j: o.gr_aux_e(a, b, c),
                  lambda a, b, c, j: ctx.gr_aux(0, a, b, c)),
        "aux_h": (lambda a, b, c, j: o.gr_aux_h(a, b, c),
                  lambda a, b, c, j: ctx.gr_aux(1, a, b, c)),
        "average_db": (lambda a, b, c, j: o.gr_average_db(a, b),
                       lambda a, b, c, j: ctx.gr_average(0, a, b)),
        "bcs": (lambda a, b, c, j: o.gr_field_bcs(b, 1, 1),
                lambda a, b, c, j: ctx.gr_field_bcs(b, 1, 1)),
    }
    for name, (fc, fg) in cases.items():
        cpu, gpu = run(fc, fg, None)
        for k in range(3):
            check(f"{name}[{k}]", cpu[k], gpu[k])


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("h", [0.0, 0.25])
def test_grpic_step_matches_oracle(real, h):
    """Five steps of GRPICEngine::step_forward (with step 0's initialisation)
    of the vertical-field Wald problem with injected pairs, on a grid with
    theta = eta and on one with stretched polar angles (h = 0.25)."""
    from entity_gb300.gr import gr_step_params, horizon_island, inject_pairs
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2, n=(64, 48), r_max=15.0, h=h)
    em = empty_field(g, 6, "cuda")
    ctx.gr_init_vertical(em)
    fields = [em, torch.zeros_like(em), torch.zeros_like(em), empty_field(g, 3, "cuda"),
              empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")]
    species = inject_pairs(g, spec, 2, 5.0, 3)
    prm = gr_step_params(ctx, cfl=0.5, ppc0=2.0, skindepth0=0.5, larmor0=0.25)
    island = horizon_island(g, spec)
    cpu_fields = [f.cpu().clone() for f in fields]
    cpu_species = [s.clone().to("cpu") for s in species]
    for step in range(5):
        ctx.grpic_step(species, fields, prm, niter=10, island=island, step=step)
        o.grpic_step(cpu_species, cpu_fields, prm, niter=10, island=island, step=step)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    # FP32: the current sums' order differs (atomics) and the step feeds J
    # back into D; five steps keep the difference below 2e-3 of each scale
    tol = 2e-3 if real == torch.float32 else 1e-9
    for k, name in ((0, "em"), (1, "em0"), (3, "cur"), (4, "cur0")):
        a, b = cpu_fields[k].double(), fields[k].cpu().double()
        for c in range(a.shape[0]):
            scale = float(a[c].abs().max())
            if scale == 0:
                continue
            err = float((a[c] - b[c]).abs().max()) / scale
            assert err <= tol, (name, c, err)
    for so, sg in zip(cpu_species, species):
        assert so.npart == sg.npart
        assert torch.equal(so.tag, sg.tag.cpu())
        alive = so.tag == 1
        for d in range(2):
            assert float((_X(so, d) - _X(sg, d))[alive].abs().max()) <= tol * 10
        for c in range(3):
            a, b = so.u[c].double(), sg.u[c].cpu().double()
            scale = float(a.abs().max()) + 1e-30
            assert float((a - b)[alive].abs().max()) <= tol * 10 * scale


@pytest.mark.parametrize("real", REALS)
def test_gr_current_filter_matches_oracle(real):
    # grpic::CurrentsFilter's axisymmetric stencil with the axis rows: pure
    # arithmetic in the reference's order, so bit-exact over three passes
    from entity_gb300.inputs import empty_field
    from tests.helpers import random_currents
    g, spec, ctx, o = _setup(real, order=2)
    J = random_currents(g, 23)
    Jg = J.cuda()
    for _ in range(3):
        o.gr_filter_pass(J, empty_field(g, 3))
    ctx.gr_filter_currents(Jg, empty_field(g, 3, "cuda"), 3)
    torch.cuda.synchronize()
    assert torch.equal(J, Jg.cpu())


@pytest.mark.parametrize("real", REALS)
def test_grpic_step_with_filter_matches_oracle(real):
    """Five GR steps with two current-filter passes per step (nfilter = 2,
    the horizon boundary's source row shifted accordingly)."""
    from entity_gb300.gr import gr_step_params, horizon_island, inject_pairs
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2, n=(64, 48), r_max=15.0)
    em = empty_field(g, 6, "cuda")
    ctx.gr_init_vertical(em)
    fields = [em, torch.zeros_like(em), torch.zeros_like(em), empty_field(g, 3, "cuda"),
              empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")]
    species = inject_pairs(g, spec, 2, 5.0, 3)
    prm = gr_step_params(ctx, cfl=0.5, ppc0=2.0, skindepth0=0.5, larmor0=0.25)
    prm.nfilter = 2
    island = horizon_island(g, spec)
    cpu_fields = [f.cpu().clone() for f in fields]
    cpu_species = [s.clone().to("cpu") for s in species]
    for step in range(5):
        ctx.grpic_step(species, fields, prm, niter=10, island=island, step=step)
        o.grpic_step(cpu_species, cpu_fields, prm, niter=10, island=island, step=step)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    tol = 2e-3 if real == torch.float32 else 1e-9
    for k, name in ((0, "em"), (1, "em0"), (3, "cur"), (4, "cur0")):
        a, b = cpu_fields[k].double(), fields[k].cpu().double()
        for c in range(a.shape[0]):
            scale = float(a[c].abs().max())
            if scale == 0:
                continue
            err = float((a[c] - b[c]).abs().max()) / scale
            assert err <= tol, (name, c, err)
    for so, sg in zip(cpu_species, species):
        assert so.npart == sg.npart
        assert torch.equal(so.tag, sg.tag.cpu())


@pytest.mark.parametrize("real", REALS)
def test_gr_magnetic_flux_stays_divergence_free(real):
    """The vertical seed field comes from a vector potential, so its discrete
    divergence d_r(sqrt h B^r) + d_theta(sqrt h B^theta) vanishes; the GR
    Faraday update is a discrete curl and keeps it so over the steps."""
    from entity_gb300.gr import gr_step_params, horizon_island, inject_pairs
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2, n=(64, 48), r_max=15.0)
    em = empty_field(g, 6, "cuda")
    ctx.gr_init_vertical(em)
    fields = [em, torch.zeros_like(em), torch.zeros_like(em), empty_field(g, 3, "cuda"),
              empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")]
    species = inject_pairs(g, spec, 2, 5.0, 3)
    prm = gr_step_params(ctx, cfl=0.5, ppc0=2.0, skindepth0=0.5, larmor0=0.25)
    island = horizon_island(g, spec)
    ng = g.ng
    n1, n2 = g.n[0], g.n[1]
    i = torch.arange(n1 + 2 * ng, dtype=torch.float64) - ng
    j = torch.arange(n2 + 2 * ng, dtype=torch.float64) - ng
    Jj, Ii = torch.meshgrid(j, i, indexing="ij")

    def sdh(x1, x2):
        pts = torch.stack([x1.reshape(-1), x2.reshape(-1)], 1)
        return o.metric(pts)["sqrt_det_h"].reshape(x1.shape)

    s_r = sdh(Ii, Jj + 0.5)    # at (i, j + 1/2), B^r
    s_t = sdh(Ii + 0.5, Jj)    # at (i + 1/2, j), B^theta

    def div(B):
        # cell (i + 1/2, j + 1/2): faces B^r at i, i + 1 and B^theta at j, j + 1
        Br = B[3, 0].double().cpu() * s_r
        Bt = B[4, 0].double().cpu() * s_t
        d = (Br[:-1, 1:] - Br[:-1, :-1]) + (Bt[1:, :-1] - Bt[:-1, :-1])
        # interior in r (the horizon boundary overwrites the first cells and
        # no MATCH boundary updates the last ghosts); all of theta
        region = d[ng:ng + n2, ng + 2:ng + n1 - 3]
        return region, float(Br.abs().max() + Bt.abs().max())

    d0, s0 = div(fields[0])
    eps = 1e-5 if real == torch.float32 else 1e-12
    assert float(d0.abs().max()) <= eps * s0
    for step in range(10):
        ctx.grpic_step(species, fields, prm, niter=10, island=island, step=step)
    d1, s1 = div(fields[0])
    assert float(d1.abs().max()) <= 20 * eps * s1


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("tags", [(1, 1), (1, 0), (0, 1)])
def test_gr_match_matches_oracle(real, tags):
    """MatchBoundaries_kernel (GRPIC, +r) toward a target field, both axes on."""
    g, spec, ctx, o = _setup(real, order=2, n=(48, 32), r_max=20.0)
    F, T = _rand_fields(g, 3), _rand_fields(g, 4)
    ds = 4.0
    Fg = F.cuda()
    o.gr_match(F, T, ds, *tags)
    ctx.gr_match_fields(Fg, T.cuda(), ds, *tags)
    torch.cuda.synchronize()
    Fc = Fg.cpu()
    scale = float(F.abs().max())
    assert float((F.double() - Fc.double()).abs().max()) <= TOL[real] * scale
    # below the layer nothing changes, bit for bit
    ng = g.ng
    assert torch.equal(F[:, 0, :, :20 + ng], Fc[:, 0, :, :20 + ng])


@pytest.mark.parametrize("real", REALS)
def test_gr_absorb_currents_matches_oracle(real):
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2, n=(48, 32), r_max=20.0)
    J = _rand_fields(g, 6)[:3].clone()
    Jg = J.cuda()
    o.gr_absorb_currents(J, 4.0)
    ctx.gr_absorb_currents(Jg, 4.0)
    torch.cuda.synchronize()
    scale = float(J.abs().max())
    assert float((J.double() - Jg.cpu().double()).abs().max()) <= TOL[real] * scale


@pytest.mark.parametrize("real", REALS)
def test_grpic_step_with_match_matches_oracle(real):
    """Five GR steps with the MATCH boundary at r max relaxing toward the
    initial vertical field and the currents absorbed there."""
    from entity_gb300.gr import gr_step_params, horizon_island, inject_pairs
    from entity_gb300.inputs import empty_field
    g, spec, ctx, o = _setup(real, order=2, n=(64, 48), r_max=15.0)
    em = empty_field(g, 6, "cuda")
    ctx.gr_init_vertical(em)
    target = em.clone()
    fields = [em, torch.zeros_like(em), torch.zeros_like(em), empty_field(g, 3, "cuda"),
              empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")]
    # pairs out to r = 14 so that the layer holds current
    species = inject_pairs(g, spec, 2, 14.0, 3)
    prm = gr_step_params(ctx, cfl=0.5, ppc0=2.0, skindepth0=0.5, larmor0=0.25)
    island = horizon_island(g, spec)
    ds = 1.5
    cpu_fields = [f.cpu().clone() for f in fields]
    cpu_species = [s.clone().to("cpu") for s in species]
    tgt_cpu = target.cpu()
    for step in range(5):
        ctx.grpic_step(species, fields, prm, niter=10, island=island, step=step,
                       match=(ds, target))
        o.grpic_step(cpu_species, cpu_fields, prm, niter=10, island=island, step=step,
                     match=(ds, tgt_cpu))
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    tol = 2e-3 if real == torch.float32 else 1e-9
    for k, name in ((0, "em"), (1, "em0"), (3, "cur")):
        a, b = cpu_fields[k].double(), fields[k].cpu().double()
        scale = float(a.abs().max()) + 1e-30
        assert float((a - b).abs().max()) <= tol * scale, name


def test_gr_metric_rejects_h_outside_its_range():
    """The reference's closed-form theta -> eta is real for 0 <= h < 1."""
    from entity_gb300 import abi
    from entity_gb300.gr import GRContext, GRSpec, gr_grid
    g = gr_grid(16, 16)
    for h in (-0.2, 1.0):
        ctx = GRContext(g, GRSpec(h=h))
        x = torch.zeros(4, 2, dtype=torch.float64, device="cuda")
        with pytest.raises(abi.PicError):
            ctx.metric_eval(x)
