"""pic_output_* on the GPU against the oracle (output_oracle.c): moments by
tolerance (atomic summation order), fields, divE and particle records bit
for bit; argument refusals; the npz writer end to end."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, make_species
from entity_gb300.sim import Context, make_species as mk
from oracle.oracle import Oracle
from tests.helpers import random_fields, species_from_lists

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _params(mid, order=1, smoothing=abi.PIC_SMOOTH_SPLINE, c1=0, c2=0, use_weights=1,
            inv_n0=0.5, dx=0.75):
    p = abi.PicMomentParams()
    p.id, p.c1, p.c2, p.order, p.smoothing = mid, c1, c2, order, smoothing
    p.use_weights, p.inv_n0, p.dx = use_weights, inv_n0, dx
    return p


def _dict(p):
    return dict(id=p.id, c1=p.c1, c2=p.c2, order=p.order, smoothing=p.smoothing,
                use_weights=p.use_weights, inv_n0=p.inv_n0, dx=p.dx)


def _species(g, seed, ppc=4, **kw):
    sp = make_species(g, ppc, 0.5, 0.3, seed, with_prev=False, **kw)
    gen = torch.Generator().manual_seed(seed)
    sp.w = (0.5 + torch.rand(sp.w.shape, generator=gen, dtype=torch.float64)).to(g.real)
    sp.tag[torch.rand(sp.tag.shape, generator=gen) < 0.05] = 0
    return sp


def _tol(real):
    return 2e-5 if real == torch.float32 else 1e-12


CASES = [(2, 1, torch.float32), (2, 2, torch.float64), (3, 2, torch.float32),
         (3, 3, torch.float64)]


def _cell_sorted(g, sp):
    """The species with its particles ordered by cell (x1 fastest), as a
    spatial sort leaves them: neighbouring lanes then share cells."""
    key = sp.i[0].long() + g.n[0] * (sp.i[1].long() + g.n[1] * sp.i[2].long())
    perm = torch.argsort(key, stable=True)
    pick = lambda xs: [None if x is None else x[perm] for x in xs]
    out = sp.clone()
    out.i, out.dx, out.u = pick(sp.i), pick(sp.dx), pick(sp.u)
    out.w, out.tag = sp.w[perm], sp.tag[perm]
    return out


@pytest.mark.parametrize("dim,order,real", CASES)
@pytest.mark.parametrize("cell_sorted", [False, True])
def test_moments_match_oracle(dim, order, real, cell_sorted):
    n = (24, 20, 1) if dim == 2 else (12, 10, 8)
    g = GridSpec(dim=dim, n=n, order=order, real=real)
    o, ctx = Oracle(g), Context(g)
    sps = [_species(g, 3, index=1), _species(g, 4, mass=2.0, charge=1.0, index=2)]
    if cell_sorted:
        sps = [_cell_sorted(g, s) for s in sps]
    sgs = [s.to("cuda") for s in sps]
    orders = [0, 1, 2, 3, 4] + ([5, 6] if g.ng >= 3 else [])
    cases = [(abi.PIC_MOM_N, k, abi.PIC_SMOOTH_SPLINE, 0, 0) for k in orders]
    cases += [(abi.PIC_MOM_RHO, 2, abi.PIC_SMOOTH_CONST, 0, 0),
              (abi.PIC_MOM_CHARGE, 1, abi.PIC_SMOOTH_SPLINE, 0, 0),
              (abi.PIC_MOM_NPPC, 3, abi.PIC_SMOOTH_SPLINE, 0, 0),
              (abi.PIC_MOM_T, 2, abi.PIC_SMOOTH_SPLINE, 0, 0),
              (abi.PIC_MOM_T, 1, abi.PIC_SMOOTH_SPLINE, 1, 3),
              (abi.PIC_MOM_V, 2, abi.PIC_SMOOTH_SPLINE, 2, 0)]
    for mid, k, sm, c1, c2 in cases:
        p = _params(mid, order=k, smoothing=sm, c1=c1, c2=c2)
        bo, bg = empty_field(g, 6), empty_field(g, 6, "cuda")
        o.output_moment(sps, _dict(p), bo, 4)
        o.sync_moments(bo, 4, 5)
        ctx.output_moment(sgs, p, bg, 4)
        ctx.sync_moments(bg, 4, 5)
        torch.cuda.synchronize()
        ng = g.ng
        sl = (4, slice(ng, ng + n[2]) if dim == 3 else 0, slice(ng, ng + n[1]),
              slice(ng, ng + n[0]))
        a, b = bo[sl].double(), bg.cpu()[sl].double()
        scale = float(a.abs().max())
        assert scale > 0
        assert float((a - b).abs().max()) <= _tol(real) * scale, (mid, k, sm)
    assert ctx.device_errors() == [0, 0, 0, 0]


def test_bulk_velocity_and_divergence_match_oracle():
    g = GridSpec(dim=3, n=(10, 9, 8), order=2, real=torch.float64)
    o, ctx = Oracle(g), Context(g)
    sp = _species(g, 9)
    sg = sp.to("cuda")
    bo, bg = empty_field(g, 6), empty_field(g, 6, "cuda")
    for k in range(3):
        p = _params(abi.PIC_MOM_V, order=2, c1=k + 1)
        o.output_moment([sp], _dict(p), bo, 3 + k)
        ctx.output_moment([sg], p, bg, 3 + k)
    p = _params(abi.PIC_MOM_RHO, order=2)
    o.sync_moments(bo, 3, 6)
    o.output_moment([sp], _dict(p), bo, 0)
    o.sync_moments(bo, 0, 1)
    o.normalize_by_rho(bo, 0, (3, 4, 5))
    ctx.sync_moments(bg, 3, 6)
    ctx.output_moment([sg], p, bg, 0)
    ctx.sync_moments(bg, 0, 1)
    ctx.normalize_by_rho(bg, 0, (3, 4, 5))
    ng = g.ng
    act = (slice(None), slice(ng, ng + 8), slice(ng, ng + 9), slice(ng, ng + 10))
    a, b = bo[act][3:6], bg.cpu()[act][3:6]
    assert float((a - b).abs().max()) <= 1e-12 * float(a.abs().max())
    EB = random_fields(g, 2)
    do, dg = empty_field(g, 6), empty_field(g, 6, "cuda")
    o.output_divergence(EB, do, 1)
    ctx.output_divergence(EB.cuda(), dg, 1)
    torch.cuda.synchronize()
    assert torch.equal(do, dg.cpu())


@pytest.mark.parametrize("dim,real", [(2, torch.float32), (3, torch.float64), (3, torch.float32)])
def test_field_output_is_bit_exact(dim, real):
    n = (17, 13, 1) if dim == 2 else (11, 9, 7)
    g = GridSpec(dim=dim, n=n, order=2, real=real)
    o, ctx = Oracle(g), Context(g)
    EB = random_fields(g, 6)
    J = random_fields(g, 7)[:3].contiguous()
    EBg, Jg = EB.cuda(), J.cuda()
    for src, srcg, is_em, c0, ncomp, flags, dwn in [
            (EB, EBg, 1, 0, 3, abi.PIC_OUT_INTERP_EDGES | abi.PIC_OUT_TO_HAT, (1, 1, 1)),
            (EB, EBg, 1, 3, 3, abi.PIC_OUT_INTERP_FACES | abi.PIC_OUT_TO_HAT, (2, 3, 2)),
            (J, Jg, 0, 0, 3, abi.PIC_OUT_INTERP_EDGES | abi.PIC_OUT_TO_HAT, (3, 1, 2)),
            (EB, EBg, 1, 0, 3, 0, (1, 2, 1)),
            (EB, EBg, 1, 4, 1, 0, (2, 2, 3))]:
        shape = tuple(math.ceil(n[d] / dwn[d]) for d in reversed(range(dim)))
        oo = torch.zeros((ncomp,) + shape, dtype=real)
        og = torch.zeros((ncomp,) + shape, dtype=real, device="cuda")
        o.output_field(src, is_em, c0, ncomp, flags, 0.75, dwn, oo)
        ctx.output_field(srcg, is_em, c0, ncomp, flags, 0.75, dwn, og)
        torch.cuda.synchronize()
        assert torch.equal(oo, og.cpu()), (c0, flags, dwn)


@pytest.mark.parametrize("dim,real,stride", [(2, torch.float32, 1), (3, torch.float64, 7)])
def test_particle_records_are_bit_exact(dim, real, stride):
    n = (16, 12, 1) if dim == 2 else (8, 8, 6)
    g = GridSpec(dim=dim, n=n, order=1, real=real)
    o, ctx = Oracle(g), Context(g)
    sp = _species(g, 2)
    sg = sp.to("cuda")
    m = sp.npart // stride
    xo = [torch.zeros(m, dtype=real) for _ in range(dim)]
    uo = [torch.zeros(m, dtype=real) for _ in range(3)]
    wo = torch.zeros(m, dtype=real)
    xg = [torch.zeros(m, dtype=real, device="cuda") for _ in range(dim)]
    ug = [torch.zeros(m, dtype=real, device="cuda") for _ in range(3)]
    wg = torch.zeros(m, dtype=real, device="cuda")
    xmin = (-3.0, 0.5, 1.25)
    assert o.output_particles(sp, stride, 0.3, xmin, xo, uo, wo) == m
    assert ctx.output_particles(sg, stride, 0.3, xmin, xg, ug, wg) == m
    torch.cuda.synchronize()
    for a, b in zip(xo + uo + [wo], xg + ug + [wg]):
        assert torch.equal(a, b.cpu())


def test_moments_known_answer_on_gpu():
    """tests/kernels/particle_moments.cpp on the device."""
    g = GridSpec(dim=2, n=(10, 10, 1), order=1, real=torch.float32)
    ctx = Context(g)
    sp = species_from_lists(g, [(5, 4), (2, 2)], [(0.15, 0.85), (0.22, 0.55)],
                            [(1.0, -2.0, 3.0), (-3.0, 2.0, -1.0)], mass=1.0, charge=1.0,
                            pusher=0).to("cuda")
    buf = empty_field(g, 6, "cuda")
    for k, c in enumerate((1, 2, 3)):
        ctx.output_moment([sp], _params(abi.PIC_MOM_T, order=1, c1=0, c2=c, use_weights=0,
                                        inv_n0=1.0, dx=1.0), buf, k)
    b = buf.cpu().double()
    eps = float(torch.finfo(torch.float32).eps) * 10
    for part in (b[:3, 0, :, :6], b[:3, 0, :, 6:]):
        v = [float(part[c].sum()) for c in range(3)]
        assert abs(1.0 + sum(x * x for x in v) - 15.0) <= 15.0 * eps


def test_argument_refusals():
    g = GridSpec(dim=2, n=(8, 8, 1), order=1, real=torch.float32)
    ctx = Context(g)
    L = abi.load()
    sp = _species(g, 1).to("cuda")
    arr = (abi.PicSpecies * 1)(mk(sp, 2))
    buf = empty_field(g, 6, "cuda")

    def mom(p, comp=0):
        return L.pic_output_moment(ctx.h, arr, 1, C.byref(p), C.c_void_p(buf.data_ptr()), comp,
                                   None)

    assert mom(_params(abi.PIC_MOM_N, order=4)) == abi.PIC_OK      # window 2 = ng
    assert mom(_params(abi.PIC_MOM_N, order=5)) == abi.PIC_ERR_ARG  # window 3 > ng
    assert mom(_params(abi.PIC_MOM_N, order=8)) == abi.PIC_ERR_UNSUPPORTED
    assert mom(_params(abi.PIC_MOM_N, smoothing=0)) == abi.PIC_ERR_ARG
    assert mom(_params(abi.PIC_MOM_V, c1=0)) == abi.PIC_ERR_ARG
    assert mom(_params(abi.PIC_MOM_N), comp=6) == abi.PIC_ERR_ARG
    photons = _species(g, 1, mass=0.0, charge=0.0).to("cuda")
    arr2 = (abi.PicSpecies * 1)(mk(photons, 2))
    p = _params(abi.PIC_MOM_RHO)
    assert L.pic_output_moment(ctx.h, arr2, 1, C.byref(p), C.c_void_p(buf.data_ptr()), 0,
                               None) == abi.PIC_ERR_ARG
    p = _params(abi.PIC_MOM_T, c1=0, c2=1)
    assert L.pic_output_moment(ctx.h, arr2, 1, C.byref(p), C.c_void_p(buf.data_ptr()), 0,
                               None) == abi.PIC_OK
    dwn = (C.c_int32 * 3)(1, 1, 1)
    out = torch.zeros((3, 8, 8), device="cuda")
    both = abi.PIC_OUT_INTERP_EDGES | abi.PIC_OUT_INTERP_FACES
    assert L.pic_output_field(ctx.h, C.c_void_p(buf.data_ptr()), 1, 0, 3, both, 1.0, dwn,
                              C.c_void_p(out.data_ptr()), None) == abi.PIC_ERR_ARG
    assert L.pic_output_field(ctx.h, C.c_void_p(buf.data_ptr()), 1, 4, 3, 0, 1.0, dwn,
                              C.c_void_p(out.data_ptr()), None) == abi.PIC_ERR_ARG
    dwn0 = (C.c_int32 * 3)(0, 1, 1)
    assert L.pic_output_field(ctx.h, C.c_void_p(buf.data_ptr()), 1, 0, 3, 0, 1.0, dwn0,
                              C.c_void_p(out.data_ptr()), None) == abi.PIC_ERR_ARG
    assert L.pic_normalize_by_rho(ctx.h, C.c_void_p(buf.data_ptr()), 0, 0, 1, 2, None) == \
        abi.PIC_ERR_ARG
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]


def test_writer_round_trip(tmp_path):
    """OutputWriter writes the device-prepared arrays under the reference's
    names; they equal the oracle's."""
    from entity_gb300.output import OutputWriter, read_checkpoint, write_checkpoint
    g = GridSpec(dim=2, n=(16, 12, 1), order=2, real=torch.float32)
    o, ctx = Oracle(g), Context(g)
    sps = [_species(g, 21, index=1), _species(g, 22, charge=1.0, index=2)]
    sgs = [s.to("cuda") for s in sps]
    EB = random_fields(g, 3)
    J = random_fields(g, 4)[:3].contiguous()
    w = OutputWriter(ctx, g, str(tmp_path), fields=("E", "B", "J", "N_1", "Rho", "T0i", "V",
                                                     "divE", "Nppc_2"),
                     dx=0.5, n0=2.0, dwn=(2, 1), smooth_order=2, species=(1, 2), prtl_stride=5,
                     use_weights=True)
    path = w.write(7, 3.5, sgs, EB.cuda(), J.cuda())
    z = np.load(path)
    assert int(z["Step"]) == 7 and float(z["Time"]) == 3.5
    shape = (12, 8)
    out = torch.zeros((3,) + shape, dtype=torch.float32)
    o.output_field(EB, 1, 0, 3, abi.PIC_OUT_INTERP_EDGES | abi.PIC_OUT_TO_HAT, 0.5, (2, 1, 1),
                   out)
    for c in range(3):
        assert np.array_equal(z[f"fE{c + 1}"], out[c].numpy())
    inv_n0 = float(torch.tensor(1.0) / torch.tensor(2.0))
    bo = empty_field(g, 6)
    o.output_moment([sps[0]], dict(id=abi.PIC_MOM_N, order=2, smoothing=2, use_weights=1,
                                   inv_n0=inv_n0, dx=0.5), bo, 0)
    o.sync_moments(bo, 0, 1)
    no = torch.zeros((1,) + shape, dtype=torch.float32)
    o.output_field(bo, 1, 0, 1, 0, 0.5, (2, 1, 1), no)
    assert np.allclose(z["fN_1"], no[0].numpy(), rtol=0, atol=2e-5 * float(no.abs().max()))
    for name in ("fRho", "fT01", "fT02", "fT03", "fV1", "fV2", "fV3", "fDivE", "fNppc_2",
                 "fB1", "fJ3", "X1", "X1e", "X2", "pX1_1", "pU3_2", "pW_2"):
        assert name in z.files, name
    assert z["pX1_1"].shape == (sps[0].npart // 5,)
    assert np.allclose(z["X1"], (np.arange(8) * 2 + 0.5) * 0.5)
    # checkpoint round trip
    ck = str(tmp_path / "ck.npz")
    write_checkpoint(ck, 2, 9, 1.25, sgs, EB.cuda())
    back = [s.clone() for s in sgs]
    for s in back:
        s.u[0].zero_()
        s.npart = 0
    EB2 = torch.zeros_like(EB).cuda()
    assert read_checkpoint(ck, 2, back, EB2) == (9, 1.25)
    assert torch.equal(EB2.cpu(), EB)
    for a, b in zip(sgs, back):
        assert a.npart == b.npart and torch.equal(a.u[0], b.u[0])
