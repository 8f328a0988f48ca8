"""Edge cases of the SR path on the GPU: empty species, a single particle,
a species whose particles are all dead, and the host-side limits.

Empty and single-particle species go through every phase of the step (the
reference skips species with npart 0 in ParticlePush and CurrentsDeposit,
particle_pusher.h / currents.h:69-86, and sorts them as empty bins); the
oracle's step is the bar. Counts at or above 2^31 are refused before any
device work (32-bit particle indices in the sort and the kernels).
"""
import ctypes as C

import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, empty_species, make_species
from entity_gb300.sim import Context, make_species as mk, step_params
from tests.helpers import random_fields
from tests.test_gpu_parity import _assert_particles_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _with_prev(sp):
    sp.i_prev = [x.clone() for x in sp.i]
    sp.dx_prev = [x.clone() for x in sp.dx]
    return sp


@pytest.mark.parametrize("real", [torch.float32, torch.float64])
@pytest.mark.parametrize("dim,order", [(2, 1), (3, 2)])
def test_steps_with_empty_and_single_particle_species(dim, order, real):
    from oracle.oracle import Oracle
    n = (16, 12, 1) if dim == 2 else (10, 8, 8)
    g = GridSpec(dim=dim, n=n, order=order, real=real)
    prm = step_params(g, cfl=0.45, ppc0=4.0, skindepth0=3.0, larmor0=2.0, nfilter=1,
                      sort_interval=2, write_prev=True)
    empty = _with_prev(empty_species(g, 8, charge=-1.0, index=1, device="cpu"))
    one = make_species(g, 1, 0.3, 0.2, 5, charge=1.0, index=2)
    for arr in (one.i, one.dx, one.i_prev, one.dx_prev, one.u):
        for k in range(len(arr)):
            if arr[k] is not None and arr[k].numel() > 1:
                arr[k] = arr[k][:1].clone()
    one.w, one.tag, one.npart = one.w[:1].clone(), one.tag[:1].clone(), 1
    EB = random_fields(g, 9, amp=0.05)
    o, ctx = Oracle(g), Context(g)
    so = [empty.clone(), one.clone()]
    sg = [empty.clone().to("cuda"), one.clone().to("cuda")]
    EBo, Jo, Bo = EB.clone(), empty_field(g, 3), empty_field(g, 3)
    EBg, Jg, Bg = EB.cuda(), empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    for step in range(4):
        o.step(so, EBo, Jo, Bo, prm, step)
        ctx.step(sg, EBg, Jg, Bg, prm, step)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]
    assert sg[0].npart == 0 and sg[1].npart == 1
    _assert_particles_equal(so[1], sg[1], dim)
    tol = 2e-4 if real == torch.float32 else 1e-10
    scale = float(EBo.abs().max())
    assert float((EBo.double() - EBg.cpu().double()).abs().max()) <= tol * scale


def test_sort_of_empty_and_all_dead_species():
    g = GridSpec(dim=3, n=(10, 8, 8), order=2, real=torch.float32)
    ctx = Context(g)
    empty = empty_species(g, 16, device="cuda")
    st = ctx.sort(empty, abi.PIC_SORT_REMOVE_DEAD | abi.PIC_SORT_SPATIAL | abi.PIC_SORT_SKIP_PREV)
    assert st == abi.PIC_OK and empty.npart == 0
    dead = make_species(g, 2, 0.1, 0.0, 3, device="cuda", with_prev=False)
    dead.tag.zero_()
    st = ctx.sort(dead, abi.PIC_SORT_REMOVE_DEAD | abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED |
                  abi.PIC_SORT_SKIP_PREV)
    torch.cuda.synchronize()
    assert st == abi.PIC_OK and dead.npart == 0
    assert ctx.device_errors() == [0, 0, 0, 0]


def test_push_deposit_with_no_particles_leaves_zero_current():
    g = GridSpec(dim=3, n=(10, 8, 8), order=2, real=torch.float32)
    ctx = Context(g)
    EB = random_fields(g, 2).cuda()
    J = empty_field(g, 3, "cuda")
    J.fill_(7.0)
    sp = [empty_species(g, 4, device="cuda"), empty_species(g, 4, charge=1.0, index=2,
                                                              device="cuda")]
    ctx.push_deposit(sp, EB, J, 0.3, 1.0, g.dx)
    torch.cuda.synchronize()
    assert torch.all(J == 0)


def test_counts_beyond_32_bit_indices_are_refused():
    g = GridSpec(dim=2, n=(8, 8, 1), order=1, real=torch.float32)
    ctx = Context(g)
    sp = make_species(g, 1, 0.1, 0.0, 1, device="cuda")
    ps = mk(sp, 2)
    ps.npart = ps.maxnpart = 1 << 31
    L = abi.load()
    EB = empty_field(g, 6, "cuda")
    st = L.pic_push(ctx.h, C.byref(ps), C.c_void_p(EB.data_ptr()), 0.3, 1.0, 1.0, None)
    assert st == abi.PIC_ERR_UNSUPPORTED
    n = C.c_int64(0)
    st = L.pic_sort(ctx.h, C.byref(ps), abi.PIC_SORT_SPATIAL, C.byref(n), None)
    assert st == abi.PIC_ERR_UNSUPPORTED
    # the context is still usable
    ctx.push(sp, EB, 0.3, 1.0, g.dx)
    torch.cuda.synchronize()
    assert ctx.device_errors() == [0, 0, 0, 0]


def test_sort_without_waiting_matches_the_waiting_sort():
    """PIC_SORT_NO_SYNC: same order as the waiting sort, no dead removal
    allowed, out-of-grid particles only counted in the error word; the tiled
    push that follows gives the same particles and J."""
    g = GridSpec(dim=3, n=(16, 12, 8), order=2, real=torch.float32)
    base = make_species(g, 3, 0.2, 0.1, 17, device="cpu", with_prev=False)
    base.tag[::13] = 0
    ca, cb = Context(g), Context(g)
    a, b = base.to("cuda"), base.to("cuda")
    fl = abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED | abi.PIC_SORT_SKIP_PREV
    assert ca.sort(a, fl) == abi.PIC_OK
    assert cb.sort(b, fl | abi.PIC_SORT_NO_SYNC) == abi.PIC_OK
    torch.cuda.synchronize()
    _assert_particles_equal(a.to("cpu"), b, 3, prev=False)
    EB = random_fields(g, 4, amp=0.05).cuda()
    Ja, Jb = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    ca.push_deposit([a], EB, Ja, 0.3, 1.0, g.dx)
    cb.push_deposit([b], EB, Jb, 0.3, 1.0, g.dx)
    torch.cuda.synchronize()
    _assert_particles_equal(a.to("cpu"), b, 3, prev=False)
    # the tile windows' overlapping halos are added with float atomics, in no
    # fixed order
    assert float((Ja - Jb).abs().max()) <= 4e-6 * float(Ja.abs().max())
    n = C.c_int64(0)
    st = abi.load().pic_sort(cb.h, C.byref(mk(b, 3)),
                             fl | abi.PIC_SORT_NO_SYNC | abi.PIC_SORT_REMOVE_DEAD, C.byref(n), None)
    assert st == abi.PIC_ERR_ARG
    b.i[0][0] = 10_000
    b.tag[0] = 1
    assert cb.sort(b, fl | abi.PIC_SORT_NO_SYNC) == abi.PIC_OK
    torch.cuda.synchronize()
    assert cb.device_errors(reset=True)[1] == 1


def test_tile_range_entry_points():
    """pic_tile_offsets / pic_push_deposit_tiles: refused without a tiled
    binning or with a bad range; covering the tiles in pieces gives the same
    particles as one pic_push_deposit."""
    g = GridSpec(dim=2, n=(48, 32, 1), order=1, real=torch.float64)
    L = abi.load()
    ctx = Context(g)
    sp = make_species(g, 4, 0.2, 0.2, 23, device="cuda", with_prev=False)
    nt = C.c_int64(0)
    ps = mk(sp, 2)
    assert L.pic_tile_offsets(ctx.h, C.byref(ps), None, 0, C.byref(nt), None) == \
        abi.PIC_ERR_UNSUPPORTED
    EB = random_fields(g, 8, amp=0.05).cuda()
    J = empty_field(g, 3, "cuda")
    args = (C.c_void_p(EB.data_ptr()), C.c_void_p(J.data_ptr()), 0.3, 1.0, 1.0)
    assert L.pic_push_deposit_tiles(ctx.h, C.byref(ps), *args, 0, 1, 0, None) == \
        abi.PIC_ERR_UNSUPPORTED
    assert ctx.sort(sp, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED | abi.PIC_SORT_SKIP_PREV) == \
        abi.PIC_OK
    ps = mk(sp, 2)
    assert L.pic_tile_offsets(ctx.h, C.byref(ps), None, 0, C.byref(nt), None) == abi.PIC_OK
    n = nt.value
    off = (C.c_int32 * (n + 1))()
    assert L.pic_tile_offsets(ctx.h, C.byref(ps), off, n + 1, C.byref(nt), None) == abi.PIC_OK
    assert off[0] == 0 and off[n] == sp.npart and all(off[t] <= off[t + 1] for t in range(n))
    assert L.pic_push_deposit_tiles(ctx.h, C.byref(ps), *args, 0, n + 1, 0, None) == \
        abi.PIC_ERR_ARG
    ref = sp.clone()
    Jr = empty_field(g, 3, "cuda")
    ctx.push_deposit([ref], EB, Jr, 0.3, 1.0, 1.0)
    for lo, hi in ((0, n // 3), (n // 3, n // 2), (n // 2, n)):
        st = L.pic_push_deposit_tiles(ctx.h, C.byref(ps), *args, lo, hi,
                                      abi.PIC_PD_NO_ZERO if lo else 0, None)
        assert st == abi.PIC_OK
    torch.cuda.synchronize()
    _assert_particles_equal(ref.to("cpu"), sp, 2, prev=False)
    assert float((J - Jr).abs().max()) <= 1e-12 * float(Jr.abs().max())
