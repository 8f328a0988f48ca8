"""The tiled push/deposit path (PIC_SORT_TILED + shared-memory windows).

After a tiled sort the particle order differs from the reference's cell key,
so the oracle starts from the GPU-sorted arrays; the bars are those of the
untiled path: particles bit-exact, J to round-off (summation order only).
Multi-step runs without re-sorting let particles drift past the window's
margin, which exercises the global-memory fallback inside the same kernel.
"""
import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, make_species
from entity_gb300.sim import Context
from tests.helpers import random_currents, random_fields
from tests.test_gpu_parity import J_TOL, _assert_J_close, _assert_particles_equal

pytestmark = pytest.mark.gpu

REALS = [torch.float32, torch.float64]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _oracle(g):
    from oracle.oracle import Oracle
    return Oracle(g)


def _grid(dim, order, real, **kw):
    # sizes that leave partial tiles at the upper edges
    n = (72, 40, 1) if dim == 2 else (20, 12, 10)
    return GridSpec(dim=dim, n=n, order=order, real=real, **kw)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("real", REALS)
def test_tiled_sort_matches_oracle(dim, real):
    g = _grid(dim, 2, real)
    sp = make_species(g, 5, 0.2, 0.0, 7)
    sp.tag[::17] = 0
    spg = sp.clone().to("cuda")
    ctx = Context(g)
    tile = ctx.tile_shape()
    _oracle(g).sort_tiled(sp, tile)
    assert ctx.sort(spg, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED) == abi.PIC_OK
    _assert_particles_equal(sp, spg, dim)


def _tiled_pair(g, seeds, temp, beta=0.3, **kw):
    """GPU species sorted by tile, and CPU copies in the same order."""
    ctx = Context(g)
    gpu, cpu = [], []
    for k, sd in enumerate(seeds):
        s = make_species(g, 4, temp, beta if k == 0 else -beta, sd,
                         charge=-1.0 if k == 0 else 1.0, index=k + 1, **kw).to("cuda")
        assert ctx.sort(s, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED) == abi.PIC_OK
        gpu.append(s)
        cpu.append(s.clone().to("cpu"))
    return ctx, gpu, cpu


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("dim", [2, 3])
def test_tiled_push_deposit(dim, order, real):
    g = _grid(dim, order, real)
    EB = random_fields(g, 5 + order)
    ctx, gpu, cpu = _tiled_pair(g, [31, 32], temp=0.3)
    o = _oracle(g)
    Jo = empty_field(g, 3)
    for s in cpu:
        o.push(s, EB, 0.45, 0.7, g.dx)
    o.deposit(cpu, Jo, 0.45, g.dx)
    o.sync_currents(Jo, empty_field(g, 3))
    o.fill_ghosts(Jo, False, 0, 3)
    Jg = empty_field(g, 3, "cuda")
    ctx.push_deposit(gpu, EB.cuda(), Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
    ctx.sync_currents(Jg)
    torch.cuda.synchronize()
    for a, b in zip(cpu, gpu):
        _assert_particles_equal(a, b, dim)
    _assert_J_close(Jo, Jg, real)
    assert ctx.device_errors() == [0, 0, 0, 0]


@pytest.mark.parametrize("real", REALS)
@pytest.mark.parametrize("dim,order", [(2, 1), (3, 2), (3, 3)])
def test_tiled_drift_beyond_margin(dim, order, real):
    # relativistic plasma pushed 8 times without re-sorting: the farthest
    # particles leave their tile by more than the drift margin
    g = _grid(dim, order, real)
    EB = random_fields(g, 77, amp=0.1)
    ctx, gpu, cpu = _tiled_pair(g, [41, 42], temp=2.0, beta=0.5)
    o = _oracle(g)
    EBg = EB.cuda()
    for step in range(8):
        Jo = empty_field(g, 3)
        for s in cpu:
            o.push(s, EB, 0.45, 0.7, g.dx)
        o.deposit(cpu, Jo, 0.45, g.dx)
        o.sync_currents(Jo, empty_field(g, 3))
        Jg = empty_field(g, 3, "cuda")
        ctx.push_deposit(gpu, EBg, Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
        ctx.sync_currents(Jg)
        torch.cuda.synchronize()
        for a, b in zip(cpu, gpu):
            _assert_particles_equal(a, b, dim)
        # compare the active cells (the oracle leaves raw deposits in ghosts)
        ng = g.ng
        sl = (slice(None), slice(None), slice(ng, -ng), slice(ng, -ng)) if dim == 2 else \
            (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))
        _assert_J_close(Jo[sl], Jg[sl], real)


@pytest.mark.parametrize("bc", [abi.PIC_BC_ABSORB, abi.PIC_BC_REFLECT])
def test_tiled_non_periodic_boundaries(bc):
    g = GridSpec(dim=3, n=(20, 12, 10), order=2, real=torch.float32, periodic=(0, 1, 1),
                 prtl_bc=((bc, bc), (0, 0), (0, 0)))
    EB = random_fields(g, 9)
    ctx, gpu, cpu = _tiled_pair(g, [51, 52], temp=1.0)
    o = _oracle(g)
    Jo = empty_field(g, 3)
    for s in cpu:
        o.push(s, EB, 0.45, 0.7, g.dx)
    o.deposit(cpu, Jo, 0.45, g.dx)
    o.sync_currents(Jo, empty_field(g, 3))
    o.fill_ghosts(Jo, False, 0, 3)
    Jg = empty_field(g, 3, "cuda")
    ctx.push_deposit(gpu, EB.cuda(), Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
    ctx.sync_currents(Jg)
    torch.cuda.synchronize()
    for a, b in zip(cpu, gpu):
        _assert_particles_equal(a, b, 3)
    # periodic axes folded; along the open axis the ghosts keep raw deposits
    _assert_J_close(Jo, Jg, torch.float32)


def test_tiled_falls_back_when_npart_changes():
    g = _grid(3, 2, torch.float32)
    EB = random_fields(g, 3)
    ctx, gpu, cpu = _tiled_pair(g, [61], temp=0.3)
    s = gpu[0]
    s.npart -= 10     # the binning no longer describes the arrays
    c = cpu[0]
    c.npart -= 10
    o = _oracle(g)
    Jo = empty_field(g, 3)
    o.push(c, EB, 0.45, 0.7, g.dx)
    o.deposit([c], Jo, 0.45, g.dx)
    Jg = empty_field(g, 3, "cuda")
    ctx.push_deposit([s], EB.cuda(), Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
    torch.cuda.synchronize()
    _assert_particles_equal(c, s, 3)
    _assert_J_close(Jo, Jg, torch.float32)


@pytest.mark.parametrize("dim,order,real", [(3, 2, torch.float32), (3, 2, torch.float64),
                                            (3, 1, torch.float32), (2, 1, torch.float32),
                                            (2, 2, torch.float64)])
def test_tma_window_matches_copy_loop(dim, order, real, monkeypatch):
    """The E/B window staged by the TMA box load equals the one the copy loop
    stages: particles bit for bit, J to the round-off of the tiles' float
    flush order. The grid has interior tiles (box load) and edge tiles whose
    windows wrap (copy loop) in the same launch."""
    n = (48, 32, 24) if dim == 3 else (96, 64, 1)
    g = GridSpec(dim=dim, n=n, order=order, real=real)
    EB = random_fields(g, 19).cuda()
    ctx, gpu, _ = _tiled_pair(g, [51, 52], temp=0.3)
    runs = []
    for no_tma in ("0", "1"):
        monkeypatch.setenv("ENTITY_PIC_NO_TMA", no_tma)
        sp = [s.clone() for s in gpu]
        Jg = empty_field(g, 3, "cuda")
        ctx.push_deposit(sp, EB, Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
        ctx.sync_currents(Jg)
        torch.cuda.synchronize()
        runs.append((sp, Jg.cpu()))
    for a, b in zip(runs[0][0], runs[1][0]):
        _assert_particles_equal(a.to("cpu"), b, dim)
    _assert_J_close(runs[1][1], runs[0][1].cuda(), real)
    assert ctx.device_errors() == [0, 0, 0, 0]
    assert ctx.wait_timeouts() == 0


@pytest.mark.parametrize("dim,order", [(3, 2), (3, 3), (2, 1)])
def test_exact_current_accumulation_repeats_bit_for_bit(dim, order):
    """FP32 J from the exact 64-bit accumulation is the same in every run,
    whatever order the tiles, the per-particle drain of the particles that
    left their tile's margin and an unsorted species add in; it agrees with
    the float-atomic deposit to round-off, and the particles are identical."""
    n = (40, 24, 16) if dim == 3 else (96, 64, 1)
    g = GridSpec(dim=dim, n=n, order=order, real=torch.float32)
    EB = random_fields(g, 23, amp=0.1).cuda()
    ctx, gpu, _ = _tiled_pair(g, [61, 62], temp=2.0, beta=0.5)
    # a third species the sort never binned: the per-particle kernel
    gpu.append(make_species(g, 3, 0.5, 0.1, 63, charge=-1.0, index=3).to("cuda"))
    runs = []
    for flags in (0, 0, abi.PIC_PD_FLOAT_ATOMICS):
        sp = [s.clone() for s in gpu]
        Js = []
        for _ in range(4):  # no re-sort: particles drift past the margin
            Jg = empty_field(g, 3, "cuda")
            ctx.push_deposit(sp, EB, Jg, 0.45, 0.7, g.dx,
                             flags=abi.PIC_PD_WRITE_PREV | flags)
            Js.append(Jg)
        torch.cuda.synchronize()
        runs.append((sp, Js))
    for Ja, Jb, Jf in zip(runs[0][1], runs[1][1], runs[2][1]):
        assert torch.equal(Ja, Jb)
        _assert_J_close(Jf.cpu(), Ja, torch.float32)
    for a, b in zip(runs[0][0], runs[2][0]):
        _assert_particles_equal(a.to("cpu"), b, dim)
    assert ctx.device_errors() == [0, 0, 0, 0]


def test_exact_current_accumulation_adds_to_J():
    """With PIC_PD_NO_ZERO the call adds its float totals to J: the same as
    depositing into zeros and adding in float."""
    g = GridSpec(dim=3, n=(24, 16, 16), order=2, real=torch.float32)
    EB = random_fields(g, 29, amp=0.1).cuda()
    ctx, gpu, _ = _tiled_pair(g, [71, 72], temp=0.3)
    J0 = random_currents(g, 30).cuda()
    Ja = J0.clone()
    ctx.push_deposit([s.clone() for s in gpu], EB, Ja, 0.45, 0.7, g.dx,
                     flags=abi.PIC_PD_WRITE_PREV | abi.PIC_PD_NO_ZERO)
    Jz = empty_field(g, 3, "cuda")
    ctx.push_deposit([s.clone() for s in gpu], EB, Jz, 0.45, 0.7, g.dx,
                     flags=abi.PIC_PD_WRITE_PREV)
    torch.cuda.synchronize()
    assert torch.equal(Ja, J0 + Jz)


@pytest.mark.parametrize("dim,order,ppc,temp", [
    (3, 1, 4, 0.3), (3, 2, 4, 0.05), (3, 2, 4, 2.0), (3, 3, 4, 0.3), (3, 1, 12, 2.0),
    (3, 2, 12, 2.0), (3, 3, 24, 2.0), (2, 1, 16, 0.3), (2, 2, 8, 0.3), (2, 1, 16, 2.0)])
def test_deposit_records_leave_J_unchanged(dim, order, ppc, temp, monkeypatch):
    """FP32, 3D orders 1-3 and 2D orders 1-2: the particles whose shape
    support moved are deposited from records after the tile's pushes, the
    others at once through the narrow stencil. J is the same to the bit as
    with every particle deposited at once (ENTITY_PIC_NO_RECORDS=1), because
    the window's integer sums do not
    depend on the order of the additions; the particles are identical. The
    hot 3D 2 x 12 ppc (orders 1-2), 2 x 24 ppc (order 3) and 2D 2 x 16 ppc
    cases fill a tile's record buffer past its capacity, so the particles
    beyond it are deposited at once as well. The 2D records carry the
    out-of-plane velocity of the third current component."""
    n = (32, 16, 16) if dim == 3 else (96, 64, 1)
    g = GridSpec(dim=dim, n=n, order=order, real=torch.float32)
    EB = random_fields(g, 37, amp=0.1).cuda()
    ctx = Context(g)
    gpu = []
    for k, sd in enumerate((81, 82)):
        s = make_species(g, ppc, temp, 0.3 if k == 0 else -0.3, sd,
                         charge=-1.0 if k == 0 else 1.0, index=k + 1).to("cuda")
        assert ctx.sort(s, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_TILED) == abi.PIC_OK
        gpu.append(s)
    runs = []
    for off in ("0", "1"):
        monkeypatch.setenv("ENTITY_PIC_NO_RECORDS", off)
        sp = [s.clone() for s in gpu]
        Js = []
        for _ in range(2):
            Jg = empty_field(g, 3, "cuda")
            ctx.push_deposit(sp, EB, Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
            Js.append(Jg)
        torch.cuda.synchronize()
        runs.append((sp, Js))
    for Ja, Jb in zip(runs[0][1], runs[1][1]):
        assert torch.equal(Ja, Jb)
        assert float(Ja.abs().max()) > 0
    for a, b in zip(runs[0][0], runs[1][0]):
        _assert_particles_equal(a.to("cpu"), b, dim)
    assert ctx.device_errors() == [0, 0, 0, 0]
    assert ctx.wait_timeouts() == 0


@pytest.mark.parametrize("dim,order", [(3, 2), (3, 3), (2, 1)])
def test_lane_stride_leaves_results_unchanged(dim, order, monkeypatch):
    """Which thread pushes which particle of a tile (ENTITY_PIC_LANE_STRIDE:
    1, 2 or 4 warps reading their particles interleaved) changes neither the
    particles nor the exactly accumulated FP32 J."""
    n = (40, 24, 16) if dim == 3 else (96, 64, 1)
    g = GridSpec(dim=dim, n=n, order=order, real=torch.float32)
    EB = random_fields(g, 43, amp=0.1).cuda()
    ctx, gpu, _ = _tiled_pair(g, [91, 92], temp=0.3)
    runs = []
    for ls in ("1", "2", "4"):
        monkeypatch.setenv("ENTITY_PIC_LANE_STRIDE", ls)
        sp = [s.clone() for s in gpu]
        Jg = empty_field(g, 3, "cuda")
        ctx.push_deposit(sp, EB, Jg, 0.45, 0.7, g.dx, flags=abi.PIC_PD_WRITE_PREV)
        torch.cuda.synchronize()
        runs.append((sp, Jg))
    for sp, Jg in runs[1:]:
        assert torch.equal(Jg, runs[0][1])
        for a, b in zip(runs[0][0], sp):
            _assert_particles_equal(a.to("cpu"), b, dim)
    assert ctx.device_errors() == [0, 0, 0, 0]
