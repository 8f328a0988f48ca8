"""pic_srpic_step_host: a domain whose state lives in pinned host memory
steps to the same state as the device-resident pic_srpic_step, with every
step's copies overlapped through the pipe."""
import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, SpeciesArrays, empty_field, make_species
from entity_gb300.sim import Context, HostPipe, step_params
from tests.helpers import random_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _pinned(sp):
    pin = lambda t: None if t is None else t.cpu().pin_memory()
    return SpeciesArrays([pin(x) for x in sp.i], [pin(x) for x in sp.dx],
                         [None] * len(sp.i_prev), [None] * len(sp.dx_prev),
                         [pin(x) for x in sp.u], pin(sp.w), pin(sp.tag), sp.mass, sp.charge,
                         sp.pusher, sp.npart, sp.index)


@pytest.mark.parametrize("nsteps", [9, 10])
@pytest.mark.parametrize("dim,sort_tiled,clear,deposit", [
    (2, False, 100, True), (3, False, 100, True), (2, True, 100, True), (3, True, 3, True),
    (2, True, 100, False)])
def test_host_resident_steps_match_device_steps(dim, sort_tiled, clear, deposit, nsteps):
    """Tiled sorts split each species into tile groups that are copied and
    pushed one by one; dead removal changes the counts and the groups. The
    weights go back to the host only on steps that sort (the last step sorts
    with 9 steps, not with 10 unless it clears), and end up equal all the
    same."""
    n = (32, 24, 1) if dim == 2 else (16, 16, 8)
    g = GridSpec(dim=dim, n=n, order=2, real=torch.float64)
    prm = step_params(g, cfl=0.45, ppc0=8.0, skindepth0=4.0, larmor0=3.0, nfilter=2,
                      sort_interval=2, clear_interval=clear, write_prev=True,
                      sort_tiled=sort_tiled, deposit=deposit)
    sps = [make_species(g, 4, 0.2, 0.3, 31, charge=-1.0),
           make_species(g, 4, 0.2, -0.3, 32, charge=1.0, index=2)]
    for s in sps:   # a few dead particles for the sort's dead removal
        s.tag[::97] = 0
    EB0 = random_fields(g, 5, amp=0.05)
    # reference: device-resident steps
    ctx = Context(g)
    da = [s.clone().to("cuda") for s in sps]
    EBa, Ja, Ba = EB0.cuda(), empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    for k in range(nsteps):
        ctx.step(da, EBa, Ja, Ba, prm, k)
    # host-resident: the state lives in pinned memory; the device arrays are
    # mirrors that start out as garbage
    ctx2 = Context(g)
    hs = [_pinned(s) for s in sps]
    ds = [s.clone().to("cuda") for s in sps]
    for s in ds:
        for t in s.u:
            t.fill_(123.0)
    hEB, hJ = EB0.clone().pin_memory(), empty_field(g, 3).pin_memory()
    EBb = torch.full_like(EBa, 7.0)
    Jb, Bb = empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    pipe = HostPipe()
    pipe.set_groups(4, 1)   # small species: still several groups each
    for k in range(nsteps):
        n_in = [h.npart for h in hs]  # the last call copies these counts in
        ctx2.step_host(pipe, hs, ds, hEB, EBb, hJ, Jb, Bb, prm, k)
    pipe.sync()
    torch.cuda.synchronize()
    nin, nout = pipe.bytes()
    pipe.close()
    assert ctx.device_errors() == [0, 0, 0, 0] and ctx2.device_errors() == [0, 0, 0, 0]
    scale = float(EBa.abs().max())
    assert float((hEB - EBa.cpu()).abs().max()) <= 1e-10 * scale
    assert float((hJ - Ja.cpu()).abs().max()) <= 1e-10 * max(float(Ja.abs().max()), 1e-30)
    rb = 8
    per = dim * 8 + 4 * rb + 2  # i, dx, u, w, tag
    want_in = hEB.numel() * rb + sum(n * per for n in n_in)
    want_out = hEB.numel() * rb
    for a, h in zip(da, hs):
        assert h.npart == a.npart
        m = a.npart
        for d in range(dim):
            assert torch.equal(h.i[d][:m], a.i[d][:m].cpu())
            assert float((h.dx[d][:m] - a.dx[d][:m].cpu()).abs().max()) <= 1e-5
        for d in range(3):
            assert torch.allclose(h.u[d][:m], a.u[d][:m].cpu(), rtol=1e-10, atol=1e-12)
        assert torch.equal(h.tag[:m], a.tag[:m].cpu())
        assert torch.equal(h.w[:m], a.w[:m].cpu())
        want_out += m * per
    last = nsteps - 1
    last_sorts = last % 2 == 0 or (last % clear == 0 and last > 0)
    weights_out = 0 if last_sorts else sum(h.npart * rb for h in hs)
    assert nin == want_in
    assert nout == want_out - weights_out + (hJ.numel() * rb if deposit else 0)
    if clear == 3:
        assert all(h.npart < s.npart for h, s in zip(hs, sps))  # the dead were removed
