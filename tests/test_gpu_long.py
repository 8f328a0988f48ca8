"""Long-horizon parity: 100 whole steps of boxes shaped like the benchmark
plasmas through pic_srpic_step, against the oracle's step sequence (which is
bit-exact with the reference's own kernels, tests/test_ref_pin.py).

  * turbulence box: 3D, 32^3 cells, e-/e+ 8 ppc each, u_th = 0.3c, order 2,
    4 filter passes, B0 z + 8 random-phase modes with dB/B0 = 1, tiled sort
    every 8 steps (the benchmark's hot kernel and cadence);
  * pair plasma: 2D, 64^2 cells, e-/e+ 16 ppc each, drift +-0.3c along x,
    u_th = 0.1c, order 1, no filter, tiled sort every 16 steps.

The oracle applies the same tile-major sort, so the particle arrays stay in
the same order on both sides. The GPU sums J in another order (fixed point
per tile, then float atomics), so the runs differ by round-off in J from the
first step, and that difference grows with the plasma's dynamics.

Bars after 100 steps (FP32; FP64 in parentheses), written relative to each
quantity's maximum:
  positions  |x_gpu - x_oracle| <= 1e-3 cells (1e-9),
  momenta    |u_gpu - u_oracle| <= 1e-3 max|u| (1e-9),
  E, B, J    |f_gpu - f_oracle| <= 2e-3 max|f| (2e-9),
and the cells of at least 99.9 % of the particles identical (all in FP64).
"""
import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, make_species, turbulent_field
from entity_gb300.sim import Context, step_params

pytestmark = pytest.mark.gpu

TOL = {torch.float32: dict(x=1e-3, u=1e-3, f=2e-3, cells=0.999),
       torch.float64: dict(x=1e-9, u=1e-9, f=2e-9, cells=1.0)}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _setup(shape, real):
    if shape == "turb3d":
        g = GridSpec(dim=3, n=(32, 32, 32), order=2, real=real)
        prm = step_params(g, cfl=0.45, ppc0=16.0, skindepth0=10.0, larmor0=10.0, nfilter=4,
                          sort_interval=8, sort_tiled=True)
        EB = turbulent_field(g, 0.1, 1.0, 8, seed=2)
        sp = [make_species(g, 8, 0.09, 0.0, 11, charge=-1.0, index=1),
              make_species(g, 8, 0.09, 0.0, 12, charge=1.0, index=2)]
    else:
        g = GridSpec(dim=2, n=(64, 64, 1), order=1, real=real)
        prm = step_params(g, cfl=0.45, ppc0=32.0, skindepth0=10.0, larmor0=10.0, nfilter=0,
                          sort_interval=16, sort_tiled=True)
        EB = empty_field(g, 6)
        sp = [make_species(g, 16, 0.01, 0.3, 11, charge=-1.0, index=1),
              make_species(g, 16, 0.01, -0.3, 12, charge=1.0, index=2)]
    return g, prm, EB, sp


@pytest.mark.parametrize("real", [torch.float32, torch.float64])
@pytest.mark.parametrize("shape", ["turb3d", "pair2d"])
def test_100_steps_track_oracle(shape, real):
    from oracle.oracle import Oracle
    g, prm, EB, sp = _setup(shape, real)
    ctx = Context(g)
    tile = ctx.tile_shape()
    o = Oracle(g)
    # the oracle sorts as the GPU does: tile-major (checked bit-exact by
    # tests/test_gpu_tiled.py), in place of the reference's cell key
    o.sort = lambda s: o.sort_tiled(s, tile)
    so = [s.clone() for s in sp]
    sg = [s.clone().to("cuda") for s in sp]
    EBo, Jo, Bo = EB.clone(), empty_field(g, 3), empty_field(g, 3)
    EBg, Jg, Bg = EB.cuda(), empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")
    for step in range(100):
        o.step(so, EBo, Jo, Bo, prm, step)
        ctx.step(sg, EBg, Jg, Bg, prm, step)
    torch.cuda.synchronize()
    assert ctx.device_errors()[:3] == [0, 0, 0]
    t = TOL[real]
    same = total = 0
    for a, b in zip(so, sg):
        assert a.npart == b.npart
        for d in range(g.dim):
            xa = a.i[d].double() + a.dx[d].double()
            xb = b.i[d].cpu().double() + b.dx[d].cpu().double()
            # a periodic wrap puts the same position n cells apart
            dxp = (xa - xb).abs()
            dxp = torch.minimum(dxp, (dxp - g.n[d]).abs())
            assert float(dxp.max()) <= t["x"], f"x{d + 1}: {float(dxp.max())}"
        ok = torch.ones(a.npart, dtype=torch.bool)
        for d in range(g.dim):
            ok &= a.i[d] == b.i[d].cpu()
        same += int(ok.sum())
        total += a.npart
        umax = max(float(a.u[d].abs().max()) for d in range(3))
        for d in range(3):
            du = float((a.u[d].double() - b.u[d].cpu().double()).abs().max())
            assert du <= t["u"] * umax, f"u{d + 1}: {du} vs {umax}"
    assert same >= t["cells"] * total, (same, total)
    for name, fo, fg in (("E", EBo[:3], EBg[:3]), ("B", EBo[3:], EBg[3:]), ("J", Jo, Jg)):
        scale = float(fo.abs().max())
        diff = float((fo.double() - fg.cpu().double()).abs().max())
        assert diff <= t["f"] * scale, f"{name}: {diff} vs {scale}"
