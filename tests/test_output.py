"""Output preparation: particle moments on the grid, cell-centred fields,
divE and particle records (pic_output_*), against the oracle and the
reference's known answers (tests/kernels/particle_moments.cpp,
tests/kernels/fields_to_phys.cpp, tests/kernels/prtls_to_phys.cpp)."""
import math

import numpy as np
import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec, empty_field, make_species
from entity_gb300.output import OutputField
from oracle.oracle import Oracle
from tests.helpers import random_fields, species_from_lists


def _bckp(g, device="cpu"):
    return empty_field(g, 6, device)


def _active(g, f, c):
    ng = g.ng
    if g.dim == 2:
        return f[c, 0, ng:ng + g.n[1], ng:ng + g.n[0]]
    return f[c, ng:ng + g.n[2], ng:ng + g.n[1], ng:ng + g.n[0]]


def _mom(mid, order=1, smoothing=2, c1=0, c2=0, use_weights=0, inv_n0=1.0, dx=1.0):
    return dict(id=mid, c1=c1, c2=c2, order=order, smoothing=smoothing, use_weights=use_weights,
                inv_n0=inv_n0, dx=dx)


def _known_answer_species(g):
    # tests/kernels/particle_moments.cpp:88-118: two alive particles
    return species_from_lists(g, [(5, 4), (2, 2)], [(0.15, 0.85), (0.22, 0.55)],
                              [(1.0, -2.0, 3.0), (-3.0, 2.0, -1.0)], mass=1.0, charge=1.0,
                              pusher=0)


@pytest.mark.parametrize("real", [torch.float32, torch.float64])
def test_moments_known_answer_on_oracle(real):
    """particle_moments.cpp: T^{0i} summed over each particle's cells gives
    u_i (so gamma^2 = 1 + |u|^2 = 15), N and Rho sum to 2, T^{00} to 2
    sqrt(15); window 1 (order 1), dx = 1, inv_n0 = 1."""
    g = GridSpec(dim=2, n=(10, 10, 1), order=1, real=real)
    o = Oracle(g)
    sp = _known_answer_species(g)
    buf = _bckp(g)
    for k, c in enumerate((1, 2, 3)):
        o.output_moment([sp], _mom(abi.PIC_MOM_T, c1=0, c2=c), buf, k)
    o.output_moment([sp], _mom(abi.PIC_MOM_N), buf, 3)
    o.output_moment([sp], _mom(abi.PIC_MOM_RHO), buf, 4)
    o.output_moment([sp], _mom(abi.PIC_MOM_T), buf, 5)
    eps = float(torch.finfo(real).eps) * 10
    b = buf.double()
    # ghost-inclusive x1 index below 6: the particle at i1 = 2; above: i1 = 5
    v2 = [float(b[c, 0, :, :6].sum()) for c in range(3)]
    v1 = [float(b[c, 0, :, 6:].sum()) for c in range(3)]
    for v in (v1, v2):
        assert abs(1.0 + sum(x * x for x in v) - 15.0) <= 15.0 * eps
    assert abs(float(b[3].sum()) - 2.0) <= 2.0 * eps
    assert abs(float(b[4].sum()) - 2.0) <= 2.0 * eps
    assert abs(float(b[5].sum()) - 2.0 * math.sqrt(15.0)) <= 8.0 * eps


@pytest.mark.parametrize("order", range(1, 7))
def test_splines_are_cardinal_bsplines(order):
    """prtl_shape::S1..S6 are the centred cardinal B-splines of degree 1..6."""
    from scipy.interpolate import BSpline
    g = GridSpec(dim=2, n=(8, 8, 1), order=1, real=torch.float64)
    o = Oracle(g)
    knots = np.arange(order + 2) - (order + 1) / 2.0
    b = BSpline.basis_element(knots, extrapolate=False)
    for x in np.linspace(0.0, (order + 1) / 2.0 + 0.5, 97):
        want = float(np.nan_to_num(b(x)))
        assert abs(o.spline(order, x) - want) <= 1e-13, (order, x)


def _random_species(g, ppc, seed, **kw):
    sp = make_species(g, ppc, 0.3, 0.2, seed, with_prev=False, **kw)
    gen = torch.Generator().manual_seed(seed + 7)
    sp.w = (0.5 + torch.rand(sp.w.shape, generator=gen, dtype=torch.float64)).to(g.real)
    sp.tag[torch.rand(sp.tag.shape, generator=gen) < 0.05] = 0
    return sp


@pytest.mark.parametrize("dim,order,mom_order,smoothing", [
    (2, 1, 0, 2), (2, 1, 1, 2), (2, 2, 2, 2), (2, 2, 3, 2), (2, 2, 4, 2), (2, 2, 4, 1),
    (3, 1, 2, 2), (3, 3, 5, 2), (3, 3, 6, 2), (3, 2, 3, 1)])
def test_number_density_sums_to_the_weights(dim, order, mom_order, smoothing):
    """Every window is a partition of unity, so after the periodic fold the
    number density over the active cells sums to sum(w) inv_n0 / dx^D."""
    n = (12, 10, 1) if dim == 2 else (8, 7, 6)
    g = GridSpec(dim=dim, n=n, order=order, real=torch.float64)
    o = Oracle(g)
    sp = _random_species(g, 3, 11)
    dx, inv_n0 = 0.5, 0.25
    buf = _bckp(g)
    o.output_moment([sp], _mom(abi.PIC_MOM_N, order=mom_order, smoothing=smoothing,
                               use_weights=1, inv_n0=inv_n0, dx=dx), buf, 2)
    o.sync_moments(buf, 2, 3)
    alive = sp.tag[:sp.npart] == 1
    want = float(sp.w[:sp.npart][alive].sum()) * inv_n0 / dx ** dim
    assert abs(float(_active(g, buf, 2).sum()) - want) <= 1e-11 * want
    # Nppc counts particles without volume or weight
    buf.zero_()
    o.output_moment([sp], _mom(abi.PIC_MOM_NPPC, order=mom_order, smoothing=smoothing,
                               use_weights=1, inv_n0=inv_n0, dx=dx), buf, 0)
    o.sync_moments(buf, 0, 1)
    assert abs(float(_active(g, buf, 0).sum()) - float(alive.sum())) <= 1e-10 * float(alive.sum())


def test_bulk_velocity_of_a_drifting_beam():
    """V normalised by Rho is u_i / u^0 wherever particles deposit, when all
    particles share one momentum (NormalizeVectorByRho)."""
    g = GridSpec(dim=2, n=(10, 8, 1), order=2, real=torch.float64)
    o = Oracle(g)
    sp = _random_species(g, 2, 5)
    u = (0.3, -0.4, 1.2)
    for d in range(3):
        sp.u[d].fill_(u[d])
    sp.tag.fill_(1)
    buf = _bckp(g)
    for k in range(3):
        o.output_moment([sp], _mom(abi.PIC_MOM_V, order=2, c1=k + 1), buf, 3 + k)
    o.sync_moments(buf, 3, 6)
    o.output_moment([sp], _mom(abi.PIC_MOM_RHO, order=2), buf, 0)
    o.sync_moments(buf, 0, 1)
    o.normalize_by_rho(buf, 0, (3, 4, 5))
    u0 = math.sqrt(1 + sum(x * x for x in u))
    for k in range(3):
        v = _active(g, buf, 3 + k)
        assert torch.allclose(v, torch.full_like(v, u[k] / u0), rtol=1e-12, atol=0)


def test_fields_to_phys_known_answer_on_oracle():
    """tests/kernels/fields_to_phys.cpp: from(5, 5) = (1, 2, 3) on a 10 x 10
    grid with 2 ghosts, interpolated from edges and from faces."""
    g = GridSpec(dim=2, n=(10, 10, 1), order=1, real=torch.float32)
    o = Oracle(g)
    J = empty_field(g, 3)
    J[:, 0, 5, 5] = torch.tensor([1.0, 2.0, 3.0])
    out = torch.zeros((3, 10, 10), dtype=torch.float32)
    o.output_field(J, 0, 0, 3, abi.PIC_OUT_INTERP_EDGES, 1.0, (1, 1, 1), out)
    # out[c][i2][i1] at active cells (i1, i2)
    assert out[0, 2, 3] == 0.5 and out[0, 3, 3] == 0.5
    assert out[1, 3, 2] == 1.0 and out[1, 3, 3] == 1.0
    for a, b in ((2, 2), (3, 2), (2, 3), (3, 3)):
        assert out[2, b, a] == 0.75
    o.output_field(J, 0, 0, 3, abi.PIC_OUT_INTERP_FACES, 1.0, (1, 1, 1), out)
    assert out[0, 3, 2] == 0.5 and out[0, 3, 3] == 0.5
    assert out[1, 2, 3] == 1.0 and out[1, 3, 3] == 1.0
    assert out[2, 3, 3] == 3.0


def test_field_output_downsamples_and_converts_to_hat():
    g = GridSpec(dim=3, n=(9, 7, 5), order=2, real=torch.float64)
    o = Oracle(g)
    EB = random_fields(g, 4)
    dwn = (2, 3, 2)
    shape = tuple(math.ceil(g.n[d] / dwn[d]) for d in (2, 1, 0))
    out = torch.zeros((3,) + shape, dtype=torch.float64)
    o.output_field(EB, 1, 3, 3, abi.PIC_OUT_INTERP_FACES | abi.PIC_OUT_TO_HAT, 0.5, dwn, out)
    ng = g.ng
    for (k, j, i) in ((0, 0, 0), (2, 2, 4), (1, 1, 3)):
        I, J_, K = i * dwn[0] + ng, j * dwn[1] + ng, k * dwn[2] + ng
        want = [0.5 * (EB[3, K, J_, I] + EB[3, K, J_, I + 1]),
                0.5 * (EB[4, K, J_, I] + EB[4, K, J_ + 1, I]),
                0.5 * (EB[5, K, J_, I] + EB[5, K + 1, J_, I])]
        for c in range(3):
            assert float(out[c, k, j, i]) == float(want[c] * 0.5)


def test_divergence_on_oracle():
    g = GridSpec(dim=3, n=(6, 5, 4), order=1, real=torch.float64)
    o = Oracle(g)
    EB = random_fields(g, 8)
    buf = _bckp(g)
    o.output_divergence(EB, buf, 2)
    E = EB.numpy()
    ng = g.ng
    a = slice(ng, ng + 6)
    b_ = slice(ng, ng + 5)
    c_ = slice(ng, ng + 4)
    want = (E[0, c_, b_, a] - E[0, c_, b_, ng - 1:ng + 5] + E[1, c_, b_, a] -
            E[1, c_, ng - 1:ng + 4, a] + E[2, c_, b_, a] - E[2, ng - 1:ng + 3, b_, a])
    assert np.allclose(_active(g, buf, 2).numpy(), want, rtol=0, atol=1e-15)


def test_particle_records_on_oracle():
    g = GridSpec(dim=2, n=(10, 10, 1), order=1, real=torch.float32)
    o = Oracle(g)
    sp = _random_species(g, 1, 3)
    stride, dx, xmin = 3, 0.25, (-1.5, 2.0, 0.0)
    n = sp.npart // stride
    x = [torch.zeros(n, dtype=torch.float32) for _ in range(2)]
    u = [torch.zeros(n, dtype=torch.float32) for _ in range(3)]
    w = torch.zeros(n, dtype=torch.float32)
    assert o.output_particles(sp, stride, dx, xmin, x, u, w) == n
    idx = torch.arange(n) * stride
    for d in range(2):
        xc = sp.i[d][idx].to(torch.float32) + sp.dx[d][idx]
        assert torch.equal(x[d], xc * torch.tensor(dx, dtype=torch.float32) +
                           torch.tensor(xmin[d], dtype=torch.float32))
    for d in range(3):
        assert torch.equal(u[d], sp.u[d][idx])
    assert torch.equal(w, sp.w[idx])


def test_output_field_names():
    """OutputField names (src/output/fields.h:86-150)."""
    assert OutputField("E").names() == ["fE1", "fE2", "fE3"]
    assert OutputField("N_1_2").name() == "fN_1_2"
    assert OutputField("T0i").names() == ["fT01", "fT02", "fT03"]
    assert OutputField("Tii_2").names() == ["fT11_2", "fT22_2", "fT33_2"]
    assert OutputField("T00").name() == "fT00"
    assert OutputField("V_1").names() == ["fV1_1", "fV2_1", "fV3_1"]
    assert OutputField("divE").name() == "fDivE"
    with pytest.raises(ValueError):
        OutputField("Tij")
    with pytest.raises(ValueError):
        OutputField("Bogus")
