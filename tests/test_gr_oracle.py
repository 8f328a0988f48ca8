"""Pins the GR oracle (QKerrSchild metric and transforms) to the reference's
own metric tests.

tests/metrics/ks-qks.cpp:185-197 builds QKerrSchild on a 32 x 42 grid over
r in [0.8, 10], theta in [0, pi] with r0 = -2, h = 0, a = 0.8, and checks at
every cell centre that h^ij and h_ij, converted to the physical basis
(transform U -> PU and D -> PD, qkerr_schild.h:735-760), equal the analytic
Kerr-Schild components, to 10 machine epsilons. The same comparison runs here
against the analytic expressions evaluated in FP64. The metric derivatives
the GR pusher uses are checked against central differences of the oracle's
own metric functions (the alternative the reference keeps commented out in
gr.hpp:286-305), and the vector transforms against the invariance of
u_i u^i between the covariant and tetrad bases.
"""
import math

import pytest
import torch

from entity_gb300.inputs import GridSpec
from oracle.oracle import GROracle

REALS = [torch.float32, torch.float64]
EPS = {torch.float32: 1.1920929e-07, torch.float64: 2.220446049250313e-16}


def _qks(real, n=(32, 42), a=0.8, r0=-2.0, rmin=0.8, rmax=10.0):
    g = GridSpec(dim=2, n=(n[0], n[1], 1), order=1, real=real)
    return GROracle(g, a=a, r_min=rmin, r_max=rmax, r0=r0), g


def _centres(n):
    i = torch.arange(n[0], dtype=torch.float64) + 0.5
    j = torch.arange(n[1], dtype=torch.float64) + 0.5
    I, Jm = torch.meshgrid(i, j, indexing="ij")
    return torch.stack([I.reshape(-1), Jm.reshape(-1)], 1)


@pytest.mark.parametrize("real", REALS)
def test_qks_metric_matches_kerr_schild(real):
    o, g = _qks(real)
    q = o.q
    x = _centres((32, 42))
    m = o.metric(x)
    chi = x[:, 0] * q.dchi + q.chi_min
    r = q.r0 + torch.exp(chi)
    th = x[:, 1] * q.deta + q.eta_min
    a = q.a
    S = r * r + (a * torch.cos(th)) ** 2
    z = 2 * r / S
    Dl = r * r - 2 * r + a * a
    A = (r * r + a * a) ** 2 - (a * torch.sin(th)) ** 2 * Dl
    s2 = torch.sin(th) ** 2
    # physical-basis factors of transform<U, PU> / <D, PD> (h = 0)
    fr = torch.exp(chi) * q.dchi
    ft = q.deta
    expect = {
        "h11": (m["h11"] * fr * fr, A / (S * (S + 2 * r))),
        "h22": (m["h22"] * ft * ft, 1 / S),
        "h33": (m["h33"], 1 / (S * s2)),
        "h13": (m["h13"] * fr, a / S),
        "h_11": (m["h_11"] / (fr * fr), 1 + z),
        "h_22": (m["h_22"] / (ft * ft), S),
        "h_33": (m["h_33"], A * s2 / S),
        "h_13": (m["h_13"] / fr, -a * (1 + z) * s2),
        "alpha": (m["alpha"], 1 / torch.sqrt(1 + z)),
        "beta1": (m["beta1"] * fr, z / (1 + z)),
        "sqrt_det_h": (m["sqrt_det_h"] / (fr * ft), S * torch.sin(th) * torch.sqrt(1 + z)),
    }
    # the FP32 oracle evaluates exp/sin/cos in float from float coordinates
    # (near the poles sin(theta) carries the rounding of theta itself);
    # the FP64 expectation is exact to rounding, so allow a few tens of eps
    tol = (100 if real == torch.float32 else 10) * EPS[real]
    for k, (got, want) in expect.items():
        rel = ((got - want).abs() / want.abs()).max()
        assert float(rel) <= tol, (k, float(rel))


def test_qks_derivatives_match_central_differences():
    o, g = _qks(torch.float64)
    x = _centres((32, 42))
    x = x[(x[:, 1] > 2) & (x[:, 1] < 40)]  # away from the poles
    m = o.metric(x)
    h = 1e-5
    for d, tag in ((0, "dr"), (1, "dt")):
        xp, xm = x.clone(), x.clone()
        xp[:, d] += h
        xm[:, d] -= h
        mp, mm = o.metric(xp), o.metric(xm)
        for f in ("alpha", "beta1", "h11", "h22", "h33", "h13"):
            fd = (mp[f] - mm[f]) / (2 * h)
            an = m[f"{tag}_{f}"]
            scale = float(an.abs().max()) + 1e-300
            err = float((fd - an).abs().max()) / scale
            assert err < 1e-6, (tag, f, err)


@pytest.mark.parametrize("real", REALS)
def test_transforms_preserve_the_norm(real):
    o, g = _qks(real, a=0.95, r0=0.0, rmin=1.2, rmax=50.0, n=(64, 48))
    x = _centres((64, 48))
    x = x[(x[:, 1] > 1) & (x[:, 1] < 47)]
    gen = torch.Generator().manual_seed(1)
    v = torch.rand((x.shape[0], 3), generator=gen, dtype=torch.float64) * 2 - 1
    vc = o.transform(0, x, v)      # covariant -> contravariant
    vt = o.transform(2, x, v)      # covariant -> tetrad
    back = o.transform(3, x, vt)   # tetrad -> covariant
    n_cov = (v * vc).sum(1)
    n_tet = (vt * vt).sum(1)
    tol = 200 * EPS[real]
    assert float(((n_cov - n_tet).abs() / n_tet.abs()).max()) < tol
    assert float(((back - v).abs()).max()) < tol * 10
    # contravariant -> tetrad of u^i equals covariant -> tetrad of u_i
    vt2 = o.transform(1, x, vc)
    assert float(((vt2 - vt).abs()).max()) < tol * 10


def test_geodesic_push_conserves_killing_energy_and_angular_momentum():
    """Without fields the GR pusher integrates geodesics of the stationary,
    axisymmetric Kerr metric: u_phi (= u_3) is kept to rounding and the Killing
    energy -u_t = alpha sqrt(1 + h^ij u_i u_j) - beta^1 u_1 to the accuracy of
    the implicit midpoint scheme."""
    from entity_gb300.inputs import SpeciesArrays, empty_field
    g = GridSpec(dim=2, n=(64, 48, 1), order=2, real=torch.float64, periodic=(0, 0, 0),
                 prtl_bc=((1, 1), (3, 3), (0, 0)))
    rh = 1.0 + math.sqrt(1.0 - 0.95 ** 2)
    o = GROracle(g, a=0.95, r_min=0.9 * rh, r_max=20.0)
    q = o.q
    # a few particles at rest or with angular momentum, r ~ 8..14, mid-latitudes
    r = torch.tensor([8.0, 10.0, 12.0, 14.0], dtype=torch.float64)
    th = torch.tensor([1.2, 1.5708, 1.0, 2.0], dtype=torch.float64)
    x1 = (torch.log(r - q.r0) - q.chi_min) / q.dchi
    x2 = (th - q.eta_min) / q.deta
    n = 4
    i1, i2 = x1.floor().to(torch.int32), x2.floor().to(torch.int32)
    d1, d2 = (x1 - i1).to(torch.float32), (x2 - i2).to(torch.float32)
    u = [torch.zeros(n, dtype=torch.float64), torch.zeros(n, dtype=torch.float64),
         torch.tensor([0.0, 1.0, 2.0, -1.5], dtype=torch.float64)]
    z = torch.zeros(n, dtype=torch.int32)
    zf = torch.zeros(n, dtype=torch.float32)
    sp = SpeciesArrays([i1, i2, z.clone()], [d1, d2, zf.clone()], [i1.clone(), i2.clone(), z.clone()],
                       [d1.clone(), d2.clone(), zf.clone()], u, torch.ones(n, dtype=torch.float64),
                       torch.ones(n, dtype=torch.int16), 1.0, -1.0, 1, n, 1)
    em = empty_field(g, 6)

    def energy():
        x = torch.stack([sp.i[0].double() + sp.dx[0].double(),
                         sp.i[1].double() + sp.dx[1].double()], 1)
        m = o.metric(x)
        uu = torch.stack(sp.u, 1)
        uc = o.transform(0, x, uu)
        return m["alpha"] * torch.sqrt(1 + (uu * uc).sum(1)) - m["beta1"] * sp.u[0]

    E0 = energy()
    u3 = sp.u[2].clone()
    for _ in range(200):
        o.gr_push(sp, em, em, 0.05, 1.0, 10)
    assert torch.equal(sp.tag, torch.ones(n, dtype=torch.int16))
    # the half E pushes round-trip u through the tetrad basis: exact up to rounding
    assert torch.allclose(sp.u[2], u3, rtol=1e-12, atol=1e-12)
    assert float(((energy() - E0) / E0).abs().max()) < 1e-3


@pytest.mark.parametrize("real", REALS)
def test_match_layer_relaxes_to_the_target(real):
    """MatchBoundaries_kernel (fields_bcs.hpp:181-340): s = tanh(4 |r - r_max|
    / ds) is 0 at r_max and ~1 a layer-width inside, so a field equal to the
    target plus a perturbation keeps the perturbation in the interior, loses
    it at the edge, and equals the target after repeated application
    wherever s < 1; cells below the layer are never touched."""
    from entity_gb300.inputs import empty_field
    o, g = _qks(real, n=(64, 16), a=0.9, r0=0.0, rmin=1.2, rmax=20.0)
    ds = 3.0
    T = empty_field(g, 6)
    gen = torch.Generator().manual_seed(5)
    T.copy_(torch.rand(T.shape, generator=gen, dtype=torch.float64).to(real))
    F0 = T + 0.5
    F = F0.clone()
    o.gr_match(F, T, ds, 1, 1, axis_min=0, axis_max=0)
    ng = g.ng
    # the layer's first cell: floor(x1(r_max - ds)) (ExtentToRange)
    chi = lambda r: math.log(r)
    x1 = lambda r: (chi(r) - chi(1.2)) / ((chi(20.0) - chi(1.2)) / 64)
    i0 = int(math.floor(x1(20.0 - ds))) + ng
    assert torch.equal(F[:, 0, :, :i0], F0[:, 0, :, :i0])
    dev = (F - T)[:, 0, :, i0:].abs()
    assert float(dev.max()) <= 0.5 + 1e-6
    # at r_max (i1 = n1 + ng, x1 = n1) the components at integer x1 match exactly
    edge = (F - T)[[1, 2, 3], 0, :, 64 + ng].abs()
    assert float(edge.max()) <= 1e-5
    for _ in range(400):
        o.gr_match(F, T, ds, 1, 1, axis_min=0, axis_max=0)
    # within a cell of the edge s <= tanh(4 dr / ds) ~ 0.83: the perturbation
    # is gone after 400 passes; deeper in, less of it is removed
    assert float((F - T)[:, 0, :, 64 + ng - 1:].abs().max()) <= 1e-4
    depth = (F - T)[3, 0, 4, i0:64 + ng].abs().double()
    assert torch.all(depth[1:] <= depth[:-1] + 1e-6)


@pytest.mark.parametrize("real", REALS)
def test_absorb_currents_layer(real):
    """AbsorbCurrents_kernel: J *= tanh(|r - r_max| / (ds / 4)); zero at
    r_max, untouched below the layer."""
    from entity_gb300.inputs import empty_field
    o, g = _qks(real, n=(64, 16), a=0.9, r0=0.0, rmin=1.2, rmax=20.0)
    J = empty_field(g, 3)
    J.fill_(1.0)
    o.gr_absorb_currents(J, 3.0)
    ng = g.ng
    assert float(J[:, 0, :, 64 + ng].abs().max()) <= 1e-5
    assert torch.all(J[:, 0, :, :40] == 1.0)
    prof = J[0, 0, 5, 40:64 + ng + 1].double()
    assert torch.all(prof[1:] <= prof[:-1] + 1e-7)   # decays toward r_max
