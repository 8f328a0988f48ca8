"""Seeded synthetic plasmas with the shapes of the benchmark configurations.

No dataset is involved: particle positions, momenta and initial fields are
generated here from a seed, on CPU (for the oracle comparisons) or directly on
the GPU (for the full-size benchmark), with torch as the array backend.

Momenta follow the reference's sampler (src/archetypes/energy_dist.h:79-179):
Box-Muller per component for temperature < 0.5, the Sobol (1976) rejection
method otherwise, and the flipping-method boost of Zenitani (2015) for a
drift along x1.

Arrays use the field layout of the C ABI: field element (i1, i2, i3, c) at
i1 + N1*(i2 + N2*(i3 + N3*c)) for the ghost-inclusive extents N1, N2, N3
(Kokkos LayoutLeft), i.e. a torch tensor of shape (ncomp, N3, N2, N1).
"""
import math
from dataclasses import dataclass, field

import torch


@dataclass
class GridSpec:
    dim: int
    n: tuple            # active cells (n1, n2, n3); n3 = 1 in 2D
    order: int          # shape order 0..3
    real: torch.dtype   # torch.float32 or torch.float64
    ng: int = 0         # ghost layers (0 = the reference's N_GHOSTS for `order`)
    periodic: tuple = (1, 1, 1)
    prtl_bc: tuple = ((0, 0), (0, 0), (0, 0))
    extent: float = 0.0  # physical length of x1 (0 = n1, i.e. dx = 1)

    def __post_init__(self):
        if self.ng == 0:
            # N_GHOSTS (src/global/global.h:130-136); 2 for the zigzag default
            self.ng = 2 if self.order == 0 else (self.order + 1) // 2 + 1
        if self.extent == 0.0:
            self.extent = float(self.n[0])

    @property
    def ext(self):
        ng = self.ng
        return (self.n[0] + 2 * ng, self.n[1] + 2 * ng,
                self.n[2] + 2 * ng if self.dim == 3 else 1)

    @property
    def dx(self):
        # Minkowski dx = (x1max - x1min) / nx1 in real_t (src/metrics/minkowski.h:50-53)
        return float(torch.tensor(self.extent, dtype=self.real) /
                     torch.tensor(float(self.n[0]), dtype=self.real))

    @property
    def real_bytes(self):
        return 4 if self.real == torch.float32 else 8

    def strides(self):
        N1, N2, N3 = self.ext
        return (1, N1, N1 * N2, N1 * N2 * N3)

    def ncells(self):
        return self.n[0] * self.n[1] * (self.n[2] if self.dim == 3 else 1)


def empty_field(g: GridSpec, ncomp: int, device="cpu"):
    N1, N2, N3 = g.ext
    return torch.zeros((ncomp, N3, N2, N1), dtype=g.real, device=device)


@dataclass
class SpeciesArrays:
    """Structure of arrays of one species (ParticleArrays)."""
    i: list
    dx: list
    i_prev: list
    dx_prev: list
    u: list
    w: torch.Tensor
    tag: torch.Tensor
    mass: float = 1.0
    charge: float = -1.0
    pusher: int = 1
    npart: int = 0
    index: int = 1
    # optional: phi (real, 1D) and the payloads, 2D (particles x columns)
    # tensors of real (pld_r) and 32-bit integers (pld_i: the reference's
    # npart_t is uint32) with any strides
    phi: torch.Tensor = None
    pld_r: torch.Tensor = None
    pld_i: torch.Tensor = None

    def _extras(self, f):
        return [None if x is None else f(x) for x in (self.phi, self.pld_r, self.pld_i)]

    def to(self, device):
        mv = lambda xs: [None if x is None else x.to(device) for x in xs]
        return SpeciesArrays(mv(self.i), mv(self.dx), mv(self.i_prev), mv(self.dx_prev),
                             mv(self.u), self.w.to(device), self.tag.to(device), self.mass,
                             self.charge, self.pusher, self.npart, self.index,
                             *self._extras(lambda x: x.to(device)))

    def astype(self, real):
        """A copy whose momenta and weights are converted to `real` (cells,
        offsets and tags are shared as copies)."""
        cl = lambda xs: [None if x is None else x.clone() for x in xs]
        phi, pr, pi = self._extras(lambda x: x.clone())
        return SpeciesArrays(cl(self.i), cl(self.dx), cl(self.i_prev), cl(self.dx_prev),
                             [x.to(real) for x in self.u], self.w.to(real), self.tag.clone(),
                             self.mass, self.charge, self.pusher, self.npart, self.index,
                             None if phi is None else phi.to(real),
                             None if pr is None else pr.to(real), pi)

    def clone(self):
        cl = lambda xs: [None if x is None else x.clone() for x in xs]
        return SpeciesArrays(cl(self.i), cl(self.dx), cl(self.i_prev), cl(self.dx_prev),
                             cl(self.u), self.w.clone(), self.tag.clone(), self.mass,
                             self.charge, self.pusher, self.npart, self.index,
                             *self._extras(lambda x: x.clone(memory_format=torch.preserve_format)))


def empty_species(g: GridSpec, capacity: int, *, mass=1.0, charge=-1.0, pusher=1, index=1,
                  device="cuda") -> SpeciesArrays:
    """A species with room for `capacity` particles and none alive yet (the
    arrays an injector appends to)."""
    z = lambda dt: torch.zeros(capacity, dtype=dt, device=device)
    return SpeciesArrays([z(torch.int32) for _ in range(3)], [z(torch.float32) for _ in range(3)],
                         [z(torch.int32) for _ in range(3)], [z(torch.float32) for _ in range(3)],
                         [z(g.real) for _ in range(3)], z(g.real), z(torch.int16), mass, charge,
                         pusher, 0, index)


def inject_params(number_density, ppc0, box, temperature, drift=((0, 0, 0), (0, 0, 0)), seed=1,
                  first_pair=0):
    """pic_inject_params: box = ((lo, hi), ...) in cells per simulated axis,
    temperature = (T1, T2) in m0 c^2, drift = two four-velocity 3-vectors."""
    from .abi import PicInjectParams
    p = PicInjectParams()
    p.number_density, p.ppc0 = number_density, ppc0
    for d, (lo, hi) in enumerate(box):
        p.xi_min[d], p.xi_max[d] = lo, hi
    for s in range(2):
        p.temperature[s] = temperature[s]
        for c in range(3):
            p.drift[s][c] = drift[s][c]
    p.seed, p.first_pair = seed, first_pair
    return p


def _uniform(shape, gen, device, dtype=torch.float64):
    return torch.rand(shape, generator=gen, device=device, dtype=dtype)


def juttner_synge(npart, temp, gen, device):
    """Momenta (u1, u2, u3) of a Maxwell-Juttner plasma at temperature `temp`
    (units of m c^2), following energy_dist.h:79-137."""
    if temp <= 0.0:
        z = torch.zeros(npart, dtype=torch.float64, device=device)
        return [z, z.clone(), z.clone()]
    if temp < 0.5:
        out = []
        for _ in range(3):
            x1 = _uniform(npart, gen, device).clamp_min(1e-300)
            x1 = torch.sqrt(-2.0 * torch.log(x1))
            x2 = 2.0 * math.pi * _uniform(npart, gen, device)
            out.append(x1 * torch.cos(x2) * math.sqrt(temp))
        return out
    # Sobol rejection: draw until eta^2 > u^2 + 1, vectorised over rejects
    u = torch.empty(npart, dtype=torch.float64, device=device)
    todo = torch.arange(npart, device=device)
    while todo.numel() > 0:
        m = todo.numel()
        x1 = (_uniform(m, gen, device) * _uniform(m, gen, device) *
              _uniform(m, gen, device)).clamp_min(1e-300)
        x2 = _uniform(m, gen, device).clamp_min(1e-300)
        uu = -temp * torch.log(x1)
        eta = -temp * torch.log(x1 * x2)
        ok = eta * eta > uu * uu + 1.0
        u[todo[ok]] = uu[ok]
        todo = todo[~ok]
    r1 = _uniform(npart, gen, device)
    r2 = _uniform(npart, gen, device)
    v0 = u * (2.0 * r1 - 1.0)
    v2 = 2.0 * u * torch.sqrt(r1 * (1.0 - r1))
    v1 = v2 * torch.cos(2.0 * math.pi * r2)
    v2 = v2 * torch.sin(2.0 * math.pi * r2)
    return [v0, v1, v2]


def boost_x1(u, beta, gen, device):
    """Flipping-method boost of a symmetric distribution to 3-velocity `beta`
    along x1 (energy_dist.h:151-172, with the 4-velocity of the drift)."""
    if beta == 0.0:
        return u
    ub = beta / math.sqrt(1.0 - beta * beta)      # drift 4-velocity
    bb = ub / math.sqrt(1.0 + ub * ub)
    gamma = torch.sqrt(1.0 + u[0] ** 2 + u[1] ** 2 + u[2] ** 2)
    flip = (-bb * u[0]) > gamma * _uniform(u[0].shape[0], gen, device)
    u0 = torch.where(flip, -u[0], u[0])
    u0 = math.sqrt(1.0 + ub * ub) * (u0 + bb * gamma)
    return [u0, u[1], u[2]]


def make_species(g: GridSpec, ppc: int, temp: float, beta: float, seed: int, *, mass=1.0,
                 charge=-1.0, pusher=1, index=1, device="cpu", shuffle=True, weights=None,
                 with_prev=True, extra=0):
    """`ppc` particles in every cell with uniform offsets, Maxwell-Juttner
    momenta boosted by `beta` along x1, seeded. `extra` reserves maxnpart."""
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    ncell = g.ncells()
    npart = ncell * ppc
    cell = torch.arange(ncell, device=device, dtype=torch.int64).repeat_interleave(ppc)
    if shuffle:
        perm = torch.randperm(npart, generator=gen, device=device)
        cell = cell[perm]
    n1, n2 = g.n[0], g.n[1]
    if g.dim == 2:
        ic = [(cell // n2).to(torch.int32), (cell % n2).to(torch.int32)]
    else:
        n3 = g.n[2]
        ic = [(cell // (n2 * n3)).to(torch.int32), ((cell // n3) % n2).to(torch.int32),
              (cell % n3).to(torch.int32)]
    dxs = [torch.rand(npart, generator=gen, device=device, dtype=torch.float32)
           for _ in range(g.dim)]
    u = juttner_synge(npart, temp, gen, device)
    u = boost_x1(u, beta, gen, device)
    u = [x.to(g.real) for x in u]
    w = (torch.ones(npart, dtype=g.real, device=device) if weights is None
         else weights(ic, dxs).to(g.real))
    tot = npart + extra

    def pad(x, fill=0):
        if extra == 0:
            return x.contiguous()
        y = torch.full((tot,), fill, dtype=x.dtype, device=device)
        y[:npart] = x
        return y

    i = [pad(x) for x in ic]
    dx = [pad(x) for x in dxs]
    if g.dim == 2:
        i.append(torch.zeros(tot, dtype=torch.int32, device=device))
        dx.append(torch.zeros(tot, dtype=torch.float32, device=device))
    if with_prev:
        ip = [x.clone() for x in i]
        dp = [x.clone() for x in dx]
    else:
        ip, dp = [None] * 3, [None] * 3
    tag = pad(torch.ones(npart, dtype=torch.int16, device=device))
    return SpeciesArrays(i, dx, ip, dp, [pad(x) for x in u], pad(w), tag, mass, charge, pusher,
                         npart, index)


def turbulent_field(g: GridSpec, B0: float, dB_over_B0: float, nmodes: int, seed: int,
                    device="cpu"):
    """EB with B = B0 z + a sum of `nmodes` random-phase Fourier modes with
    |k| in 2 pi / L * {1, 2} and amplitudes perpendicular to k (divergence
    free in the continuum), evaluated at each component's Yee position; E = 0.
    Ghost cells hold the periodic images."""
    gen = torch.Generator(device="cpu")
    gen.manual_seed(seed)
    EB = empty_field(g, 6, device)
    N1, N2, N3 = g.ext
    ng = g.ng
    L = [g.n[0], g.n[1], g.n[2] if g.dim == 3 else 1]
    modes = []
    cand = []
    rng = range(-2, 3)
    for a in rng:
        for b in rng:
            for c in (rng if g.dim == 3 else [0]):
                k2 = a * a + b * b + c * c
                if 1 <= k2 <= 4 and (a, b, c) > (0, 0, 0):
                    cand.append((a, b, c))
    pick = torch.randperm(len(cand), generator=gen)[:nmodes].tolist()
    amp = dB_over_B0 * B0 / math.sqrt(max(nmodes, 1) / 2.0)
    for idx in pick:
        kv = torch.tensor(cand[idx], dtype=torch.float64)
        khat = kv / kv.norm()
        r = torch.randn(3, generator=gen, dtype=torch.float64)
        a_perp = r - (r @ khat) * khat
        a_perp = a_perp / a_perp.norm() * amp
        phase = float(torch.rand(1, generator=gen, dtype=torch.float64)) * 2.0 * math.pi
        modes.append((kv, a_perp, phase))
    # coordinates (cell units) of ghost-inclusive indices
    x1 = torch.arange(N1, dtype=torch.float64, device=device) - ng
    x2 = torch.arange(N2, dtype=torch.float64, device=device) - ng
    x3 = (torch.arange(N3, dtype=torch.float64, device=device) - ng) if g.dim == 3 else \
        torch.zeros(1, dtype=torch.float64, device=device)
    # staggering of bx1, bx2, bx3: half-cell shifts along the dual axes
    shifts = [(0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)]
    for comp in range(3):
        s = shifts[comp]
        X3, X2, X1 = torch.meshgrid(x3 + (s[2] if g.dim == 3 else 0.0), x2 + s[1], x1 + s[0],
                                    indexing="ij")
        val = torch.zeros_like(X1)
        for kv, a_perp, phase in modes:
            arg = (2.0 * math.pi * (kv[0] * X1 / L[0] + kv[1] * X2 / L[1] +
                                    (kv[2] * X3 / L[2] if g.dim == 3 else 0.0)) + phase)
            val = val + float(a_perp[comp]) * torch.cos(arg)
        if comp == 2:
            val = val + B0
        # contravariant components: physical / dx for the simulated axes
        scale = (1.0 / g.dx) if comp < g.dim else 1.0
        EB[3 + comp] = (val * scale).to(g.real)
    return EB
