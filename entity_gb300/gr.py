"""Python mirror of the reference's GR engine phases over the C ABI.

`GRContext` wraps a pic_ctx on a 2D (r, theta) grid together with the
QKerrSchild parameters (pic_gr_metric) and exposes the phase functions of
GRPICEngine::step_forward (src/engines/grpic/grpic.hpp:66-634) by their
reference names. `wald_setup` builds the Wald problem's grid, vertical seed
field and a pair plasma injected on the device (the reference's wald pgen
injects none).
Device memory is held in torch tensors; all computation runs in
libentity_pic.so.
"""
import ctypes as C
import math
from dataclasses import dataclass

import torch

from . import abi
from .inputs import GridSpec, SpeciesArrays, empty_field
from .sim import Context, _ptr, _stream_ptr, make_species, step_params


@dataclass
class GRSpec:
    a: float = 0.95
    r_min: float = 0.0      # 0: 0.9 r_horizon
    r_max: float = 50.0
    th_min: float = 0.0
    th_max: float = math.pi
    r0: float = 0.0
    h: float = 0.0
    axis_min: int = 1
    axis_max: int = 1
    horizon: int = 1

    @property
    def r_horizon(self):
        return 1.0 + math.sqrt(1.0 - self.a * self.a)

    def metric(self) -> abi.PicGRMetric:
        m = abi.PicGRMetric()
        m.a, m.r0, m.h = self.a, self.r0, self.h
        m.x1min = self.r_min if self.r_min > 0 else 0.9 * self.r_horizon
        m.x1max = self.r_max
        m.x2min, m.x2max = self.th_min, self.th_max
        m.axis_min, m.axis_max, m.horizon = self.axis_min, self.axis_max, self.horizon
        return m

    def x1_of_r(self, g: GridSpec, r):
        """Code coordinate of radius r (log-spaced grid, r0 = 0)."""
        m = self.metric()
        chi_min = math.log(m.x1min - self.r0)
        dchi = (math.log(m.x1max - self.r0) - chi_min) / g.n[0]
        return (math.log(r - self.r0) - chi_min) / dchi


def gr_grid(n1, n2, order=2, real=torch.float32):
    """(r, theta) grid with absorbing particles in r and axes in theta."""
    return GridSpec(dim=2, n=(n1, n2, 1), order=order, real=real, periodic=(0, 0, 0),
                    prtl_bc=((1, 1), (3, 3), (0, 0)))


class GRContext(Context):
    def __init__(self, g: GridSpec, spec: GRSpec):
        super().__init__(g)
        self.spec = spec
        self.m = spec.metric()
        self.match = None

    def metric_eval(self, x, stream=None):
        x = torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()
        out = torch.empty((x.shape[0], 24), dtype=torch.float64, device="cuda")
        abi.call("pic_gr_metric_eval", self.h, C.byref(self.m), _ptr(x), x.shape[0], _ptr(out),
                 _stream_ptr(stream))
        return out

    def gr_push(self, sp: SpeciesArrays, em, em0, dt, omegaB0, niter=10, island=(0, 0),
                stream=None):
        """island = (lo, hi): particles with lo <= i1 < hi push in FP64."""
        ps = make_species(sp, 2)
        abi.call("pic_gr_push", self.h, C.byref(self.m), C.byref(ps), _ptr(em), _ptr(em0), dt,
                 omegaB0, niter, island[0], island[1], _stream_ptr(stream))

    def gr_particle_push(self, species, em, em0, dt, omegaB0, niter=10, island=(0, 0),
                         stream=None):
        """grpic::ParticlePush: every species, islands run concurrently."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, 2) for s in species])
        abi.call("pic_gr_particle_push", self.h, C.byref(self.m), arr, len(species), _ptr(em),
                 _ptr(em0), dt, omegaB0, niter, island[0], island[1], _stream_ptr(stream))

    def gr_deposit(self, species, J, dt, island=(0, 0), zero=True, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, 2) for s in species])
        abi.call("pic_gr_deposit", self.h, C.byref(self.m), arr, len(species), _ptr(J), dt,
                 island[0], island[1], 0 if zero else abi.PIC_PD_NO_ZERO, _stream_ptr(stream))

    def gr_faraday(self, Bin, Bout, E, coeff, stream=None):
        abi.call("pic_gr_faraday", self.h, C.byref(self.m), _ptr(Bin), _ptr(Bout), _ptr(E), coeff,
                 _stream_ptr(stream))

    def gr_ampere(self, Din, Dout, H, coeff, stream=None):
        abi.call("pic_gr_ampere", self.h, C.byref(self.m), _ptr(Din), _ptr(Dout), _ptr(H), coeff,
                 _stream_ptr(stream))

    def gr_currents_ampere(self, D, J, coeff, stream=None):
        abi.call("pic_gr_currents_ampere", self.h, C.byref(self.m), _ptr(D), _ptr(J), coeff,
                 _stream_ptr(stream))

    def gr_aux(self, which, D, B, out, stream=None):
        abi.call("pic_gr_aux", self.h, C.byref(self.m), which, _ptr(D), _ptr(B), _ptr(out),
                 _stream_ptr(stream))

    def gr_average(self, which, a, b, stream=None):
        abi.call("pic_gr_average", self.h, which, _ptr(a), _ptr(b), _stream_ptr(stream))

    def gr_filter_currents(self, J, buff, npasses, stream=None):
        abi.call("pic_gr_filter_currents", self.h, C.byref(self.m), _ptr(J), _ptr(buff),
                 int(npasses), _stream_ptr(stream))

    def gr_field_bcs(self, fld, set_e, set_b, nfilter=0, stream=None):
        abi.call("pic_gr_field_bcs", self.h, C.byref(self.m), _ptr(fld), int(set_e), int(set_b),
                 nfilter, _stream_ptr(stream))

    def gr_init_vertical(self, EB, stream=None):
        abi.call("pic_gr_init_vertical", self.h, C.byref(self.m), _ptr(EB), _stream_ptr(stream))

    def gr_inject_uniform_maxwellians(self, sp1: SpeciesArrays, sp2: SpeciesArrays, params, V0,
                                      stream=None):
        """pic_gr_inject_uniform_maxwellians: covariant velocities, weight
        sqrt(det h) / V0; returns the number of pairs."""
        p1, p2 = make_species(sp1, 2), make_species(sp2, 2)
        n = C.c_int64(0)
        abi.call("pic_gr_inject_uniform_maxwellians", self.h, C.byref(self.m), C.byref(p1),
                 C.byref(p2), C.byref(params), V0, C.byref(n), _stream_ptr(stream))
        sp1.npart, sp2.npart = p1.npart, p2.npart
        return n.value

    def gr_min_cell_size(self, stream=None):
        out = C.c_double(0)
        abi.call("pic_gr_min_cell_size", self.h, C.byref(self.m), C.byref(out),
                 _stream_ptr(stream))
        return out.value

    def gr_match_fields(self, fld, target, ds, set_e=True, set_b=True, stream=None):
        abi.call("pic_gr_match_fields", self.h, C.byref(self.m), _ptr(fld), _ptr(target), ds,
                 int(set_e), int(set_b), _stream_ptr(stream))

    def gr_absorb_currents(self, J, ds, stream=None):
        abi.call("pic_gr_absorb_currents", self.h, C.byref(self.m), _ptr(J), ds,
                 _stream_ptr(stream))

    def grpic_step(self, species, fields, prm, niter=10, island=(0, 0), step=0, match=None,
                   stream=None):
        """fields: list [em, em0, aux, cur, cur0, buff]; swapped in place like
        the reference's views. match = (ds, target field) enables the MATCH
        boundary at r max."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, 2) for s in species])
        ptrs = (C.c_void_p * 6)(*[t.data_ptr() for t in fields])
        gp = abi.PicGRParams()
        gp.niter, gp.island_lo, gp.island_hi = niter, island[0], island[1]
        if match is not None:
            gp.match_ds, gp.match_target = float(match[0]), match[1].data_ptr()
        abi.call("pic_grpic_step", self.h, C.byref(self.m), arr, len(species), ptrs,
                 C.byref(prm), C.byref(gp), step, _stream_ptr(stream))
        by_ptr = {t.data_ptr(): t for t in fields}
        fields[:] = [by_ptr[ptrs[k]] for k in range(6)]
        for k, s in enumerate(species):
            s.npart = arr[k].npart


def horizon_island(g: GridSpec, spec: GRSpec, cells=3):
    """The FP64 island (lo, hi): the horizon's cell and `cells` cells on
    either side of it, i1 in [lo, hi)."""
    ih = int(math.floor(spec.x1_of_r(g, spec.r_horizon)))
    return max(0, ih - cells), max(0, ih + 1 + cells)


def gr_step_params(ctx: GRContext, *, cfl, ppc0, skindepth0, larmor0, sort_interval=0,
                   clear_interval=100, deposit=True):
    """Scales of the GR engine (parameters.cpp:47-78, grid.cpp:39-51):
    dt = CFL * dxMin (qkerr_schild.h:112-129), V0 = sqrt(det h) at the first
    cell centre, q0 = V0 / (ppc0 skindepth0^2), B0 = omegaB0 = 1 / larmor0."""
    g = ctx.g
    R = g.real
    t = lambda v: torch.tensor(v, dtype=R)
    dxmin = t(ctx.gr_min_cell_size())
    p = step_params(g, cfl=cfl, ppc0=ppc0, skindepth0=skindepth0, larmor0=larmor0, nfilter=0,
                    sort_interval=sort_interval, clear_interval=clear_interval,
                    write_prev=True, deposit=deposit)
    V0 = t(float(ctx.metric_eval([[0.5, 0.5]])[0, 10]))
    p.dt = float(t(cfl) * dxmin)
    p.V0 = float(V0)
    p.q0 = float(V0 / (t(ppc0) * (t(skindepth0) * t(skindepth0))))
    return p


def inject_pairs(g: GridSpec, spec: GRSpec, ppc: int, r_inject: float, seed: int,
                 device="cuda"):
    """e-/e+ at rest (u_i = 0), `ppc` per cell in r < r_inject, uniform
    offsets; the two species share positions."""
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    n1 = min(g.n[0], int(math.ceil(spec.x1_of_r(g, r_inject))))
    n2 = g.n[1]
    ncell = n1 * n2
    cell = torch.arange(ncell, device=device, dtype=torch.int64).repeat_interleave(ppc)
    npart = ncell * ppc
    i1 = (cell // n2).to(torch.int32)
    i2 = (cell % n2).to(torch.int32)
    dx1 = torch.rand(npart, generator=gen, device=device, dtype=torch.float32)
    dx2 = torch.rand(npart, generator=gen, device=device, dtype=torch.float32)
    z = lambda dt: torch.zeros(npart, dtype=dt, device=device)
    out = []
    for k, q in enumerate((-1.0, 1.0)):
        out.append(SpeciesArrays([i1.clone(), i2.clone(), z(torch.int32)],
                                 [dx1.clone(), dx2.clone(), z(torch.float32)],
                                 [i1.clone(), i2.clone(), z(torch.int32)],
                                 [dx1.clone(), dx2.clone(), z(torch.float32)],
                                 [z(g.real), z(g.real), z(g.real)],
                                 torch.ones(npart, dtype=g.real, device=device),
                                 torch.ones(npart, dtype=torch.int16, device=device),
                                 1.0, q, 1, npart, k + 1))
    return out


def wald_setup(n=(1024, 512), a=0.95, r_max=50.0, order=2, ppc=4, r_inject=6.0,
               real=torch.float32, seed=5):
    """The Wald problem: QKerrSchild a, r in [0.9 r_h, r_max], theta in
    [0, pi], vertical seed field, and e-/e+ pairs at rest injected on the
    device by pic_gr_inject_uniform_maxwellians: `ppc` pairs per cell on
    average, uniform in code coordinates over r < r_inject, weights
    sqrt(det h) / V0 (the reference's GR injection weights), V0 = sqrt(det h)
    at the first cell centre; then one cell sort of each species. ctx.match
    holds the MATCH boundary's (ds, target field) for grpic_step."""
    from .inputs import empty_species, inject_params
    g = gr_grid(n[0], n[1], order=order, real=real)
    spec = GRSpec(a=a, r_max=r_max)
    ctx = GRContext(g, spec)
    em = empty_field(g, 6, "cuda")
    ctx.gr_init_vertical(em)
    fields = [em, torch.zeros_like(em), torch.zeros_like(em), empty_field(g, 3, "cuda"),
              empty_field(g, 3, "cuda"), empty_field(g, 3, "cuda")]
    # MATCH at r max toward the seed field, ds = 1 % of the radial extent
    # (grid.boundaries.match.ds's default, parameters/grid.cpp:295-305)
    m = spec.metric()
    ctx.match = (0.01 * (m.x1max - m.x1min), em.clone())
    x1_inj = min(float(g.n[0]), spec.x1_of_r(g, r_inject))
    cap = int(math.ceil(ppc * x1_inj * g.n[1])) + 1
    species = [empty_species(g, cap, charge=q, index=k + 1) for k, q in enumerate((-1.0, 1.0))]
    V0 = float(ctx.metric_eval([[0.5, 0.5]])[0, 10])
    # pairs = ppc0 * density / 2 per cell (ComputeNumInject) with ppc0 = 1
    prm = inject_params(2.0 * ppc, 1.0, ((0.0, x1_inj), (0.0, float(g.n[1]))), (0.0, 0.0),
                        seed=seed)
    ctx.gr_inject_uniform_maxwellians(species[0], species[1], prm, V0)
    # the injector places pairs in random order: one cell sort, as the
    # reference's SortParticles would at step 0 with spatial sorting on
    for sp in species:
        ctx.sort(sp, abi.PIC_SORT_SPATIAL | abi.PIC_SORT_SKIP_PREV)
    return g, spec, ctx, fields, species
