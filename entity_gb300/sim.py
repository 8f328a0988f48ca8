"""Python mirror of the reference's SR phase functions, driving the C ABI.

Each function has the reference's name and argument meaning
(srpic::Faraday, srpic::Ampere, srpic::CurrentsAmpere, srpic::ParticlePush,
srpic::CurrentsDeposit, srpic::CurrentsFilter, Metadomain::SynchronizeFields,
Metadomain::CommunicateFields, Metadomain::SortParticles; see
include/entity_pic.h for the file:line of each) and raises PicError where the
reference raises. Device memory is held in torch tensors; torch is only the
allocator here, every computation runs in libentity_pic.so.
"""
import ctypes as C

import numpy as np
import torch

from . import abi
from .inputs import GridSpec, SpeciesArrays


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(stream.cuda_stream)


class SpeciesAdjoint:
    """Adjoint arrays of one species (pic_species_adjoint): gradients with
    respect to positions (per simulated axis), momenta and weights."""

    def __init__(self, g: GridSpec, npart: int, device="cuda"):
        z = lambda: torch.zeros(max(npart, 1), dtype=g.real, device=device)
        self.lx = [z() for _ in range(g.dim)]
        self.lu = [z() for _ in range(3)]
        self.lw = z()

    def c(self) -> abi.PicSpeciesAdjoint:
        a = abi.PicSpeciesAdjoint()
        a.lx1, a.lx2 = self.lx[0].data_ptr(), self.lx[1].data_ptr()
        a.lx3 = self.lx[2].data_ptr() if len(self.lx) > 2 else None
        a.lu1, a.lu2, a.lu3 = (t.data_ptr() for t in self.lu)
        a.lw = self.lw.data_ptr()
        return a


def make_grid(g: GridSpec) -> abi.PicGrid:
    pg = abi.PicGrid()
    pg.dim = g.dim
    for d in range(3):
        pg.n[d] = g.n[d] if d < g.dim else 1
        pg.fld_periodic[d] = int(g.periodic[d]) if d < g.dim else 0
        pg.prtl_bc[d][0] = g.prtl_bc[d][0]
        pg.prtl_bc[d][1] = g.prtl_bc[d][1]
    pg.ng = g.ng
    pg.order = g.order
    pg.real_bytes = g.real_bytes
    s = g.strides()
    for k in range(4):
        pg.em_stride[k] = s[k]
        pg.cur_stride[k] = s[k]
    return pg


def make_species(sp: SpeciesArrays, dim: int) -> abi.PicSpecies:
    ps = abi.PicSpecies()
    ps.i1, ps.i2 = _ptr(sp.i[0]), _ptr(sp.i[1])
    ps.dx1, ps.dx2 = _ptr(sp.dx[0]), _ptr(sp.dx[1])
    ps.i1_prev, ps.i2_prev = _ptr(sp.i_prev[0]), _ptr(sp.i_prev[1])
    ps.dx1_prev, ps.dx2_prev = _ptr(sp.dx_prev[0]), _ptr(sp.dx_prev[1])
    if dim == 3:
        ps.i3, ps.dx3 = _ptr(sp.i[2]), _ptr(sp.dx[2])
        ps.i3_prev, ps.dx3_prev = _ptr(sp.i_prev[2]), _ptr(sp.dx_prev[2])
    ps.ux1, ps.ux2, ps.ux3 = _ptr(sp.u[0]), _ptr(sp.u[1]), _ptr(sp.u[2])
    ps.weight = _ptr(sp.w)
    ps.tag = _ptr(sp.tag)
    ps.npart = sp.npart
    ps.maxnpart = sp.tag.numel()
    ps.mass = sp.mass
    ps.charge = sp.charge
    ps.pusher = sp.pusher
    ps.index = sp.index
    if getattr(sp, "phi", None) is not None:
        ps.phi = _ptr(sp.phi)
    for name in ("pld_r", "pld_i"):
        t = getattr(sp, name, None)
        if t is not None and t.numel() > 0:
            if name == "pld_i" and t.element_size() != 4:
                raise ValueError("pld_i holds 32-bit integers (npart_t)")
            setattr(ps, name, _ptr(t))
            st = getattr(ps, name + "_stride")
            st[0], st[1] = t.stride(0), t.stride(1)
            setattr(ps, "n" + name, t.shape[1])
    return ps


class HostPipe:
    """pic_host_pipe: the copy streams of a domain whose state lives in pinned
    host memory (Context.step_host)."""

    def __init__(self):
        h = C.c_void_p()
        abi.call("pic_host_pipe_create", C.byref(h))
        self.h = h

    def sync(self):
        abi.call("pic_host_pipe_sync", self.h)

    def set_groups(self, max_groups, min_group_bytes):
        """pic_host_pipe_set_groups: how binned species are cut into groups."""
        abi.call("pic_host_pipe_set_groups", self.h, int(max_groups), int(min_group_bytes))

    def bytes(self):
        """(host-to-device, device-to-host) bytes of the last step."""
        a, b = C.c_int64(0), C.c_int64(0)
        abi.call("pic_host_pipe_bytes", self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def close(self):
        if self.h:
            abi.call("pic_host_pipe_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One domain's context (pic_create / pic_destroy)."""

    def __init__(self, g: GridSpec):
        self.g = g
        self.grid = make_grid(g)
        h = C.c_void_p()
        abi.call("pic_create", C.byref(self.grid), C.byref(h))
        self.h = h

    def close(self):
        if self.h:
            abi.call("pic_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tile_shape(self):
        out = (C.c_int32 * 3)()
        abi.call("pic_tile_shape", self.h, out)
        return tuple(out)

    # --- field solvers -----------------------------------------------------
    def faraday(self, EB, coeff1, coeff2, stencil=None, stream=None):
        st = None if stencil is None else (C.c_double * 9)(*stencil)
        abi.call("pic_faraday", self.h, _ptr(EB), coeff1, coeff2, st, _stream_ptr(stream))

    def ampere(self, EB, coeff1, coeff2, stream=None):
        abi.call("pic_ampere", self.h, _ptr(EB), coeff1, coeff2, _stream_ptr(stream))

    def currents_ampere(self, EB, J, coeff, ppc0, stream=None):
        abi.call("pic_currents_ampere", self.h, _ptr(EB), _ptr(J), coeff, ppc0,
                 _stream_ptr(stream))

    def ampere_currents(self, EB, J, coeff1, coeff2, jcoeff, ppc0, stream=None):
        abi.call("pic_ampere_currents", self.h, _ptr(EB), _ptr(J), coeff1, coeff2, jcoeff, ppc0,
                 _stream_ptr(stream))

    # --- particles ---------------------------------------------------------
    def push(self, sp: SpeciesArrays, EB, dt, omegaB0, dx, stream=None):
        ps = make_species(sp, self.g.dim)
        abi.call("pic_push", self.h, C.byref(ps), _ptr(EB), dt, omegaB0, dx, _stream_ptr(stream))

    def deposit(self, species, J, dt, dx, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_deposit", self.h, arr, len(species), _ptr(J), dt, dx, _stream_ptr(stream))

    def push_deposit(self, species, EB, J, dt, omegaB0, dx, flags=0, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_push_deposit", self.h, arr, len(species), _ptr(EB), _ptr(J), dt, omegaB0,
                 dx, flags, _stream_ptr(stream))

    def sort(self, sp: SpeciesArrays, flags, stream=None):
        ps = make_species(sp, self.g.dim)
        n = C.c_int64(0)
        st = abi.load().pic_sort(self.h, C.byref(ps), flags, C.byref(n), _stream_ptr(stream))
        if st not in (abi.PIC_OK, abi.PIC_ERR_DEVICE):
            abi.check("pic_sort", st)
        sp.npart = n.value
        return st

    # --- currents ------------------------------------------------------------
    def sync_currents(self, J, buff=None, stream=None):
        abi.call("pic_sync_currents", self.h, _ptr(J), _ptr(buff), _stream_ptr(stream))

    def filter_currents(self, J, buff, npasses, stream=None):
        abi.call("pic_filter_currents", self.h, _ptr(J), _ptr(buff), npasses, _stream_ptr(stream))

    def fill_ghosts(self, fld, is_em, c0, c1, stream=None):
        abi.call("pic_fill_ghosts", self.h, _ptr(fld), int(is_em), c0, c1, _stream_ptr(stream))

    # --- diagnostics ---------------------------------------------------------
    def field_energy(self, EB, dx, stream=None):
        out = (C.c_double * 2)()
        abi.call("pic_field_energy", self.h, _ptr(EB), dx, out, _stream_ptr(stream))
        return out[0], out[1]

    def particle_moments(self, species, stream=None):
        """FP64 sums (m gamma, u1, u2, u3, w m (gamma - 1), w) over alive particles."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        out = (C.c_double * 6)()
        abi.call("pic_particle_moments", self.h, arr, len(species), out, _stream_ptr(stream))
        return list(out)

    def charge_density(self, species, rho, stream=None):
        """Adds the deposit-consistent node charge density to rho[0] (J layout)."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_charge_density", self.h, arr, len(species), _ptr(rho), _stream_ptr(stream))

    def set_field_bcs(self, kinds, x_min=(0.0, 0.0, 0.0), dx=1.0, match_ds=None, target=None):
        """pic_set_field_bcs: kinds = ((min, max), ...) per axis of
        abi.PIC_FBC_*; MATCH sides need match_ds ((min, max), ...) and the
        target field (kept alive by the caller)."""
        b = abi.PicFieldBCs()
        for d in range(3):
            for h in range(2):
                b.kind[d][h] = kinds[d][h] if d < len(kinds) else abi.PIC_FBC_PERIODIC
                if match_ds is not None and d < len(match_ds):
                    b.match_ds[d][h] = match_ds[d][h]
            b.x_min[d] = x_min[d] if d < len(x_min) else 0.0
        b.dx = dx
        b.match_target = target.data_ptr() if target is not None else None
        self._fbc_target = target
        abi.call("pic_set_field_bcs", self.h, C.byref(b))

    def field_boundaries(self, EB, set_e, set_b, stream=None):
        abi.call("pic_field_boundaries", self.h, _ptr(EB), int(set_e), int(set_b),
                 _stream_ptr(stream))

    def inject_uniform_maxwellians(self, sp1: SpeciesArrays, sp2: SpeciesArrays, params,
                                   stream=None):
        """pic_inject_uniform_maxwellians: appends the pairs to both species
        (npart advances); returns the number of pairs."""
        p1, p2 = make_species(sp1, self.g.dim), make_species(sp2, self.g.dim)
        n = C.c_int64(0)
        abi.call("pic_inject_uniform_maxwellians", self.h, C.byref(p1), C.byref(p2),
                 C.byref(params), C.byref(n), _stream_ptr(stream))
        sp1.npart, sp2.npart = p1.npart, p2.npart
        return n.value

    def output_moment(self, species, params, bckp, comp, stream=None):
        """pic_output_moment: adds the moment of `params` (abi.PicMomentParams)
        of the species into bckp[comp] (EB layout)."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_output_moment", self.h, arr, len(species), C.byref(params), _ptr(bckp),
                 int(comp), _stream_ptr(stream))

    def sync_moments(self, bckp, c0, c1, stream=None):
        abi.call("pic_sync_moments", self.h, _ptr(bckp), int(c0), int(c1), _stream_ptr(stream))

    def normalize_by_rho(self, bckp, c_rho, cv, stream=None):
        abi.call("pic_normalize_by_rho", self.h, _ptr(bckp), int(c_rho), int(cv[0]), int(cv[1]),
                 int(cv[2]), _stream_ptr(stream))

    def output_divergence(self, EB, bckp, comp, stream=None):
        abi.call("pic_output_divergence", self.h, _ptr(EB), _ptr(bckp), int(comp),
                 _stream_ptr(stream))

    def output_field(self, src, is_em, c0, ncomp, flags, dx, dwn, out, stream=None):
        """pic_output_field into `out`, a device tensor of
        ncomp x ceil(n3/d3) x ceil(n2/d2) x ceil(n1/d1) (2D: no n3 axis)."""
        d = (C.c_int32 * 3)(*[int(x) for x in (list(dwn) + [1, 1, 1])[:3]])
        abi.call("pic_output_field", self.h, _ptr(src), int(is_em), int(c0), int(ncomp),
                 int(flags), float(dx), d, _ptr(out), _stream_ptr(stream))

    def output_particles(self, sp: SpeciesArrays, stride, dx, xmin, x, u, w, stream=None):
        """pic_output_particles: writes npart // stride records into the
        device tensors x (dim of them), u (3) and w; returns the count."""
        ps = make_species(sp, self.g.dim)
        xm = (C.c_double * 3)(*[float(v) for v in (list(xmin) + [0.0, 0.0, 0.0])[:3]])
        xp = (C.c_void_p * 3)(*[(_ptr(x[d]) if d < len(x) else None) for d in range(3)])
        up = (C.c_void_p * 3)(*[_ptr(t) for t in u])
        n = C.c_int64(0)
        abi.call("pic_output_particles", self.h, C.byref(ps), int(stride), float(dx), xm, xp, up,
                 _ptr(w), C.byref(n), _stream_ptr(stream))
        return n.value

    def device_errors(self, reset=False, stream=None):
        out = (C.c_int64 * 4)()
        abi.call("pic_get_device_errors", self.h, out, int(reset), _stream_ptr(stream))
        return list(out)

    def wait_timeouts(self, reset=False, stream=None):
        """Kernel waits that ran out of their iteration limit (0 normally)."""
        out = C.c_int64(0)
        abi.call("pic_get_wait_timeouts", self.h, C.byref(out), int(reset), _stream_ptr(stream))
        return out.value

    # --- adjoint ----------------------------------------------------------------
    def gradient(self, species, adjoints, EB, J, buff, prm: abi.PicStepParams, nsteps,
                 checkpoint_every, lamEB, stream=None):
        """Gradient of the final E-field energy after nsteps with respect to the
        initial state (pic_srpic_gradient); returns the energy. `adjoints` is
        one SpeciesAdjoint per species; species and EB end at the initial state."""
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        adj = (abi.PicSpeciesAdjoint * len(adjoints))(*[a.c() for a in adjoints])
        loss = C.c_double(0)
        abi.call("pic_srpic_gradient", self.h, arr, adj, len(species), _ptr(EB), _ptr(J),
                 _ptr(buff), C.byref(prm), nsteps, checkpoint_every, _ptr(lamEB),
                 C.byref(loss), _stream_ptr(stream))
        for k, s in enumerate(species):
            s.npart = arr[k].npart
        return loss.value

    def step_host(self, pipe: HostPipe, host_species, dev_species, hEB, dEB, hJ, dJ, buff,
                  prm: abi.PicStepParams, step, stream=None):
        """pic_srpic_step_host: host_species / hEB / hJ are pinned CPU tensors,
        dev_species / dEB / dJ their device mirrors. Asynchronous: the host
        arrays hold the result after pipe.sync()."""
        hs = (abi.PicSpecies * len(host_species))(
            *[make_species(s, self.g.dim) for s in host_species])
        ds = (abi.PicSpecies * len(dev_species))(
            *[make_species(s, self.g.dim) for s in dev_species])
        abi.call("pic_srpic_step_host", self.h, pipe.h, hs, ds, len(dev_species), _ptr(hEB),
                 _ptr(dEB), _ptr(hJ), _ptr(dJ), _ptr(buff), C.byref(prm), int(step),
                 _stream_ptr(stream))
        for k in range(len(dev_species)):
            host_species[k].npart = hs[k].npart
            dev_species[k].npart = ds[k].npart

    def step_adjoint(self, species, adjoints, EB, lamEB, prm: abi.PicStepParams, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        adj = (abi.PicSpeciesAdjoint * len(adjoints))(*[a.c() for a in adjoints])
        abi.call("pic_srpic_step_adjoint", self.h, arr, adj, len(species), _ptr(EB), _ptr(lamEB),
                 C.byref(prm), _stream_ptr(stream))

    def energy_adjoint_seed(self, EB, lamEB, dx, stream=None):
        abi.call("pic_field_energy_adjoint_seed", self.h, _ptr(EB), _ptr(lamEB), dx,
                 _stream_ptr(stream))

    def checkpoint_save(self, slot, species, EB, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_checkpoint_save", self.h, slot, arr, len(species), _ptr(EB),
                 _stream_ptr(stream))

    def checkpoint_restore(self, slot, species, EB, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_checkpoint_restore", self.h, slot, arr, len(species), _ptr(EB),
                 _stream_ptr(stream))
        for k, s in enumerate(species):
            s.npart = arr[k].npart

    # --- phase timers ---------------------------------------------------------
    def timers(self, on=True):
        abi.call("pic_timers_enable", self.h, int(on))
        abi.call("pic_timers_reset", self.h)

    def read_timers(self):
        ms = (C.c_double * 6)()
        cnt = (C.c_int64 * 6)()
        abi.call("pic_timers_read", self.h, ms, cnt)
        return {name: (ms[k], cnt[k]) for k, name in enumerate(abi.PIC_PHASES)}

    def step(self, species, EB, J, buff, prm: abi.PicStepParams, step, stream=None):
        arr = (abi.PicSpecies * len(species))(*[make_species(s, self.g.dim) for s in species])
        abi.call("pic_srpic_step", self.h, arr, len(species), _ptr(EB), _ptr(J), _ptr(buff),
                 C.byref(prm), step, _stream_ptr(stream))
        for k, s in enumerate(species):
            s.npart = arr[k].npart


def step_params(g: GridSpec, *, cfl, ppc0, skindepth0, larmor0, nfilter=0, sort_interval=0,
                clear_interval=100, correction=1.0, write_prev=False, fieldsolver=True,
                deposit=True, sort_tiled=False):
    """Scales of SimulationParams (src/framework/parameters/parameters.cpp:47-78,
    algorithms.cpp:18-27, minkowski.h:82-84) in real_t arithmetic: numpy
    scalars of the real type, whose square root rounds correctly (torch's CPU
    sqrt of a float64 scalar can be one ulp off)."""
    R = np.float32 if g.real == torch.float32 else np.float64
    t = lambda v: R(v)
    dx = t(g.dx)
    dxmin = dx / np.sqrt(t(float(g.dim)))
    dt = t(cfl) * dxmin
    # V0 = sqrt_det_h (minkowski.h:144-152): SQR(dx) in 2D, CUBE(dx) in 3D
    V0 = dx * dx if g.dim == 2 else dx * dx * dx
    q0 = V0 / (t(ppc0) * (t(skindepth0) * t(skindepth0)))
    B0 = t(1.0) / t(larmor0)
    p = abi.PicStepParams()
    p.dt, p.dx, p.omegaB0 = float(dt), float(dx), float(B0)
    p.correction = float(t(correction))
    p.q0, p.B0, p.V0, p.ppc0 = float(q0), float(B0), float(V0), float(t(ppc0))
    p.nfilter, p.sort_interval, p.clear_interval = nfilter, sort_interval, clear_interval
    p.fieldsolver_enabled, p.deposit_enabled = int(fieldsolver), int(deposit)
    p.write_prev = int(write_prev)
    p.sort_tiled = int(sort_tiled)
    return p
