"""ctypes binding of oracle/_ref: Entity's own SR kernels compiled from the
reference sources against the host Kokkos shim (TEST INFRASTRUCTURE ONLY).

RefOracle has the Oracle's interface for the kernels the reference build
provides (push, deposit, Faraday, Ampere, CurrentsAmpere, one filter pass,
the field exchange through comm::CommunicateField, the sort key), so
Oracle.step runs the reference's kernels in the reference's step order.
"""
import ctypes as C

import torch

from . import build_ref
from .oracle import GR_NAMES, GR_NQ, GROracle, Oracle, OrcGrid, OrcSpecies, _p

_libs = {}


def available():
    return build_ref.reference_root() is not None


def lib(real, order):
    tag = "f32" if real == torch.float32 else "f64"
    key = (tag, order)
    if key not in _libs:
        paths = build_ref.build()
        if key not in paths:
            raise RuntimeError("the reference checkout is not available")
        L = C.CDLL(paths[key])
        G = C.POINTER(OrcGrid)
        S = C.POINTER(OrcSpecies)
        V = C.c_void_p
        D = C.c_double
        for f in ("ref_shape_order", "ref_n_ghosts", "ref_real_size"):
            getattr(L, f).restype = C.c_int
        L.ref_push.restype = C.c_int
        L.ref_push.argtypes = [G, S, V, D, D, D]
        L.ref_deposit.restype = C.c_int
        L.ref_deposit.argtypes = [G, S, V, D, D]
        L.ref_faraday.restype = C.c_int
        L.ref_faraday.argtypes = [G, V, D, D, C.POINTER(D)]
        L.ref_ampere.restype = C.c_int
        L.ref_ampere.argtypes = [G, V, D, D]
        L.ref_currents_ampere.restype = C.c_int
        L.ref_currents_ampere.argtypes = [G, V, V, D, D]
        L.ref_filter_pass.restype = C.c_int
        L.ref_filter_pass.argtypes = [G, V, V]
        L.ref_filter_pass_axisym.restype = C.c_int
        L.ref_filter_pass_axisym.argtypes = [G, V, V, C.c_int, C.c_int]
        PD = C.POINTER(C.c_double)
        PI = C.POINTER(C.c_int)
        L.ref_gr_metric.restype = C.c_int
        L.ref_gr_metric.argtypes = [C.c_int, C.c_int, PD, V, C.c_int64, V]
        L.ref_gr_push.restype = C.c_int
        L.ref_gr_push.argtypes = [G, PD, S, V, V, D, D, C.c_int, PI, PI]
        L.ref_gr_convert_x2.restype = C.c_int
        L.ref_gr_convert_x2.argtypes = [C.c_int, C.c_int, PD, C.c_int, V, C.c_int64, V]
        L.ref_gr_field.restype = C.c_int
        L.ref_gr_field.argtypes = [G, PD, C.c_int, V, V, V, D, C.c_int, C.c_int]
        L.ref_gr_field_bcs.restype = C.c_int
        L.ref_gr_field_bcs.argtypes = [G, V] + [C.c_int] * 6
        L.ref_gr_deposit.restype = C.c_int
        L.ref_gr_deposit.argtypes = [G, PD, S, V, D]
        L.ref_sort_keys.restype = C.c_int
        L.ref_sort_keys.argtypes = [G, S, C.POINTER(C.c_uint32)]
        L.ref_communicate.argtypes = [G, V, C.c_int, C.c_int, C.c_int]
        L.ref_sync_currents.argtypes = [G, V, V]
        L.ref_conductor_walls.argtypes = [G, V, C.c_int, C.c_int]
        L.ref_output_divergence.argtypes = [G, V, V, C.c_int, D]
        _libs[key] = L
    return _libs[key]


def particles_lib(real):
    key = ("particles", "f32" if real == torch.float32 else "f64")
    if key not in _libs:
        paths = build_ref.build()
        if key not in paths:
            raise RuntimeError("the reference checkout is not available")
        L = C.CDLL(paths[key])
        L.ref_output_moment.restype = C.c_int
        L.ref_output_moment.argtypes = [C.POINTER(OrcGrid), C.POINTER(OrcSpecies)] + \
            [C.c_int] * 6 + [C.c_double, C.c_double, C.c_void_p, C.c_int]
        L.ref_sort.restype = C.c_int64
        L.ref_sort.argtypes = [C.POINTER(OrcGrid), C.POINTER(OrcSpecies), C.c_int, C.c_void_p,
                               C.c_int, C.c_void_p, C.c_int]
        _libs[key] = L
    return _libs[key]


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"reference kernel call failed ({rc})")


class RefOracle(Oracle):
    """The reference's kernels for one grid; order = the grid's shape order."""

    def __init__(self, g):
        super().__init__(g)
        self.R = lib(g.real, g.order)
        assert self.R.ref_n_ghosts() == g.ng, "ghost layers differ from the reference build"

    def push(self, sp, EB, dt, omegaB0, dx):
        s = self.species(sp)
        _check(self.R.ref_push(C.byref(self.og), C.byref(s), _p(EB), dt, omegaB0, dx))
        return 0

    def deposit(self, species, J, dt, dx, zero=True):
        if zero:
            J.zero_()
        for sp in species:
            s = self.species(sp)
            _check(self.R.ref_deposit(C.byref(self.og), C.byref(s), _p(J), dt, dx))

    def faraday(self, EB, c1, c2, stencil=None):
        st = None if stencil is None else (C.c_double * 9)(*stencil)
        _check(self.R.ref_faraday(C.byref(self.og), _p(EB), c1, c2, st))

    def ampere(self, EB, c1, c2):
        _check(self.R.ref_ampere(C.byref(self.og), _p(EB), c1, c2))

    def currents_ampere(self, EB, J, coeff, ppc0):
        _check(self.R.ref_currents_ampere(C.byref(self.og), _p(EB), _p(J), coeff, ppc0))

    def filter_pass(self, J, buff):
        _check(self.R.ref_filter_pass(C.byref(self.og), _p(J), _p(buff)))

    def gr_filter_pass(self, J, buff, axis_min=1, axis_max=1):
        _check(self.R.ref_filter_pass_axisym(C.byref(self.og), _p(J), _p(buff), axis_min,
                                             axis_max))

    def output_divergence(self, EB, bckp, comp, dx=1.0):
        _check(self.R.ref_output_divergence(C.byref(self.og), _p(EB), _p(bckp), comp, dx))

    def conductor_walls(self, EB, set_e, set_b):
        """The CONDUCTOR sides of the grid's field boundaries (set_field_bcs)."""
        _check(self.R.ref_conductor_walls(C.byref(self.og), _p(EB), int(set_e), int(set_b)))

    def fill_ghosts(self, fld, is_em, c0, c1):
        _check(self.R.ref_communicate(C.byref(self.og), _p(fld), int(is_em), c0, c1))

    def sync_currents(self, J, buff):
        _check(self.R.ref_sync_currents(C.byref(self.og), _p(J), _p(buff)))

    def output_moment(self, species, mom, bckp, comp):
        """ParticleMoments_kernel of the reference's container, as ComputeMoments
        launches it; mom as Oracle.output_moment."""
        S = particles_lib(self.g.real)
        for sp in species:
            s = self.species(sp)
            _check(S.ref_output_moment(C.byref(self.og), C.byref(s), mom["id"], mom.get("c1", 0),
                                       mom.get("c2", 0), mom.get("order", 0),
                                       mom.get("smoothing", 2), int(mom.get("use_weights", 0)),
                                       float(mom["inv_n0"]), float(mom["dx"]), _p(bckp), comp))

    def sort_particles(self, sp, remove_dead, pld_r=None, pld_i=None):
        """Particles::RemoveDead (when remove_dead) and SortSpatially of the
        reference's own particle container on the species, in place; the
        payloads (row-major particle x column tensors, pld_i int32) move with
        it. Returns the new particle count."""
        S = particles_lib(self.g.real)
        s = self.species(sp)
        nr = 0 if pld_r is None else pld_r.shape[1]
        ni = 0 if pld_i is None else pld_i.shape[1]
        assert pld_r is None or pld_r.is_contiguous()
        assert pld_i is None or (pld_i.is_contiguous() and pld_i.dtype == torch.int32)
        n = S.ref_sort(C.byref(self.og), C.byref(s), int(remove_dead),
                       None if pld_r is None else _p(pld_r), nr,
                       None if pld_i is None else _p(pld_i), ni)
        if n < 0:
            raise RuntimeError("reference sort failed")
        sp.npart = int(n)
        return int(n)

    def sort_keys(self, sp):
        s = self.species(sp)
        keys = torch.empty(max(sp.npart, 1), dtype=torch.int32)
        _check(self.R.ref_sort_keys(C.byref(self.og), C.byref(s),
                                    C.cast(keys.data_ptr(), C.POINTER(C.c_uint32))))
        return keys[:sp.npart].to(torch.int64) & 0xFFFFFFFF


class RefGROracle(GROracle):
    """The reference's GR kernels (gr::Pusher_kernel, the GRPIC deposit and
    metric::QKerrSchild<Dim::_2D>) with GROracle's interface; everything else
    stays the restated oracle's."""

    def __init__(self, g, a, r_min, r_max, th_min=0.0, th_max=3.141592653589793, r0=0.0,
                 h=0.0):
        super().__init__(g, a, r_min, r_max, th_min, th_max, r0, h)
        self.R = lib(g.real, g.order)
        assert self.R.ref_n_ghosts() == g.ng, "ghost layers differ from the reference build"
        self.mp = (C.c_double * 7)(r_min, r_max, th_min, th_max, a, r0, h)

    def metric(self, x):
        x = torch.as_tensor(x, dtype=torch.float64).contiguous()
        n = x.shape[0]
        out = torch.empty((n, GR_NQ), dtype=torch.float64)
        _check(self.R.ref_gr_metric(self.g.n[0], self.g.n[1], self.mp, _p(x), n, _p(out)))
        return {k: out[:, j] for j, k in enumerate(GR_NAMES)}

    def convert_x2(self, x, to_code):
        x = torch.as_tensor(x, dtype=torch.float64).contiguous()
        out = torch.empty_like(x)
        _check(self.R.ref_gr_convert_x2(self.g.n[0], self.g.n[1], self.mp, int(to_code), _p(x),
                                        x.numel(), _p(out)))
        return out

    def gr_push(self, sp, em, em0, dt, omegaB0, niter=10, absorb=(1, 1), axis=(1, 1),
                island=(0, 0)):
        assert island[1] <= island[0], "the reference has no FP64 island"
        s = self.species(sp)
        _check(self.R.ref_gr_push(C.byref(self.og), self.mp, C.byref(s), _p(em), _p(em0), dt,
                                  omegaB0, niter, (C.c_int * 2)(*absorb), (C.c_int * 2)(*axis)))

    def gr_deposit(self, species, J, dt, island=(0, 0), zero=True):
        assert island[1] <= island[0], "the reference has no FP64 island"
        if zero:
            J.zero_()
        for sp in species:
            s = self.species(sp)
            _check(self.R.ref_gr_deposit(C.byref(self.og), self.mp, C.byref(s), _p(J), dt))

    def _field(self, op, a, b, c, coeff=0.0, axis_min=1, axis_max=1):
        _check(self.R.ref_gr_field(C.byref(self.og), self.mp, op, _p(a), _p(b), _p(c), coeff,
                                   axis_min, axis_max))

    def gr_faraday(self, Bin, Bout, E, coeff, axis_min=1):
        self._field(0, Bin, Bout, E, coeff, axis_min, 1)

    def gr_ampere(self, Din, Dout, H, coeff, axis_min=1, axis_max=1):
        self._field(1, Din, Dout, H, coeff, axis_min, axis_max)

    def gr_currents_ampere(self, D, J, coeff, axis_min=1, axis_max=1):
        self._field(2, D, None, J, coeff, axis_min, axis_max)

    def gr_aux_e(self, D, B, E, axis_max=1):
        self._field(3, D, B, E, 0.0, 1, axis_max)

    def gr_aux_h(self, D, B, H, axis_max=1):
        self._field(4, D, B, H, 0.0, 1, axis_max)

    def gr_average_db(self, f, f0):
        self._field(5, f, f0, None)

    def gr_average_j(self, J, J0):
        self._field(6, J, J0, None)

    def gr_field_bcs(self, fld, set_e, set_b, axis_min=1, axis_max=1, horizon=1, nfilter=0):
        _check(self.R.ref_gr_field_bcs(C.byref(self.og), _p(fld), int(set_e), int(set_b),
                                       axis_min, axis_max, horizon, nfilter))
