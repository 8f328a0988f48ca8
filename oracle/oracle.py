"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker. Arrays are CPU torch tensors in the same layout as the
GPU path (see entity_gb300/inputs.py).
"""
import ctypes as C
import math
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


class OrcGrid(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int), ("ng", C.c_int),
        ("em_s", C.c_int64 * 4), ("cur_s", C.c_int64 * 4),
        ("periodic", C.c_int * 3), ("prtl_bc", (C.c_int * 2) * 3),
        ("fbc", (C.c_int * 2) * 3),
    ]


class OrcSpecies(C.Structure):
    _fields_ = [
        ("i1", C.c_void_p), ("i2", C.c_void_p), ("i3", C.c_void_p),
        ("i1_prev", C.c_void_p), ("i2_prev", C.c_void_p), ("i3_prev", C.c_void_p),
        ("dx1", C.c_void_p), ("dx2", C.c_void_p), ("dx3", C.c_void_p),
        ("dx1_prev", C.c_void_p), ("dx2_prev", C.c_void_p), ("dx3_prev", C.c_void_p),
        ("ux1", C.c_void_p), ("ux2", C.c_void_p), ("ux3", C.c_void_p),
        ("weight", C.c_void_p), ("tag", C.c_void_p),
        ("npart", C.c_int64), ("mass", C.c_float), ("charge", C.c_float), ("pusher", C.c_int),
    ]


_libs = {}


class OrcInjectParams(C.Structure):
    _fields_ = [("number_density", C.c_double), ("ppc0", C.c_double),
                ("xi_min", C.c_double * 3), ("xi_max", C.c_double * 3),
                ("temperature", C.c_double * 2), ("drift", (C.c_double * 3) * 2),
                ("seed", C.c_uint64), ("first_pair", C.c_uint64)]


def inject_params(number_density, ppc0, box, temperature, drift=((0, 0, 0), (0, 0, 0)), seed=1,
                  first_pair=0, cls=None):
    """Fills an injection parameter struct (the oracle's or, with cls, the
    product's identical layout); box = ((lo, hi), ...) per simulated axis."""
    p = (cls or OrcInjectParams)()
    p.number_density, p.ppc0 = number_density, ppc0
    for d, (lo, hi) in enumerate(box):
        p.xi_min[d], p.xi_max[d] = lo, hi
    for s in range(2):
        p.temperature[s] = temperature[s]
        for c in range(3):
            p.drift[s][c] = drift[s][c]
    p.seed, p.first_pair = seed, first_pair
    return p


def philox4x32_10(ctr, key):
    """One Philox4x32-10 block of the oracle (four uint32 words)."""
    L = lib(torch.float64)
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


def lib(real):
    tag = "f32" if real == torch.float32 else "f64"
    if tag not in _libs:
        from . import build_oracle
        paths = build_oracle.build()
        L = C.CDLL(paths[tag])
        V = C.c_void_p
        G = C.POINTER(OrcGrid)
        S = C.POINTER(OrcSpecies)
        L.orc_push.restype = C.c_int64
        L.orc_push.argtypes = [G, S, V, C.c_int, C.c_double, C.c_double, C.c_double]
        L.orc_deposit.argtypes = [G, S, V, C.c_int, C.c_double, C.c_double]
        L.orc_faraday.argtypes = [G, V, C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.orc_ampere.argtypes = [G, V, C.c_double, C.c_double]
        L.orc_currents_ampere.argtypes = [G, V, V, C.c_double, C.c_double]
        L.orc_filter_pass.argtypes = [G, V, V]
        L.orc_fill_ghosts.argtypes = [G, V, C.c_int, C.c_int, C.c_int]
        L.orc_sync_currents.argtypes = [G, V, V]
        L.orc_sort.argtypes = [G, S, C.POINTER(C.c_int64)]
        L.orc_sort_tiled.argtypes = [G, S, C.POINTER(C.c_int), C.POINTER(C.c_int64)]
        L.orc_remove_dead.restype = C.c_int64
        L.orc_remove_dead.argtypes = [G, S]
        L.orc_field_energy.argtypes = [G, V, C.c_double, C.POINTER(C.c_double)]
        L.orc_kinetic_energy.restype = C.c_double
        L.orc_kinetic_energy.argtypes = [S]
        L.orc_charge_density.argtypes = [G, S, V, C.c_int]
        L.orc_particle_moments.argtypes = [S, C.POINTER(C.c_double)]
        L.orc_field_boundaries.argtypes = [G, V, C.c_int, C.c_int, V, C.c_double * 3,
                                           C.c_double, (C.c_double * 2) * 3]
        L.orc_max_threads.restype = C.c_int
        L.orc_real_size.restype = C.c_int
        P = C.POINTER(OrcInjectParams)
        U32 = C.POINTER(C.c_uint32)
        L.orc_philox4x32_10.argtypes = [U32, U32, U32]
        L.orc_inject_count.restype = C.c_int64
        L.orc_inject_count.argtypes = [C.c_int, P]
        L.orc_inject_uniform.restype = C.c_int64
        L.orc_inject_uniform.argtypes = [G, S, S, P, C.POINTER(C.c_int64)]
        I, D_ = C.c_int, C.c_double
        L.orc_output_moment.argtypes = [G, S, I, I, I, I, I, I, D_, D_, V, I]
        L.orc_spline.restype = C.c_double
        L.orc_spline.argtypes = [I, D_]
        L.orc_sync_moments.argtypes = [G, V, I, I]
        L.orc_output_divergence.argtypes = [G, V, V, I]
        L.orc_normalize_by_rho.argtypes = [G, V, I, I, I, I]
        L.orc_output_field.argtypes = [G, V, I, I, I, C.c_uint, D_, C.POINTER(C.c_int), V]
        L.orc_output_particles.restype = C.c_int64
        L.orc_output_particles.argtypes = [G, S, C.c_int64, D_, C.POINTER(C.c_double), V, V, V,
                                           V, V, V, V]
        _libs[tag] = L
    return _libs[tag]


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class Oracle:
    """The reference algorithm on the CPU for one grid (see srpic_oracle.h)."""

    def __init__(self, g):
        self.g = g
        self.L = lib(g.real)
        og = OrcGrid()
        og.dim, og.ng = g.dim, g.ng
        og.n1, og.n2 = g.n[0], g.n[1]
        og.n3 = g.n[2] if g.dim == 3 else 1
        s = g.strides()
        for k in range(4):
            og.em_s[k] = s[k]
            og.cur_s[k] = s[k]
        for d in range(3):
            og.periodic[d] = int(g.periodic[d]) if d < g.dim else 0
            og.prtl_bc[d][0] = g.prtl_bc[d][0]
            og.prtl_bc[d][1] = g.prtl_bc[d][1]
            for h in range(2):
                og.fbc[d][h] = 0 if (d >= g.dim or g.periodic[d]) else 1
        self.og = og
        self.fbc_args = None

    def species(self, sp):
        os_ = OrcSpecies()
        os_.i1, os_.i2, os_.i3 = _p(sp.i[0]), _p(sp.i[1]), _p(sp.i[2])
        os_.i1_prev, os_.i2_prev, os_.i3_prev = _p(sp.i_prev[0]), _p(sp.i_prev[1]), _p(sp.i_prev[2])
        os_.dx1, os_.dx2, os_.dx3 = _p(sp.dx[0]), _p(sp.dx[1]), _p(sp.dx[2])
        os_.dx1_prev, os_.dx2_prev, os_.dx3_prev = (_p(sp.dx_prev[0]), _p(sp.dx_prev[1]),
                                                    _p(sp.dx_prev[2]))
        os_.ux1, os_.ux2, os_.ux3 = _p(sp.u[0]), _p(sp.u[1]), _p(sp.u[2])
        os_.weight, os_.tag = _p(sp.w), _p(sp.tag)
        os_.npart, os_.mass, os_.charge, os_.pusher = sp.npart, sp.mass, sp.charge, sp.pusher
        return os_

    def set_field_bcs(self, kinds, x_min=(0.0, 0.0, 0.0), dx=1.0, match_ds=None, target=None):
        """Field boundary kinds per side (0 periodic, 1 none, 2 conductor,
        3 match), as the product's pic_set_field_bcs."""
        for d in range(len(kinds)):
            for h in range(2):
                self.og.fbc[d][h] = kinds[d][h]
        ds = ((C.c_double * 2) * 3)()
        for d in range(3):
            for h in range(2):
                ds[d][h] = match_ds[d][h] if (match_ds is not None and d < len(match_ds)) else 0.0
        xm = (C.c_double * 3)(*[x_min[d] if d < len(x_min) else 0.0 for d in range(3)])
        self.fbc_args = (target, xm, dx, ds)

    def field_boundaries(self, EB, set_e, set_b):
        if not any(self.og.fbc[d][h] >= 2 for d in range(3) for h in range(2)):
            return
        target, xm, dx, ds = self.fbc_args
        self.L.orc_field_boundaries(C.byref(self.og), _p(EB), int(set_e), int(set_b), _p(target),
                                    xm, dx, ds)

    def inject_uniform(self, sp1, sp2, params):
        """Appends the injected pairs (both species' npart advance); returns
        (pairs, sampler failures)."""
        s1, s2 = self.species(sp1), self.species(sp2)
        bad = C.c_int64(0)
        n = self.L.orc_inject_uniform(C.byref(self.og), C.byref(s1), C.byref(s2),
                                      C.byref(params), C.byref(bad))
        sp1.npart, sp2.npart = s1.npart, s2.npart
        return n, bad.value

    def push(self, sp, EB, dt, omegaB0, dx):
        s = self.species(sp)
        return self.L.orc_push(C.byref(self.og), C.byref(s), _p(EB), self.g.order, dt, omegaB0, dx)

    def deposit(self, species, J, dt, dx, zero=True):
        if zero:
            J.zero_()
        for sp in species:
            s = self.species(sp)
            self.L.orc_deposit(C.byref(self.og), C.byref(s), _p(J), self.g.order, dt, dx)

    def faraday(self, EB, c1, c2, stencil=None):
        st = None if stencil is None else (C.c_double * 9)(*stencil)
        self.L.orc_faraday(C.byref(self.og), _p(EB), c1, c2, st)

    def ampere(self, EB, c1, c2):
        self.L.orc_ampere(C.byref(self.og), _p(EB), c1, c2)

    def currents_ampere(self, EB, J, coeff, ppc0):
        self.L.orc_currents_ampere(C.byref(self.og), _p(EB), _p(J), coeff, ppc0)

    def filter_pass(self, J, buff):
        self.L.orc_filter_pass(C.byref(self.og), _p(J), _p(buff))

    def fill_ghosts(self, fld, is_em, c0, c1):
        self.L.orc_fill_ghosts(C.byref(self.og), _p(fld), int(is_em), c0, c1)

    def sync_currents(self, J, buff):
        self.L.orc_sync_currents(C.byref(self.og), _p(J), _p(buff))

    def sort(self, sp):
        s = self.species(sp)
        perm = torch.empty(max(sp.npart, 1), dtype=torch.int64)
        self.L.orc_sort(C.byref(self.og), C.byref(s), C.cast(perm.data_ptr(), C.POINTER(C.c_int64)))
        return perm[:sp.npart]

    def sort_tiled(self, sp, tile):
        s = self.species(sp)
        perm = torch.empty(max(sp.npart, 1), dtype=torch.int64)
        ts = (C.c_int * 3)(*tile)
        self.L.orc_sort_tiled(C.byref(self.og), C.byref(s), ts,
                              C.cast(perm.data_ptr(), C.POINTER(C.c_int64)))
        return perm[:sp.npart]

    def remove_dead(self, sp):
        s = self.species(sp)
        n = self.L.orc_remove_dead(C.byref(self.og), C.byref(s))
        sp.npart = n
        return n

    def field_energy(self, EB, dx):
        out = (C.c_double * 2)()
        self.L.orc_field_energy(C.byref(self.og), _p(EB), dx, out)
        return out[0], out[1]

    def kinetic_energy(self, sp):
        s = self.species(sp)
        return self.L.orc_kinetic_energy(C.byref(s))

    def charge_density(self, species, rho):
        for sp in species:
            if sp.charge == 0.0:
                continue
            s = self.species(sp)
            self.L.orc_charge_density(C.byref(self.og), C.byref(s), _p(rho), self.g.order)

    def particle_moments(self, species):
        out = (C.c_double * 6)()
        for sp in species:
            s = self.species(sp)
            self.L.orc_particle_moments(C.byref(s), out)
        return list(out)

    # output preparation (output_oracle.c)
    def output_moment(self, species, mom, bckp, comp):
        """mom: dict(id, c1, c2, order, smoothing, use_weights, inv_n0, dx)."""
        for sp in species:
            s = self.species(sp)
            self.L.orc_output_moment(C.byref(self.og), C.byref(s), mom["id"], mom.get("c1", 0),
                                     mom.get("c2", 0), mom.get("order", 0),
                                     mom.get("smoothing", 2), int(mom.get("use_weights", 0)),
                                     float(mom["inv_n0"]), float(mom["dx"]), _p(bckp), comp)

    def spline(self, order, x):
        return self.L.orc_spline(order, x)

    def output_divergence(self, EB, bckp, comp):
        self.L.orc_output_divergence(C.byref(self.og), _p(EB), _p(bckp), comp)

    def sync_moments(self, bckp, c0, c1):
        self.L.orc_sync_moments(C.byref(self.og), _p(bckp), c0, c1)

    def normalize_by_rho(self, bckp, c_rho, cv):
        self.L.orc_normalize_by_rho(C.byref(self.og), _p(bckp), c_rho, cv[0], cv[1], cv[2])

    def output_field(self, src, is_em, c0, ncomp, flags, dx, dwn, out):
        d = (C.c_int * 3)(*[int(x) for x in (list(dwn) + [1, 1, 1])[:3]])
        self.L.orc_output_field(C.byref(self.og), _p(src), int(is_em), c0, ncomp, flags, dx, d,
                                _p(out))

    def output_particles(self, sp, stride, dx, xmin, x, u, w):
        s = self.species(sp)
        xm = (C.c_double * 3)(*[float(v) for v in (list(xmin) + [0.0, 0.0, 0.0])[:3]])
        xs = [(_p(x[d]) if d < len(x) else None) for d in range(3)]
        return self.L.orc_output_particles(C.byref(self.og), C.byref(s), int(stride), float(dx),
                                           xm, *xs, _p(u[0]), _p(u[1]), _p(u[2]), _p(w))

    # the SR step sequence of SRPICEngine::step_forward (srpic.hpp:65-188)
    def step(self, species, EB, J, buff, prm, step, filter_passes=None):
        g = self.g
        R = g.real
        t = lambda v: torch.tensor(v, dtype=R)
        if step == 0:
            self.fill_ghosts(EB, True, 0, 6)
        dT = t(0.5) * t(prm.correction) * t(prm.dt)
        # dx = sqrt(h_11) (fieldsolvers.h:50), rounded correctly
        npR = np.float32 if R == torch.float32 else np.float64
        dxm = t(float(np.sqrt(npR(prm.dx) * npR(prm.dx))))
        c1 = dT / (dxm * dxm) if g.dim == 2 else dT / dxm
        c2 = dT if g.dim == 2 else t(0.0)
        if prm.fieldsolver_enabled:
            self.faraday(EB, float(c1), float(c2))
            self.fill_ghosts(EB, True, 3, 6)
            self.field_boundaries(EB, 0, 1)
        for sp in species:
            if sp.pusher != 0 and sp.npart > 0:
                self.push(sp, EB, prm.dt, prm.omegaB0, prm.dx)
        if prm.deposit_enabled:
            self.deposit(species, J, prm.dt, prm.dx)
            self.sync_currents(J, buff)
            self.fill_ghosts(J, False, 0, 3)
            for _ in range(prm.nfilter if filter_passes is None else filter_passes):
                self.filter_pass(J, buff)
                self.fill_ghosts(J, False, 0, 3)
        if prm.fieldsolver_enabled:
            self.faraday(EB, float(c1), float(c2))
            self.fill_ghosts(EB, True, 3, 6)
            self.field_boundaries(EB, 0, 1)
            dT1 = t(1.0) * t(prm.correction) * t(prm.dt)
            a1 = dT1 / (dxm * dxm) if g.dim == 2 else dT1 / dxm
            a2 = dT1 if g.dim == 2 else t(0.0)
            self.ampere(EB, float(a1), float(a2))
            if prm.deposit_enabled:
                jc = -t(prm.dt) * t(prm.q0) / (t(prm.B0) * t(prm.V0))
                self.currents_ampere(EB, J, float(jc), prm.ppc0)
                self.fill_ghosts(EB, True, 0, 3)
                self.fill_ghosts(J, False, 0, 3)
            else:
                self.fill_ghosts(EB, True, 0, 3)
            self.field_boundaries(EB, 1, 0)
        for sp in species:
            if prm.clear_interval > 0 and step % prm.clear_interval == 0 and step > 0:
                self.remove_dead(sp)
            if prm.sort_interval > 0 and step % prm.sort_interval == 0:
                self.sort(sp)


# ---------------------------------------------------------------------------
# GR (QKerrSchild) oracle, grpic_oracle.h
# ---------------------------------------------------------------------------
class OrcQKS(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("a", "rh", "r0", "h", "chi_min", "eta_min", "dchi",
                                          "deta", "dchi_inv", "deta_inv", "x2_small",
                                          "x2_large")] + [
        ("small_angle", C.c_int)]


GR_NQ = 24
GR_NAMES = ["h_11", "h_22", "h_33", "h_13", "h11", "h22", "h33", "h13", "alpha", "beta1",
            "sqrt_det_h", "sqrt_det_h_tilde", "dr_alpha", "dt_alpha", "dr_beta1", "dt_beta1",
            "dr_h11", "dr_h22", "dr_h33", "dr_h13", "dt_h11", "dt_h22", "dt_h33", "dt_h13"]


def _gr_sigs(L):
    if getattr(L, "_gr_ready", False):
        return L
    V, D = C.c_void_p, C.c_double
    Q, G, S = C.POINTER(OrcQKS), C.POINTER(OrcGrid), C.POINTER(OrcSpecies)
    I2 = C.c_int * 2
    L.orc_qks_init.argtypes = [Q, C.c_int, C.c_int, D, D, D, D, D, D, D]
    L.orc_qks_theta2eta.restype = D
    L.orc_qks_theta2eta.argtypes = [D, D]
    L.orc_qks_eta2theta.restype = D
    L.orc_qks_eta2theta.argtypes = [D, D]
    L.orc_gr_convert_x2.argtypes = [Q, C.c_int, V, C.c_int64, V]
    L.orc_gr_metric.argtypes = [Q, V, C.c_int64, V]
    L.orc_gr_transform.argtypes = [Q, C.c_int, V, V, C.c_int64, V]
    L.orc_gr_push.argtypes = [G, Q, S, V, V, D, D, C.c_int, C.c_int, I2, I2, C.c_int, C.c_int]
    L.orc_gr_deposit.argtypes = [G, Q, S, V, D, C.c_int, C.c_int]
    L.orc_gr_faraday.argtypes = [G, Q, V, V, V, D, C.c_int]
    L.orc_gr_ampere.argtypes = [G, Q, V, V, V, D, C.c_int, C.c_int]
    L.orc_gr_currents_ampere.argtypes = [G, Q, V, V, D, C.c_int, C.c_int]
    L.orc_gr_aux_e.argtypes = [G, Q, V, V, V, C.c_int]
    L.orc_gr_aux_h.argtypes = [G, Q, V, V, V, C.c_int]
    L.orc_gr_average_db.argtypes = [G, V, V]
    L.orc_gr_average_j.argtypes = [G, V, V]
    L.orc_gr_filter_pass.argtypes = [G, V, V, C.c_int, C.c_int]
    L.orc_gr_field_bcs.argtypes = [G, V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.orc_gr_match.argtypes = [G, Q, V, V, D, D, D, C.c_int, C.c_int, C.c_int, C.c_int]
    L.orc_gr_absorb_currents.argtypes = [G, Q, V, D, D, D]
    L.orc_gr_inject_uniform.restype = C.c_int64
    L.orc_gr_inject_uniform.argtypes = [G, Q, S, S, C.POINTER(OrcInjectParams), D,
                                        C.POINTER(C.c_int64)]
    L._gr_ready = True
    return L


class GROracle(Oracle):
    """The reference's GR kernels on the CPU for one (r, theta) grid."""

    def __init__(self, g, a, r_min, r_max, th_min=0.0, th_max=math.pi, r0=0.0, h=0.0):
        super().__init__(g)
        _gr_sigs(self.L)
        self.q = OrcQKS()
        self.L.orc_qks_init(C.byref(self.q), g.n[0], g.n[1], r_min, r_max, th_min, th_max, a,
                            r0, h)
        self.r_min, self.r_max = r_min, r_max

    def convert_x2(self, x, to_code):
        """theta -> code x2 (to_code) or code x2 -> theta at the points x."""
        x = torch.as_tensor(x, dtype=torch.float64).contiguous()
        out = torch.empty_like(x)
        self.L.orc_gr_convert_x2(C.byref(self.q), int(to_code), _p(x), x.numel(), _p(out))
        return out

    def gr_match(self, fld, target, ds, set_e=1, set_b=1, axis_min=1, axis_max=1):
        self.L.orc_gr_match(C.byref(self.og), C.byref(self.q), _p(fld), _p(target), ds,
                            self.r_min, self.r_max, int(set_e), int(set_b), axis_min, axis_max)

    def gr_absorb_currents(self, J, ds):
        self.L.orc_gr_absorb_currents(C.byref(self.og), C.byref(self.q), _p(J), ds, self.r_min,
                                      self.r_max)

    def gr_inject_uniform(self, sp1, sp2, params, V0):
        s1, s2 = self.species(sp1), self.species(sp2)
        bad = C.c_int64(0)
        n = self.L.orc_gr_inject_uniform(C.byref(self.og), C.byref(self.q), C.byref(s1),
                                         C.byref(s2), C.byref(params), V0, C.byref(bad))
        sp1.npart, sp2.npart = s1.npart, s2.npart
        return n, bad.value

    def metric(self, x):
        x = torch.as_tensor(x, dtype=torch.float64).contiguous()
        n = x.shape[0]
        out = torch.empty((n, GR_NQ), dtype=torch.float64)
        self.L.orc_gr_metric(C.byref(self.q), _p(x), n, _p(out))
        return {k: out[:, j] for j, k in enumerate(GR_NAMES)}

    def transform(self, kind, x, v):
        x = torch.as_tensor(x, dtype=torch.float64).contiguous()
        v = torch.as_tensor(v, dtype=torch.float64).contiguous()
        out = torch.empty_like(v)
        self.L.orc_gr_transform(C.byref(self.q), kind, _p(x), _p(v), x.shape[0], _p(out))
        return out

    def gr_push(self, sp, em, em0, dt, omegaB0, niter=10, absorb=(1, 1), axis=(1, 1),
                island=(0, 0)):
        s = self.species(sp)
        self.L.orc_gr_push(C.byref(self.og), C.byref(self.q), C.byref(s), _p(em), _p(em0), dt,
                           omegaB0, niter, self.g.order, (C.c_int * 2)(*absorb),
                           (C.c_int * 2)(*axis), island[0], island[1])

    def gr_deposit(self, species, J, dt, island=(0, 0), zero=True):
        if zero:
            J.zero_()
        for sp in species:
            s = self.species(sp)
            self.L.orc_gr_deposit(C.byref(self.og), C.byref(self.q), C.byref(s), _p(J), dt,
                                  island[0], island[1])

    def gr_faraday(self, Bin, Bout, E, coeff, axis_min=1):
        self.L.orc_gr_faraday(C.byref(self.og), C.byref(self.q), _p(Bin), _p(Bout), _p(E), coeff,
                              axis_min)

    def gr_ampere(self, Din, Dout, H, coeff, axis_min=1, axis_max=1):
        self.L.orc_gr_ampere(C.byref(self.og), C.byref(self.q), _p(Din), _p(Dout), _p(H), coeff,
                             axis_min, axis_max)

    def gr_currents_ampere(self, D, J, coeff, axis_min=1, axis_max=1):
        self.L.orc_gr_currents_ampere(C.byref(self.og), C.byref(self.q), _p(D), _p(J), coeff,
                                      axis_min, axis_max)

    def gr_aux_e(self, D, B, E, axis_max=1):
        self.L.orc_gr_aux_e(C.byref(self.og), C.byref(self.q), _p(D), _p(B), _p(E), axis_max)

    def gr_aux_h(self, D, B, H, axis_max=1):
        self.L.orc_gr_aux_h(C.byref(self.og), C.byref(self.q), _p(D), _p(B), _p(H), axis_max)

    def gr_average_db(self, f, f0):
        self.L.orc_gr_average_db(C.byref(self.og), _p(f), _p(f0))

    def gr_average_j(self, J, J0):
        self.L.orc_gr_average_j(C.byref(self.og), _p(J), _p(J0))

    def gr_filter_pass(self, J, buff, axis_min=1, axis_max=1):
        self.L.orc_gr_filter_pass(C.byref(self.og), _p(J), _p(buff), axis_min, axis_max)

    def gr_field_bcs(self, fld, set_e, set_b, axis_min=1, axis_max=1, horizon=1, nfilter=0):
        self.L.orc_gr_field_bcs(C.byref(self.og), _p(fld), int(set_e), int(set_b), axis_min,
                                axis_max, horizon, nfilter)

    # GRPICEngine::step_forward (grpic.hpp:66-634), the sequence of the
    # product's engine: fields = [em, em0, aux, cur, cur0, buff], swapped in
    # place; axis/horizon boundaries on em and em0 after each update
    def grpic_step(self, species, fields, prm, niter=10, island=(0, 0), step=0, flags=(1, 1, 1),
                   match=None):
        R = self.g.real
        t = lambda v: torch.tensor(v, dtype=R)
        amin, amax, hor = flags

        def bc(set_e, set_b):
            # orth order: horizon (-x1), axis (-x2, +x2), match (+x1)
            for f in fields[:2]:
                self.gr_field_bcs(f, set_e, set_b, amin, amax, hor, prm.nfilter)
                if match is not None:
                    self.gr_match(f, match[1], match[0], set_e, set_b, amin, amax)

        def swap():
            fields[0], fields[1] = fields[1], fields[0]
            fields[3], fields[4] = fields[4], fields[3]

        dt = t(prm.dt)
        dT1 = float(t(1.0) * t(prm.correction) * dt)
        dTh = float(t(0.5) * t(prm.correction) * dt)
        jc = float(-dt * t(prm.q0) / t(prm.B0))
        fs, dep = prm.fieldsolver_enabled, prm.deposit_enabled
        em, em0, aux = fields[0], fields[1], fields[2]
        if step == 0:
            if fs:
                bc(1, 1)
                fields[1].copy_(fields[0])
                em, em0 = fields[0], fields[1]
                self.gr_aux_e(em, em0, aux, amax)
                self.gr_aux_h(em, em0, aux, amax)
                self.gr_faraday(em0, em0, aux, dTh, amin)
                bc(0, 1)
                self.gr_ampere(em, em, aux, dTh, amin, amax)
                bc(1, 0)
                self.gr_aux_e(em, em0, aux, amax)
                self.gr_aux_h(em, em0, aux, amax)
                self.gr_faraday(em, em0, aux, dT1, amin)
                bc(0, 1)
                self.gr_ampere(em0, em0, aux, dT1, amin, amax)
                bc(1, 0)
                self.gr_aux_h(em0, em0, aux, amax)
                self.gr_ampere(em, em0, aux, dT1, amin, amax)
                bc(1, 0)
                swap()
            else:
                fields[1].copy_(fields[0])
        em, em0 = fields[0], fields[1]
        if fs:
            self.gr_average_db(em, em0)
            self.gr_aux_e(em0, em, aux, amax)
            self.gr_faraday(em0, em0, aux, dT1, amin)
            bc(0, 1)
            self.gr_aux_h(em, em0, aux, amax)
        for sp in species:
            if sp.npart > 0 and sp.pusher != 0:
                self.gr_push(sp, em, em0, float(dt), prm.omegaB0, niter, island=island)
        if dep:
            self.gr_deposit(species, fields[4], float(dt), island=island)
            if match is not None and self.g.prtl_bc[0][1] == 1:
                self.gr_absorb_currents(fields[4], match[0])
            for _ in range(prm.nfilter):
                self.gr_filter_pass(fields[4], fields[5], amin, amax)
        if fs:
            cur, cur0 = fields[3], fields[4]
            if dep:
                self.gr_average_j(cur, cur0)
            self.gr_aux_e(em, em0, aux, amax)
            self.gr_faraday(em, em0, aux, dT1, amin)
            bc(0, 1)
            self.gr_ampere(em0, em0, aux, dT1, amin, amax)
            if dep:
                self.gr_currents_ampere(em0, cur, jc, amin, amax)
            bc(1, 0)
            self.gr_aux_h(em0, em0, aux, amax)
            self.gr_ampere(em, em0, aux, dT1, amin, amax)
            if dep:
                self.gr_currents_ampere(em0, cur0, jc, amin, amax)
            swap()
            bc(1, 0)
        for sp in species:
            if prm.clear_interval > 0 and step % prm.clear_interval == 0 and step > 0:
                self.remove_dead(sp)
            if prm.sort_interval > 0 and step % prm.sort_interval == 0:
                self.sort(sp)
