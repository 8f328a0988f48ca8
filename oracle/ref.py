"""ctypes binding of oracle/_ref: Entity's own SR kernels compiled from the
reference sources against the host Kokkos shim (TEST INFRASTRUCTURE ONLY).

RefOracle has the Oracle's interface for the kernels the reference build
provides (push, deposit, Faraday, Ampere, CurrentsAmpere, one filter pass,
the sort key) and keeps the restated exchange routines for the rest, so
Oracle.step runs the reference's kernels in the reference's step order.
"""
import ctypes as C

import torch

from . import build_ref
from .oracle import Oracle, OrcGrid, OrcSpecies, _p

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
        L.ref_sort_keys.restype = C.c_int
        L.ref_sort_keys.argtypes = [G, S, C.POINTER(C.c_uint32)]
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

    def sort_keys(self, sp):
        s = self.species(sp)
        keys = torch.empty(max(sp.npart, 1), dtype=torch.int32)
        _check(self.R.ref_sort_keys(C.byref(self.og), C.byref(s),
                                    C.cast(keys.data_ptr(), C.POINTER(C.c_uint32))))
        return keys[:sp.npart].to(torch.int64) & 0xFFFFFFFF
