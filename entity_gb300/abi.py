"""ctypes binding of libentity_pic.so (the C ABI declared in include/entity_pic.h).

This is the same binding a Python caller of the reference-facing ABI would
write. There is no fallback: if the library is missing or fails to load, every
call raises.
"""
import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libentity_pic.so")

PIC_OK = 0
PIC_ERR_ARG = -1
PIC_ERR_CUDA = -2
PIC_ERR_UNSUPPORTED = -3
PIC_ERR_NOMEM = -4
PIC_ERR_DEVICE = -5

PIC_TAG_DEAD = 0
PIC_TAG_ALIVE = 1

PIC_PUSHER_NONE = 0
PIC_PUSHER_BORIS = 1
PIC_PUSHER_VAY = 2
PIC_PUSHER_PHOTON = 3

PIC_BC_PERIODIC = 0
PIC_BC_ABSORB = 1
PIC_BC_REFLECT = 2
PIC_BC_AXIS = 3

PIC_PD_WRITE_PREV = 1
PIC_PD_NO_ZERO = 2
PIC_PD_FLOAT_ATOMICS = 4

PIC_SORT_REMOVE_DEAD = 1
PIC_SORT_SKIP_PREV = 2
PIC_SORT_SPATIAL = 4
PIC_SORT_TILED = 8
PIC_SORT_NO_SYNC = 16


class PicGrid(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("n", C.c_int32 * 3),
        ("ng", C.c_int32),
        ("order", C.c_int32),
        ("real_bytes", C.c_int32),
        ("fld_periodic", C.c_int32 * 3),
        ("prtl_bc", (C.c_int32 * 2) * 3),
        ("em_stride", C.c_int64 * 4),
        ("cur_stride", C.c_int64 * 4),
    ]


class PicSpecies(C.Structure):
    _fields_ = [
        ("i1", C.c_void_p), ("i2", C.c_void_p), ("i3", C.c_void_p),
        ("i1_prev", C.c_void_p), ("i2_prev", C.c_void_p), ("i3_prev", C.c_void_p),
        ("dx1", C.c_void_p), ("dx2", C.c_void_p), ("dx3", C.c_void_p),
        ("dx1_prev", C.c_void_p), ("dx2_prev", C.c_void_p), ("dx3_prev", C.c_void_p),
        ("ux1", C.c_void_p), ("ux2", C.c_void_p), ("ux3", C.c_void_p),
        ("weight", C.c_void_p),
        ("tag", C.c_void_p),
        ("npart", C.c_int64),
        ("maxnpart", C.c_int64),
        ("mass", C.c_float),
        ("charge", C.c_float),
        ("pusher", C.c_int32),
        ("index", C.c_int32),
        ("phi", C.c_void_p),
        ("pld_r", C.c_void_p),
        ("pld_i", C.c_void_p),
        ("pld_r_stride", C.c_int64 * 2),
        ("pld_i_stride", C.c_int64 * 2),
        ("npld_r", C.c_int32),
        ("npld_i", C.c_int32),
    ]


class PicSpeciesAdjoint(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("lx1", "lx2", "lx3", "lu1", "lu2", "lu3", "lw")]


class PicGRMetric(C.Structure):
    _fields_ = [("a", C.c_double), ("r0", C.c_double), ("h", C.c_double),
                ("x1min", C.c_double), ("x1max", C.c_double),
                ("x2min", C.c_double), ("x2max", C.c_double),
                ("axis_min", C.c_int32), ("axis_max", C.c_int32), ("horizon", C.c_int32)]


class PicInjectParams(C.Structure):
    _fields_ = [("number_density", C.c_double), ("ppc0", C.c_double),
                ("xi_min", C.c_double * 3), ("xi_max", C.c_double * 3),
                ("temperature", C.c_double * 2), ("drift", (C.c_double * 3) * 2),
                ("seed", C.c_uint64), ("first_pair", C.c_uint64)]


PIC_FBC_PERIODIC, PIC_FBC_NONE, PIC_FBC_CONDUCTOR, PIC_FBC_MATCH = 0, 1, 2, 3

PIC_MOM_RHO, PIC_MOM_CHARGE, PIC_MOM_N, PIC_MOM_NPPC, PIC_MOM_T, PIC_MOM_V = range(6)
PIC_SMOOTH_CONST, PIC_SMOOTH_SPLINE = 1, 2
PIC_OUT_INTERP_EDGES, PIC_OUT_INTERP_FACES, PIC_OUT_TO_HAT = 1, 2, 4


class PicMomentParams(C.Structure):
    _fields_ = [("id", C.c_int32), ("c1", C.c_int32), ("c2", C.c_int32), ("order", C.c_int32),
                ("smoothing", C.c_int32), ("use_weights", C.c_int32), ("inv_n0", C.c_double),
                ("dx", C.c_double)]


class PicFieldBCs(C.Structure):
    _fields_ = [("kind", (C.c_int32 * 2) * 3), ("x_min", C.c_double * 3), ("dx", C.c_double),
                ("match_ds", (C.c_double * 2) * 3), ("match_target", C.c_void_p)]


class PicGRParams(C.Structure):
    _fields_ = [("niter", C.c_int32), ("island_lo", C.c_int32), ("island_hi", C.c_int32),
                ("match_ds", C.c_double), ("match_target", C.c_void_p)]


class PicStepParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("dx", C.c_double), ("omegaB0", C.c_double),
        ("correction", C.c_double),
        ("q0", C.c_double), ("B0", C.c_double), ("V0", C.c_double), ("ppc0", C.c_double),
        ("nfilter", C.c_int32), ("sort_interval", C.c_int32), ("clear_interval", C.c_int32),
        ("fieldsolver_enabled", C.c_int32), ("deposit_enabled", C.c_int32),
        ("write_prev", C.c_int32), ("sort_tiled", C.c_int32), ("deposit_flags", C.c_int32),
    ]


# name -> (restype, argtypes); the complete exported surface of entity_pic.h
_VP = C.c_void_p
SIGNATURES = {
    "pic_version": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pic_status_string": (C.c_char_p, [C.c_int]),
    "pic_kernel_launches": (C.c_int64, []),
    "pic_create": (C.c_int, [C.POINTER(PicGrid), C.POINTER(_VP)]),
    "pic_destroy": (C.c_int, [_VP]),
    "pic_get_grid": (C.c_int, [_VP, C.POINTER(PicGrid)]),
    "pic_tile_shape": (C.c_int, [_VP, C.POINTER(C.c_int32)]),
    "pic_faraday": (C.c_int, [_VP, _VP, C.c_double, C.c_double, C.POINTER(C.c_double), _VP]),
    "pic_ampere": (C.c_int, [_VP, _VP, C.c_double, C.c_double, _VP]),
    "pic_currents_ampere": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_double, _VP]),
    "pic_ampere_currents": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_double, C.c_double,
                                      C.c_double, _VP]),
    "pic_push": (C.c_int, [_VP, C.POINTER(PicSpecies), _VP, C.c_double, C.c_double,
                           C.c_double, _VP]),
    "pic_deposit": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32, _VP, C.c_double,
                              C.c_double, _VP]),
    "pic_push_deposit": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32, _VP, _VP, C.c_double,
                                   C.c_double, C.c_double, C.c_uint32, _VP]),
    "pic_tile_offsets": (C.c_int, [_VP, C.POINTER(PicSpecies), C.POINTER(C.c_int32), C.c_int64,
                                   C.POINTER(C.c_int64), _VP]),
    "pic_push_deposit_tiles": (C.c_int, [_VP, C.POINTER(PicSpecies), _VP, _VP, C.c_double,
                                         C.c_double, C.c_double, C.c_int64, C.c_int64, C.c_uint32,
                                         _VP]),
    "pic_sync_currents": (C.c_int, [_VP, _VP, _VP, _VP]),
    "pic_filter_currents": (C.c_int, [_VP, _VP, _VP, C.c_int32, _VP]),
    "pic_fill_ghosts": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, C.c_int32, _VP]),
    "pic_sort": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_uint32, C.POINTER(C.c_int64), _VP]),
    "pic_field_energy": (C.c_int, [_VP, _VP, C.c_double, C.POINTER(C.c_double), _VP]),
    "pic_field_energy_noalloc": (C.c_int, [C.POINTER(PicGrid), _VP, C.c_double,
                                           C.POINTER(C.c_double), _VP]),
    "pic_get_device_errors": (C.c_int, [_VP, C.POINTER(C.c_int64), C.c_int32, _VP]),
    "pic_get_wait_timeouts": (C.c_int, [_VP, C.POINTER(C.c_int64), C.c_int32, _VP]),
    "pic_particle_moments": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32,
                                       C.POINTER(C.c_double), _VP]),
    "pic_charge_density": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32, _VP, _VP]),
    "pic_set_field_bcs": (C.c_int, [_VP, C.POINTER(PicFieldBCs)]),
    "pic_field_boundaries": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, _VP]),
    "pic_output_moment": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32,
                                    C.POINTER(PicMomentParams), _VP, C.c_int32, _VP]),
    "pic_sync_moments": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, _VP]),
    "pic_normalize_by_rho": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       _VP]),
    "pic_output_divergence": (C.c_int, [_VP, _VP, _VP, C.c_int32, _VP]),
    "pic_output_field": (C.c_int, [_VP, _VP, C.c_int32, C.c_int32, C.c_int32, C.c_uint32,
                                   C.c_double, C.POINTER(C.c_int32), _VP, _VP]),
    "pic_output_particles": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int64, C.c_double,
                                       C.POINTER(C.c_double), C.POINTER(_VP), C.POINTER(_VP),
                                       _VP, C.POINTER(C.c_int64), _VP]),
    "pic_inject_uniform_maxwellians": (C.c_int, [_VP, C.POINTER(PicSpecies),
                                                 C.POINTER(PicSpecies),
                                                 C.POINTER(PicInjectParams),
                                                 C.POINTER(C.c_int64), _VP]),
    "pic_gr_inject_uniform_maxwellians": (C.c_int, [_VP, C.POINTER(PicGRMetric),
                                                    C.POINTER(PicSpecies), C.POINTER(PicSpecies),
                                                    C.POINTER(PicInjectParams), C.c_double,
                                                    C.POINTER(C.c_int64), _VP]),
    "pic_srpic_step": (C.c_int, [_VP, C.POINTER(PicSpecies), C.c_int32, _VP, _VP, _VP,
                                 C.POINTER(PicStepParams), C.c_int64, _VP]),
    "pic_host_pipe_create": (C.c_int, [C.POINTER(_VP)]),
    "pic_host_pipe_destroy": (C.c_int, [_VP]),
    "pic_host_pipe_sync": (C.c_int, [_VP]),
    "pic_host_pipe_set_groups": (C.c_int, [_VP, C.c_int32, C.c_int64]),
    "pic_host_pipe_bytes": (C.c_int, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "pic_srpic_step_host": (C.c_int, [_VP, _VP, C.POINTER(PicSpecies), C.POINTER(PicSpecies),
                                      C.c_int32, _VP, _VP, _VP, _VP, _VP,
                                      C.POINTER(PicStepParams), C.c_int64, _VP]),
    "pic_checkpoint_save": (C.c_int, [_VP, C.c_int32, C.POINTER(PicSpecies), C.c_int32, _VP,
                                      _VP]),
    "pic_checkpoint_restore": (C.c_int, [_VP, C.c_int32, C.POINTER(PicSpecies), C.c_int32,
                                         _VP, _VP]),
    "pic_checkpoint_release": (C.c_int, [_VP]),
    "pic_checkpoint_view": (C.c_int, [_VP, C.c_int32, C.POINTER(PicSpecies), C.c_int32,
                                      C.POINTER(PicSpecies), C.POINTER(_VP)]),
    "pic_field_energy_adjoint_seed": (C.c_int, [_VP, _VP, _VP, C.c_double, _VP]),
    "pic_srpic_step_adjoint": (C.c_int, [_VP, C.POINTER(PicSpecies),
                                         C.POINTER(PicSpeciesAdjoint), C.c_int32, _VP, _VP,
                                         C.POINTER(PicStepParams), _VP]),
    "pic_srpic_gradient": (C.c_int, [_VP, C.POINTER(PicSpecies), C.POINTER(PicSpeciesAdjoint),
                                     C.c_int32, _VP, _VP, _VP, C.POINTER(PicStepParams),
                                     C.c_int64, C.c_int64, _VP, C.POINTER(C.c_double), _VP]),
    "pic_gr_metric_eval": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, C.c_int64, _VP, _VP]),
    "pic_gr_push": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.POINTER(PicSpecies), _VP, _VP,
                              C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32, _VP]),
    "pic_gr_particle_push": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.POINTER(PicSpecies),
                                       C.c_int32, _VP, _VP, C.c_double, C.c_double, C.c_int32,
                                       C.c_int32, C.c_int32, _VP]),
    "pic_gr_deposit": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.POINTER(PicSpecies), C.c_int32,
                                 _VP, C.c_double, C.c_int32, C.c_int32, C.c_uint32, _VP]),
    "pic_gr_faraday": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP, _VP, C.c_double, _VP]),
    "pic_gr_ampere": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP, _VP, C.c_double, _VP]),
    "pic_gr_currents_ampere": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP, C.c_double,
                                         _VP]),
    "pic_gr_aux": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.c_int32, _VP, _VP, _VP, _VP]),
    "pic_gr_average": (C.c_int, [_VP, C.c_int32, _VP, _VP, _VP]),
    "pic_gr_filter_currents": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP, C.c_int32,
                                         _VP]),
    "pic_gr_field_bcs": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, C.c_int32, C.c_int32,
                                   C.c_int32, _VP]),
    "pic_gr_init_vertical": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP]),
    "pic_gr_match_fields": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, _VP, C.c_double,
                                      C.c_int32, C.c_int32, _VP]),
    "pic_gr_absorb_currents": (C.c_int, [_VP, C.POINTER(PicGRMetric), _VP, C.c_double, _VP]),
    "pic_gr_min_cell_size": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.POINTER(C.c_double),
                                       _VP]),
    "pic_grpic_step": (C.c_int, [_VP, C.POINTER(PicGRMetric), C.POINTER(PicSpecies), C.c_int32,
                                 C.POINTER(_VP), C.POINTER(PicStepParams),
                                 C.POINTER(PicGRParams), C.c_int64, _VP]),
    "pic_timers_enable": (C.c_int, [_VP, C.c_int32]),
    "pic_timers_reset": (C.c_int, [_VP]),
    "pic_timers_read": (C.c_int, [_VP, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "pic_timer_mark": (C.c_int, [_VP, C.c_int32, C.c_int32, _VP]),
}

PIC_PHASES = ["FieldSolver", "PushDeposit", "Communications", "CurrentFiltering",
              "ParticleSort", "Step"]

_lib = None


class PicError(RuntimeError):
    def __init__(self, fn, status):
        self.status = status
        super().__init__(f"{fn} returned {status} ({status_string(status)})")


def load(path=LIB_PATH):
    """Loads the library (once) and declares every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(st):
    return load().pic_status_string(st).decode()


def check(fn_name, st):
    if st != PIC_OK:
        raise PicError(fn_name, st)
    return st


def call(name, *args):
    """Calls an entry point and raises PicError on a non-zero status."""
    return check(name, getattr(load(), name)(*args))
