"""Field and particle output of one SR Cartesian domain.

The reference writes output in Metadomain::Write
(src/framework/domain/metadomain_io.cpp:380-700) and Particles::OutputWrite
(src/framework/containers/particles_io.cpp:93-235) through ADIOS2. This
module does the same steps with the device doing all the array work:
- pic_output_moment, pic_sync_moments and pic_normalize_by_rho prepare the
  moments;
- pic_output_divergence computes divE;
- pic_output_field gives cell-centred tetrad components, downsampled;
- pic_output_particles gives every stride-th particle in physical units.

The packed arrays are copied to the host once per quantity. One `.npz` file
per output step holds the arrays under the reference's variable names:
`fE1`, `fB2`, `fJ3`, `fN_1_2`, `fRho`, `fT00`, `fT0i` components such as
`fT01`, `fV1`, `fNppc`, `fDivE`, `pX1_1`, `pU1_1`, `pW_1`, the mesh `X1`
and `X1e`, `Step` and `Time`. Field arrays are indexed [x3][x2][x1], the
transpose of the reference's (x1, x2, x3) extents. ADIOS2 is not part of
this build, so these are the arrays ADIOS2 would receive, not a BP file.

Field names follow OutputField (src/output/fields.cpp:20-84,
src/output/fields.h:86-150) and InterpretComponents
(src/output/utils/interpret_prompt.cpp:14-92).
"""
import math
import os
from dataclasses import dataclass, field

import numpy as np
import torch

from . import abi
from .inputs import GridSpec

# FldsID names (src/global/enums.h:248-280) this output supports
_FIELDS = {"e": "E", "b": "B", "j": "J"}
_MOMENTS = {"rho": abi.PIC_MOM_RHO, "charge": abi.PIC_MOM_CHARGE, "n": abi.PIC_MOM_N,
            "nppc": abi.PIC_MOM_NPPC, "t": abi.PIC_MOM_T, "v": abi.PIC_MOM_V}
_CASE = {"rho": "Rho", "charge": "Charge", "n": "N", "nppc": "Nppc", "t": "T", "v": "V",
         "dive": "DivE"}


def _components(chars):
    """InterpretComponents: list of component tuples for 1 or 2 characters."""
    m = {"t": 0, "x": 1, "y": 2, "z": 3, "0": 0, "1": 1, "2": 2, "3": 3, "i": -1, "j": -2}
    if len(chars) > 2 or any(c not in m for c in chars):
        raise ValueError("Invalid field name")
    cs = [m[c] for c in chars]
    if len(cs) == 1:
        c = cs[0]
        if c < 0:
            return [(k,) for k in (1, 2, 3)]
        if c == 0 or c > 3:
            raise ValueError("Invalid field name")
        return [(c,)]
    c1, c2 = cs
    out = []
    if c1 < 0:
        for i in range(3):
            if c2 < 0:
                if c2 == c1:
                    out.append((i + 1, i + 1))
                else:
                    out.extend((i + 1, j + 1) for j in range(i, 3))
            else:
                out.append((i + 1, c2))
    elif c2 < 0:
        out.extend((c1, j + 1) for j in range(3))
    else:
        out.append((c1, c2))
    return out


@dataclass
class OutputField:
    """One requested quantity (OutputField, src/output/fields.cpp:20-84)."""
    name_in: str
    kind: str = ""                  # "e", "b", "j", "dive" or a moment key
    species: list = field(default_factory=list)
    comp: list = field(default_factory=list)

    def __post_init__(self):
        raw = self.name_in.split("_")[0]
        low = raw.lower()
        if low not in ("dive",):
            cut = min([raw.find(c) for c in "0123ijxyzt" if raw.find(c) > 0] + [len(raw)])
            low = raw[:cut].lower()
        if low not in _FIELDS and low not in _MOMENTS and low != "dive":
            raise ValueError(f"unsupported output field {self.name_in!r}")
        self.kind = low
        if low in _MOMENTS:
            parts = self.name_in.split("_")[1:]
            self.species = [int(s) for s in parts]
        if low in _FIELDS or low == "v":
            self.comp = [(1,), (2,), (3,)]
        elif low == "t":
            self.comp = _components(list(self.name_in.split("_")[0][1:3]))
            if len(self.comp) not in (1, 3):
                raise ValueError("Wrong # of components requested for T output")

    def is_moment(self):
        return self.kind in _MOMENTS

    def _suffix(self):
        return "_" + "_".join(str(s) for s in self.species) if self.species else ""

    def name(self):
        """OutputField::name() for scalars."""
        if self.kind == "t":
            base = "T" + self.name_in.split("_")[0][1:3]
        elif self.kind in _FIELDS:
            base = _FIELDS[self.kind] + "i"
        elif self.kind == "v":
            base = "Vi"
        else:
            base = _CASE[self.kind]
        return "f" + base + self._suffix()

    def names(self):
        """OutputField::name(ci) for every component of a vector quantity."""
        head = _FIELDS.get(self.kind) or _CASE[self.kind]
        return ["f" + head + "".join(str(c) for c in cs) + self._suffix() for cs in self.comp]


class OutputWriter:
    """Writes fields and particles of one SR Cartesian domain.

    ctx: sim.Context of the grid; x_min: physical coordinates of the first
    active cell's corner; dx: cell size; n0: scales.n0; dwn: downsampling per
    axis (output.fields.downsampling); smooth_order / smooth_method:
    output.fields.smoothing; prtl_stride: output.particles.stride; species:
    indices written as particles (output.particles.species, 1-based)."""

    def __init__(self, ctx, g: GridSpec, root, *, fields=("E", "B", "J"), x_min=(0.0, 0.0, 0.0),
                 dx=1.0, n0=1.0, dwn=(1, 1, 1), smooth_order=0, smooth_method="spline",
                 use_weights=False, prtl_stride=100, species=(), as_is=False):
        self.ctx, self.g, self.root = ctx, g, root
        self.fields = [OutputField(f) for f in fields]
        self.x_min = tuple(float(v) for v in x_min)
        self.dx, self.n0 = float(dx), float(n0)
        self.dwn = tuple(int(d) for d in (list(dwn) + [1, 1, 1])[:3])
        self.smooth_order = int(smooth_order)
        m = smooth_method.lower()
        if m not in ("spline", "const"):
            raise ValueError("smoothing method must be spline or const")
        self.smoothing = abi.PIC_SMOOTH_SPLINE if m == "spline" else abi.PIC_SMOOTH_CONST
        self.use_weights = bool(use_weights)
        self.prtl_stride = int(prtl_stride)
        self.species_out = list(species)
        self.as_is = bool(as_is)
        N1, N2, N3 = g.ext
        self.bckp = torch.zeros((6, N3, N2, N1), dtype=g.real, device="cuda")
        os.makedirs(root, exist_ok=True)

    def out_shape(self):
        o = [math.ceil(self.g.n[d] / self.dwn[d]) for d in range(self.g.dim)]
        return tuple(reversed(o))

    def mesh(self):
        """X_d (cell centres) and X_de (edges) of GenerateMesh
        (metadomain_io.cpp:419-453) in real_t, first cell 0."""
        out = {}
        R = self.g.real
        for d in range(self.g.dim):
            n_dwn = math.ceil(self.g.n[d] / self.dwn[d])
            i = torch.arange(n_dwn, dtype=R) * self.dwn[d]
            dx = torch.tensor(self.dx, dtype=R)
            x0 = torch.tensor(self.x_min[d], dtype=R)
            xc = (i + 0.5) * dx + x0
            xe = torch.cat([i, i[-1:] + 1]) * dx + x0
            out[f"X{d + 1}"] = xc.numpy()
            out[f"X{d + 1}e"] = xe.numpy()
        return out

    def _params(self, mid, c1=0, c2=0):
        p = abi.PicMomentParams()
        p.id, p.c1, p.c2 = mid, c1, c2
        p.order, p.smoothing, p.use_weights = self.smooth_order, self.smoothing, int(self.use_weights)
        p.inv_n0 = float(torch.tensor(1.0, dtype=self.g.real) / torch.tensor(self.n0, dtype=self.g.real))
        p.dx = self.dx
        return p

    def _moment(self, fld, species, mid, comp, c1=0, c2=0):
        sel = [s for s in species if s.index in fld.species] if fld.species else \
              [s for s in species if s.mass > 0]
        self.ctx.output_moment(sel, self._params(mid, c1, c2), self.bckp, comp)

    def _packed(self, src, is_em, c0, ncomp, flags):
        out = torch.empty((ncomp,) + self.out_shape(), dtype=self.g.real, device="cuda")
        self.ctx.output_field(src, is_em, c0, ncomp, flags, self.dx, self.dwn, out)
        return out

    def field_arrays(self, species, EB, J):
        """{name: device tensor} for the requested fields (the ghosts of EB
        and J must be filled)."""
        res = {}
        for f in self.fields:
            self.bckp.zero_()
            if f.kind in _FIELDS:
                is_em = f.kind != "j"
                c0 = 3 if f.kind == "b" else 0
                src = J if f.kind == "j" else EB
                if self.as_is:
                    flags = 0
                else:
                    flags = abi.PIC_OUT_TO_HAT | (abi.PIC_OUT_INTERP_FACES if f.kind == "b"
                                                  else abi.PIC_OUT_INTERP_EDGES)
                arr = self._packed(src, is_em, c0, 3, flags)
                for k, nm in enumerate(f.names()):
                    res[nm] = arr[k]
            elif f.kind == "dive":
                self.ctx.output_divergence(EB, self.bckp, 0)
                self.ctx.sync_moments(self.bckp, 0, 1)
                res[f.name()] = self._packed(self.bckp, True, 0, 1, 0)[0]
            elif len(f.comp) == 0 or (f.kind == "t" and len(f.comp) == 1):
                mid = _MOMENTS[f.kind]
                cs = f.comp[0] if f.comp else (0, 0)
                self._moment(f, species, mid, 0, cs[0], cs[1] if len(cs) > 1 else 0)
                self.ctx.sync_moments(self.bckp, 0, 1)
                res[f.name()] = self._packed(self.bckp, True, 0, 1, 0)[0]
            else:
                mid = _MOMENTS[f.kind]
                for k, cs in enumerate(f.comp):
                    self._moment(f, species, mid, 3 + k, cs[0], cs[1] if len(cs) > 1 else 0)
                self.ctx.sync_moments(self.bckp, 3, 6)
                if f.kind == "v":
                    self._moment(f, species, abi.PIC_MOM_RHO, 0)
                    self.ctx.sync_moments(self.bckp, 0, 1)
                    self.ctx.normalize_by_rho(self.bckp, 0, (3, 4, 5))
                arr = self._packed(self.bckp, True, 3, 3, 0)
                for k, nm in enumerate(f.names()):
                    res[nm] = arr[k]
        return res

    def particle_arrays(self, species):
        res = {}
        R = self.g.real
        for sp in species:
            if sp.index not in self.species_out:
                continue
            n = sp.npart // self.prtl_stride
            x = [torch.empty(max(n, 1), dtype=R, device="cuda") for _ in range(self.g.dim)]
            u = [torch.empty(max(n, 1), dtype=R, device="cuda") for _ in range(3)]
            w = torch.empty(max(n, 1), dtype=R, device="cuda")
            nout = self.ctx.output_particles(sp, self.prtl_stride, self.dx, self.x_min, x, u, w)
            for d in range(self.g.dim):
                res[f"pX{d + 1}_{sp.index}"] = x[d][:nout]
            for d in range(3):
                res[f"pU{d + 1}_{sp.index}"] = u[d][:nout]
            res[f"pW_{sp.index}"] = w[:nout]
        return res

    def write(self, step, time, species, EB, J, *, fields=True, particles=True):
        """Writes <root>/output.<step:08d>.npz and returns its path."""
        arrays = {}
        if fields:
            arrays.update(self.field_arrays(species, EB, J))
        if particles and self.species_out:
            arrays.update(self.particle_arrays(species))
        torch.cuda.synchronize()
        host = {k: v.cpu().numpy() for k, v in arrays.items()}
        if fields:
            host.update(self.mesh())
        host["Step"] = np.array(step, dtype=np.uint64)
        host["Time"] = np.array(time, dtype=np.float64)
        path = os.path.join(self.root, f"output.{int(step):08d}.npz")
        np.savez(path, **host)
        return path


def write_checkpoint(path, dim, step, time, species, EB, em0=None):
    """Metadomain::WriteCheckpoint (src/framework/domain/metadomain_chckpt.cpp:
    103-160) for one domain: EB (and em0 when given) and every species'
    arrays under the reference's checkpoint names (s<k>_npart, s<k>_i1,
    s<k>_dx1, s<k>_i1_prev, s<k>_dx1_prev, s<k>_ux1, s<k>_tag, s<k>_weight;
    src/framework/containers/particles_io.cpp:360-410), plus Step and Time."""
    a = {"Step": np.array(step, dtype=np.uint64), "Time": np.array(time, dtype=np.float64),
         "em": EB.detach().cpu().numpy()}
    if em0 is not None:
        a["em0"] = em0.detach().cpu().numpy()
    for sp in species:
        k, n = sp.index, sp.npart
        a[f"s{k}_npart"] = np.array(n, dtype=np.int64)
        for d in range(dim):
            a[f"s{k}_i{d + 1}"] = sp.i[d][:n].cpu().numpy()
            a[f"s{k}_dx{d + 1}"] = sp.dx[d][:n].cpu().numpy()
            if sp.i_prev and sp.i_prev[d] is not None:
                a[f"s{k}_i{d + 1}_prev"] = sp.i_prev[d][:n].cpu().numpy()
                a[f"s{k}_dx{d + 1}_prev"] = sp.dx_prev[d][:n].cpu().numpy()
        for d in range(3):
            a[f"s{k}_ux{d + 1}"] = sp.u[d][:n].cpu().numpy()
        a[f"s{k}_tag"] = sp.tag[:n].cpu().numpy()
        a[f"s{k}_weight"] = sp.w[:n].cpu().numpy()
    np.savez(path, **a)
    return path


def read_checkpoint(path, dim, species, EB, em0=None):
    """Restores what write_checkpoint saved into the caller's arrays (same
    field shapes, enough particle capacity); returns (step, time)."""
    z = np.load(path)
    EB.copy_(torch.from_numpy(z["em"]).to(EB.device))
    if em0 is not None and "em0" in z:
        em0.copy_(torch.from_numpy(z["em0"]).to(em0.device))
    for sp in species:
        k = sp.index
        n = int(z[f"s{k}_npart"])
        if n > sp.tag.numel():
            raise ValueError(f"species {k}: checkpoint holds {n} particles, "
                             f"capacity {sp.tag.numel()}")
        sp.npart = n

        def put(dst, key):
            if dst is not None and key in z.files:
                dst[:n].copy_(torch.from_numpy(z[key]).to(dst.device))

        for d in range(dim):
            put(sp.i[d], f"s{k}_i{d + 1}")
            put(sp.dx[d], f"s{k}_dx{d + 1}")
            if sp.i_prev:
                put(sp.i_prev[d], f"s{k}_i{d + 1}_prev")
                put(sp.dx_prev[d], f"s{k}_dx{d + 1}_prev")
        for d in range(3):
            put(sp.u[d], f"s{k}_ux{d + 1}")
        put(sp.tag, f"s{k}_tag")
        put(sp.w, f"s{k}_weight")
    return int(z["Step"]), float(z["Time"])
