"""Scenario builders shared by the CPU (oracle) and GPU tests."""
import math

import torch

from entity_gb300.inputs import GridSpec, SpeciesArrays, empty_field


def species_from_lists(g: GridSpec, cells, offsets, u, *, prev_cells=None, prev_offsets=None,
                       tags=None, weights=None, mass=1.0, charge=1.0, pusher=1, pad_to=None):
    """A species from explicit per-particle lists (cells/offsets per axis)."""
    n = len(cells)
    tot = pad_to or n
    R = g.real

    def arr(vals, dtype, fill=0):
        t = torch.full((tot,), fill, dtype=dtype)
        if n:
            t[:n] = torch.tensor(vals, dtype=dtype)
        return t

    i = [arr([c[a] for c in cells], torch.int32) for a in range(g.dim)]
    dx = [arr([o[a] for o in offsets], torch.float32) for a in range(g.dim)]
    if g.dim == 2:
        i.append(torch.zeros(tot, dtype=torch.int32))
        dx.append(torch.zeros(tot, dtype=torch.float32))
    pc = prev_cells or cells
    po = prev_offsets or offsets
    ip = [arr([c[a] for c in pc], torch.int32) for a in range(g.dim)]
    dp = [arr([o[a] for o in po], torch.float32) for a in range(g.dim)]
    if g.dim == 2:
        ip.append(torch.zeros(tot, dtype=torch.int32))
        dp.append(torch.zeros(tot, dtype=torch.float32))
    uu = [arr([x[a] for x in u], R) for a in range(3)]
    w = arr(weights if weights is not None else [1.0] * n, R)
    tg = arr(tags if tags is not None else [1] * n, torch.int16)
    return SpeciesArrays(i, dx, ip, dp, uu, w, tg, mass, charge, pusher, tot, 1)


def random_fields(g: GridSpec, seed: int, amp=0.3, device="cpu"):
    gen = torch.Generator()
    gen.manual_seed(seed)
    EB = empty_field(g, 6)
    EB.copy_((torch.rand(EB.shape, generator=gen, dtype=torch.float64) * 2 - 1).to(g.real) * amp)
    return EB.to(device)


def random_currents(g: GridSpec, seed: int, device="cpu"):
    gen = torch.Generator()
    gen.manual_seed(seed)
    J = empty_field(g, 3)
    J.copy_((torch.rand(J.shape, generator=gen, dtype=torch.float64) * 2 - 1).to(g.real))
    return J.to(device)


def staggered_coords(g: GridSpec, shift):
    """Code coordinates (ghost-shifted) of every ghost-inclusive index with a
    half-cell `shift` per axis; returns (X1, X2, X3) of shape (N3, N2, N1)."""
    N1, N2, N3 = g.ext
    x1 = torch.arange(N1, dtype=torch.float64) - g.ng + shift[0]
    x2 = torch.arange(N2, dtype=torch.float64) - g.ng + shift[1]
    if g.dim == 3:
        x3 = torch.arange(N3, dtype=torch.float64) - g.ng + shift[2]
    else:
        x3 = torch.zeros(1, dtype=torch.float64)
    X3, X2, X1 = torch.meshgrid(x3, x2, x1, indexing="ij")
    return X1, X2, X3


def active(g: GridSpec, f):
    """View of the active cells of a (ncomp, N3, N2, N1) field."""
    ng = g.ng
    if g.dim == 2:
        return f[:, :, ng:-ng, ng:-ng]
    return f[:, ng:-ng, ng:-ng, ng:-ng]


def make_plasma(g: GridSpec, ppc, temp, seed, *, beta=0.0, charge=-1.0, mass=1.0, pusher=1,
                index=1, shuffle=True):
    from entity_gb300.inputs import make_species
    return make_species(g, ppc, temp, beta, seed, mass=mass, charge=charge, pusher=pusher,
                        index=index, shuffle=shuffle)


def copy_species(sp: SpeciesArrays, device):
    return sp.clone().to(device) if device != "cpu" else sp.clone()


def tensors_equal(a, b):
    return bool(torch.equal(a.cpu(), b.cpu()))


def max_rel(a, b):
    a = a.double().cpu()
    b = b.double().cpu()
    scale = max(float(b.abs().max()), 1e-300)
    return float((a - b).abs().max()) / scale


TWO_PI = 2.0 * math.pi
