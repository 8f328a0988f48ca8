"""pic_field_energy_noalloc, the field energy for callers that cannot
allocate device memory (a framework that reserves all device memory for its
own pool, a hook between steps where cudaMalloc could synchronise the device,
a fixed memory budget). It needs no context and keeps its scratch in a fixed
array inside the library.

Checked through the C ABI against pic_field_energy on two calls in a row
(the second on different fields, so a stale scratch would show), in float
and double, 2D and 3D, and the size limit is enforced. This file is named to
be collected last; it passes alone in a fresh process as well.
"""
import ctypes as C

import pytest
import torch

from entity_gb300 import abi
from entity_gb300.inputs import GridSpec
from entity_gb300.sim import Context, make_grid
from tests.helpers import random_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from entity_gb300 import build
    build.build()
    abi.load()


def _noalloc(g, EB):
    pg = make_grid(g)
    out = (C.c_double * 2)()
    st = abi.load().pic_field_energy_noalloc(C.byref(pg), C.c_void_p(EB.data_ptr()), g.dx, out,
                                              None)
    return st, (out[0], out[1])


@pytest.mark.parametrize("real", [torch.float32, torch.float64])
@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_energy_matches_context_version(dim, real):
    n = (40, 36, 1) if dim == 2 else (24, 20, 16)
    g = GridSpec(dim=dim, n=n, order=2, real=real, extent=2.0 * n[0])
    ctx = Context(g)
    for call, seed in enumerate((101, 202)):      # two calls in a row
        EB = random_fields(g, seed, amp=0.5 + call).cuda()
        st, got = _noalloc(g, EB)
        assert st == abi.PIC_OK, abi.status_string(st)
        ref = ctx.field_energy(EB, g.dx)
        assert got[0] == pytest.approx(ref[0], rel=1e-12)
        assert got[1] == pytest.approx(ref[1], rel=1e-12)
    ctx.close()


def test_noalloc_energy_is_reproducible():
    g = GridSpec(dim=3, n=(32, 32, 32), order=2, real=torch.float32)
    EB = random_fields(g, 7).cuda()
    st1, a = _noalloc(g, EB)
    st2, b = _noalloc(g, EB)
    assert st1 == st2 == abi.PIC_OK
    assert a == b                                 # fixed summation order


def test_noalloc_energy_rejects_grids_beyond_its_scratch():
    g = GridSpec(dim=3, n=(8, 512, 129), order=1, real=torch.float32)   # 66048 rows
    pg = make_grid(g)
    out = (C.c_double * 2)()
    EB = torch.zeros(16, device="cuda")           # never read: the size check comes first
    st = abi.load().pic_field_energy_noalloc(C.byref(pg), C.c_void_p(EB.data_ptr()), 1.0, out,
                                              None)
    assert st == abi.PIC_ERR_UNSUPPORTED
