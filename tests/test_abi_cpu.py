"""CPU-side checks of the C ABI: the library builds and loads, exports every
function include/*.h declares, and rejects invalid arguments on the host
before touching the device."""
import ctypes as C
import glob
import os
import re

import pytest

from entity_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(pic_[a-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from entity_gb300 import build
    build.build()
    return abi.load()


def test_header_declares_entry_points():
    names = _declared_functions()
    assert {"pic_create", "pic_push_deposit", "pic_sort", "pic_faraday"} <= names


def test_library_exports_every_declared_symbol(lib):
    for name in sorted(_declared_functions()):
        assert hasattr(lib, name), name


def test_binding_covers_header(lib):
    assert _declared_functions() <= set(abi.SIGNATURES)


def test_version(lib):
    v, sm = C.c_int32(), C.c_int32()
    assert lib.pic_version(C.byref(v), C.byref(sm)) == abi.PIC_OK
    assert v.value == 1 and sm.value == 103


def _grid(**kw):
    g = abi.PicGrid()
    g.dim = kw.get("dim", 3)
    n = kw.get("n", (16, 16, 16))
    for d in range(3):
        g.n[d] = n[d]
        g.fld_periodic[d] = 1
    g.ng = kw.get("ng", 2)
    g.order = kw.get("order", 2)
    g.real_bytes = kw.get("real_bytes", 4)
    N1, N2, N3 = n[0] + 2 * g.ng, n[1] + 2 * g.ng, (n[2] + 2 * g.ng if g.dim == 3 else 1)
    s = (1, N1, N1 * N2, N1 * N2 * N3)
    for k in range(4):
        g.em_stride[k] = s[k]
        g.cur_stride[k] = s[k]
    return g


@pytest.mark.parametrize("bad,expect", [
    (dict(dim=4), abi.PIC_ERR_UNSUPPORTED),
    (dict(order=5), abi.PIC_ERR_UNSUPPORTED),
    (dict(real_bytes=2), abi.PIC_ERR_UNSUPPORTED),
    (dict(order=3, ng=2), abi.PIC_ERR_ARG),          # N_GHOSTS = 3 at order 3
    (dict(n=(3, 16, 16)), abi.PIC_ERR_ARG),           # fewer cells than 2 ghost layers
    (dict(dim=2, n=(16, 16, 4)), abi.PIC_ERR_ARG),    # 2D needs n3 = 1
])
def test_create_rejects_invalid_grids(lib, bad, expect):
    g = _grid(**bad)
    h = C.c_void_p()
    assert lib.pic_create(C.byref(g), C.byref(h)) == expect
    assert not h.value


def test_null_arguments_rejected_without_device(lib):
    assert lib.pic_create(None, None) == abi.PIC_ERR_ARG
    assert lib.pic_destroy(None) == abi.PIC_ERR_ARG
    assert lib.pic_faraday(None, None, 1.0, 1.0, None, None) == abi.PIC_ERR_ARG
    assert lib.pic_push_deposit(None, None, 0, None, None, 1.0, 1.0, 1.0, 0, None) == abi.PIC_ERR_ARG
    assert lib.pic_sort(None, None, 0, None, None) == abi.PIC_ERR_ARG
    assert lib.pic_status_string(abi.PIC_ERR_DEVICE) == b"device-side check failed"


def test_product_library_does_not_link_the_oracle(lib):
    # the checker is never part of the shipped path
    maps = open(f"/proc/{os.getpid()}/maps").read()
    so = [l.split()[-1] for l in maps.splitlines() if "libentity_pic" in l]
    assert so, "library not mapped"
    import subprocess
    out = subprocess.run(["ldd", so[0]], capture_output=True, text=True).stdout
    assert "oracle" not in out


STRUCTS = {"pic_grid": "PicGrid", "pic_species": "PicSpecies",
           "pic_species_adjoint": "PicSpeciesAdjoint", "pic_gr_metric": "PicGRMetric",
           "pic_inject_params": "PicInjectParams", "pic_moment_params": "PicMomentParams",
           "pic_field_bcs": "PicFieldBCs", "pic_gr_params": "PicGRParams",
           "pic_step_params": "PicStepParams"}


def test_binding_structs_match_header_layout(tmp_path):
    """Every ctypes structure has the size and the field offsets the C
    compiler gives the header's struct (gcc on this host)."""
    import shutil
    import subprocess
    from entity_gb300 import abi
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "entity_pic.h"',
             "int main(void) {"]
    expect = []
    for cname, pyname in STRUCTS.items():
        cls = getattr(abi, pyname)
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(cls))
        for f in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {f[0]}));')
            expect.append(getattr(cls, f[0]).offset)
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.check_call(["gcc", "-std=c11", "-I", inc, str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got == expect
