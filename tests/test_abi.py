"""The C-ABI library builds, loads without a GPU, and exports every function
declared in include/*.h (no compute calls: this runs on CPU-only hosts)."""
import glob
import os
import re

from suntans_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:int|void|char|long long|double)\s*\*?\s*(sgpu_\w+)\s*\(", src,
                             flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    build.build()
    lib = capi.load()
    decl = declared_functions()
    assert decl, "no declarations found"
    missing = [n for n in sorted(decl) if not hasattr(lib, n)]
    assert not missing, missing
    assert decl == set(capi.EXPORTS), decl ^ set(capi.EXPORTS)


def test_create_without_device_reports_no_device():
    """On a host without a GPU the library refuses with SGPU_NO_DEVICE (no CPU fallback)."""
    import ctypes as C
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    from suntans_gb300 import gridgen as gg
    g = gg.quad_channel(4, 3, Nkmax=3)
    lib = capi.load()
    arrs = [g.nfaces, g.neigh, g.face, g.Nk, g.Nke, g.cellp, g.celldist, g.Ac, g.df, g.dg]
    d = capi.GridDesc(g.Nc, g.Ne, g.maxfaces, g.Nkmax, *[a.ctypes.data_as(capi._ip) for a in arrs[:7]],
                      *[a.ctypes.data_as(capi._dp) for a in arrs[7:]])
    h = C.c_void_p()
    assert lib.sgpu_create(C.byref(d), 0, C.byref(h)) == capi.NO_DEVICE


def test_status_strings():
    lib = capi.load()
    for code in range(10):
        assert lib.sgpu_status_string(code)
