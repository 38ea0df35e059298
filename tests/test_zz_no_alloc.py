"""The allocation-free free-surface solve, sgpu_cgsolve_noalloc.

It serves callers that cannot call cudaMalloc: a host program whose device
memory belongs entirely to its own pool allocator, or a time-critical loop that
cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.  Such a
caller passes device buffers it owns (here torch tensors stand in for them) and
the solver's scratch comes from a fixed static array inside the library.

The test calls the entry point through the C ABI twice in a row on the same
inputs and compares each result with the allocating entry point sgpu_cgsolve
and with the reference's own solutions on one of its example grids, within the
parity tolerance of the other GPU tests (relative L2 <= 1e-9), and checks that
a grid beyond the stated capacity is refused with SGPU_TOO_LARGE.
The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from suntans_gb300 import gridgen as gg
from suntans_gb300.capi import OK, TOO_LARGE, Context, NoallocGrid, Stats, load, props_struct
from tests._cases import h_props, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _noalloc_call(lib, g, hp, props, torch):
    keep = {k: _dev(getattr(g, k), torch) for k in ("cellp", "nfaces", "neigh", "face", "Ac", "df", "dg")}
    ng = NoallocGrid(g.Nc, g.Ne, g.maxfaces, int(g.celldist[1]),
                     *[keep[k].data_ptr() for k in ("cellp", "nfaces", "neigh", "face", "Ac", "df", "dg")])
    D = _dev(hp.D, torch)
    h = _dev(hp.h, torch)
    htmp = _dev(hp.htmp, torch)
    st = Stats()
    pr = props_struct(props)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    rc = lib.sgpu_cgsolve_noalloc(C.byref(ng), D.data_ptr(), h.data_ptr(), htmp.data_ptr(), C.byref(pr),
                                  C.byref(st), stream)
    return rc, h.cpu().numpy(), st


@pytest.mark.parametrize("hprecond", [1, 0])
def test_noalloc_matches_allocating_solve_twice(gpu_lib, hprecond):
    torch = pytest.importorskip("torch")
    lib = load()
    g = gg.delaunay_seamount(600, 2000, 1000, Nkmax=15, sigma=300, ctop_frac=0.2, h_sigma=0.05, open_x0=True,
                             seed=5)
    hp = gg.make_h_problem(g, seed=2)
    props = h_props(hprecond)
    ctx = Context(g)
    h_ref, st_ref = ctx.cgsolve(hp, props)
    ctx.close()
    comp = g.comp_cells()
    bdy = g.cellp[g.celldist[1]:g.celldist[2]]
    for _ in range(2):
        rc, h, st = _noalloc_call(lib, g, hp, props, torch)
        assert rc == OK and st.status == OK
        assert abs(st.niters - st_ref.niters) <= 2
        assert rel_l2(h[comp], h_ref[comp]) <= TOL
        assert np.array_equal(h[bdy], hp.h[bdy])


def test_noalloc_matches_reference_on_example_grid(gpu_lib):
    """Against the reference's own CGSolve solutions stored with the riverplume
    hexagon grid (cells of 5-7 faces), two calls in a row, both hprecond modes."""
    torch = pytest.importorskip("torch")
    from tests._golden import load_example, props_for
    lib = load()
    g, qp, hp, props, d = load_example("riverplume_hex")
    comp = g.cellp[g.celldist[0]:g.celldist[1]]
    for hpc in (0, 1):
        ref = d[f"h_hp{hpc}"]
        for _ in range(2):
            rc, h, st = _noalloc_call(lib, g, hp, props_for(props, hprecond=hpc), torch)
            assert rc == OK and st.status == OK
            assert rel_l2(h[comp], ref[comp]) <= TOL


def test_noalloc_refuses_too_large(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = load()
    # 524,288 triangles need 8*(5+3)*Nc + 33,280 bytes > 32 MiB; sizes only: no data is read
    Nc = 524_288
    ng = NoallocGrid(Nc, Nc * 2, 3, Nc, *([1] * 7))
    st = Stats()
    pr = props_struct(h_props(1))
    rc = lib.sgpu_cgsolve_noalloc(C.byref(ng), 8, 8, 8, C.byref(pr), C.byref(st), 0)
    assert rc == TOO_LARGE
