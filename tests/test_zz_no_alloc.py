"""ggem_local_matvec_noalloc, the entry point for callers that cannot
allocate device memory (a caching pool holds it all, or allocation is not
allowed where they run), checked through the C ABI against the context
entry point ggem_local_matvec_dev on the same inputs.

The file name sorts last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import ggem_gb300 as G
from ggem_gb300 import build as B

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12  # the tolerance of the FP64 parity tests


def _noalloc_fn():
    L = G.lib()
    fn = L.ggem_local_matvec_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(G.Params), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_matches_context_matvec_on_two_calls_in_a_row():
    import torch

    B.build()
    fn = _noalloc_fn()
    xyz, L = G.make_suspension(77, 3000, 0.1)
    p = G.default_params()
    for d in range(3):
        p.box_lo[d], p.box_hi[d], p.periodic[d] = 0.0, L, 1
    p.nb_mode, p.rc, p.precision = G.NB_CUTOFF, 7.0, G.FP64
    d_xyz = torch.from_numpy(xyz.reshape(-1)).cuda()
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(5)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles_dev(d_xyz.data_ptr(), len(xyz))
        ctx.build_cells()
        for call in range(2):
            f = torch.from_numpy(rng.standard_normal(3 * len(xyz))).cuda()
            want = torch.empty_like(f)
            got = torch.full_like(f, float("nan"))
            ctx.local_matvec_dev(f.data_ptr(), want.data_ptr(), 1, G.SELF_BEAD)
            ctx.synchronize()
            torch.cuda.synchronize()
            rc = fn(C.byref(p), len(xyz), d_xyz.data_ptr(), f.data_ptr(), got.data_ptr(),
                    G.SELF_BEAD, status.data_ptr(), None)
            assert rc == 0
            torch.cuda.synchronize()
            assert int(status.item()) == 0
            err = float(torch.linalg.norm(got - want) / torch.linalg.norm(want))
            assert err <= FP64_TOL, (call, err)


def test_noalloc_rejects_sizes_beyond_its_limit():
    fn = _noalloc_fn()
    p = G.default_params()
    for d in range(3):
        p.box_hi[d] = 500.0
    p.nb_mode, p.rc = G.NB_CUTOFF, 7.0
    # more particles than GGEM_NOALLOC_MAX_PARTICLES: refused before any launch
    assert fn(C.byref(p), 32769, 1, 1, 1, G.SELF_BEAD, 1, None) == G.ERR_BAD_ARG
    # 71^3 cells of side >= rc exceed GGEM_NOALLOC_MAX_CELLS
    assert fn(C.byref(p), 10, 1, 1, 1, G.SELF_BEAD, 1, None) == G.ERR_BAD_ARG


def test_noalloc_status_bits_then_a_clean_call():
    """A bead beyond the box on a non-periodic axis sets status bit 1, a NaN
    coordinate bit 2 (the context path's GGEM_ERR_OUT_OF_DOMAIN and its
    non-finite GGEM_ERR_BAD_ARG); the next call on valid input clears the
    status and matches the context entry point."""
    import torch

    B.build()
    fn = _noalloc_fn()
    rng = np.random.default_rng(9)
    Lx = 30.0
    xyz = rng.uniform(0.5, Lx - 0.5, (400, 3))
    p = G.default_params()
    for d in range(3):
        p.box_lo[d], p.box_hi[d], p.periodic[d] = 0.0, Lx, 1
    p.periodic[2] = 0
    p.nb_mode, p.rc, p.precision = G.NB_CUTOFF, 7.0, G.FP64
    f = torch.from_numpy(rng.standard_normal(3 * len(xyz))).cuda()
    u = torch.empty_like(f)
    status = torch.full((1,), -7, dtype=torch.int32, device="cuda")

    def call(x):
        d_x = torch.from_numpy(np.ascontiguousarray(x).reshape(-1)).cuda()
        rc = fn(C.byref(p), len(x), d_x.data_ptr(), f.data_ptr(), u.data_ptr(), G.SELF_BEAD,
                status.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        return int(status.item())

    out = xyz.copy()
    out[17, 2] = Lx + 3.0  # beyond the open z faces
    assert call(out) == 1
    bad = xyz.copy()
    bad[5, 0] = np.nan
    assert call(bad) == 2
    both = out.copy()
    both[5, 1] = np.inf
    assert call(both) == 3
    # beads on the periodic upper faces' rounding edge stay in the box
    edge = xyz.copy()
    edge[0, 0] = np.nextafter(Lx, 0.0)
    edge[1, 1] = np.nextafter(Lx, 0.0)
    assert call(edge) == 0
    got = u.clone()
    with G.Context(box_hi=(Lx,) * 3, periodic=(1, 1, 0), rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles(edge)
        ctx.build_cells()
        want = ctx.local_matvec(f.cpu().numpy().reshape(len(edge), 3), G.SELF_BEAD)
    err = np.linalg.norm(got.cpu().numpy() - want.reshape(-1)) / np.linalg.norm(want)
    assert err <= FP64_TOL
