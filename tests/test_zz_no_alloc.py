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
