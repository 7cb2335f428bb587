"""The element spread (every quadrature point of every element, reference
mode) through the C ABI against the FP64 oracle's per-point spread over
the element neighbour lists (assemble_stokes.C:645-662 with
ggem_stokes.C:117-128).

Tolerances: FP64 within 1e-12 (norm-wise); the FP32 path's error is
printed per component and bounded at 1e-6 norm-wise and 1e-5 of the
largest component.
"""
import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
ALPHA = 0.5


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def gauss_points(lo, L, nm):
    """2 x 2 x 2 Gauss points of every element of an nm[0] x nm[1] x nm[2]
    mesh (x fastest), element-major"""
    lo, L, nm = np.asarray(lo, float), np.asarray(L, float), np.asarray(nm)
    h = L / nm
    g = np.array([0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)])
    loc = np.array([[g[a], g[b], g[c]] for c in range(2) for b in range(2) for a in range(2)])
    ez, ey, ex = np.meshgrid(np.arange(nm[2]), np.arange(nm[1]), np.arange(nm[0]), indexing="ij")
    base = np.stack([ex.ravel(), ey.ravel(), ez.ravel()], axis=1)
    q = (base[:, None, :] + loc[None, :, :]) * h + lo
    return q.reshape(-1, 3), len(loc)


def _check(lo, L, nm, periodic, xyz, seed):
    lo, L = np.asarray(lo, float), np.asarray(L, float)
    hi = lo + L
    h = L / np.asarray(nm)
    sre = 0.5 * h.max() + 4.0 / ALPHA + 1e-3
    box = O.make_box(lo, hi, periodic)
    mesh = O.make_mesh(*nm, sre)
    c = O.constants(alpha=ALPHA)
    enb, _ = O.elem_lists(box, mesh, xyz)
    q, nq = gauss_points(lo, L, nm)
    qe = np.repeat(np.arange(int(np.prod(nm))), nq).astype(np.int32)
    f = np.random.default_rng(seed).standard_normal((len(xyz), 3))
    want = O.spread_qp(c, box, enb, xyz, f, q, qe)
    out = {}
    with G.Context(alpha=ALPHA, box_lo=tuple(lo), box_hi=tuple(hi), periodic=periodic,
                   nb_mode=G.NB_REFERENCE, n_mesh=tuple(nm), search_radius_e=sre,
                   precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        ctx.set_quadrature(q, nq)
        for prec in (G.FP64, G.FP32):
            out[prec] = ctx.spread_elements(f, prec)
            again = ctx.spread_elements(f, prec)
            assert np.array_equal(out[prec], again)  # no state carried between calls
    e64 = rel(out[G.FP64], want)
    e32 = rel(out[G.FP32], want)
    comp = np.abs(out[G.FP32] - want).max() / np.abs(want).max()
    print(f"spread nm={nm} n={len(xyz)} periodic={periodic}: FP64 {e64:.2e}, FP32 norm-wise "
          f"{e32:.2e}, max component {comp:.2e} of the largest")
    assert e64 <= FP64_TOL
    assert e32 <= 1e-6 and comp <= 1e-5


def test_spread_small_mesh_whole_axis_stencil():
    """6 elements per axis: the element stencil covers every axis (offsets
    wrap, minimum image inside the brick)"""
    rng = np.random.default_rng(8)
    L = 24.0
    _check((0, 0, 0), (L,) * 3, (6, 6, 6), (1, 1, 1), rng.uniform(0, L, (150, 3)), 1)


def test_spread_fine_mesh_suspension():
    """h = 1.43 (the spread's mesh size), beads at phi = 0.1: bricks whose
    dilated frame wraps the periodic box faces"""
    xyz, L = G.make_suspension(44, 1500, 0.1)
    nm = int(np.floor(L / 1.414))
    _check((0, 0, 0), (L,) * 3, (nm,) * 3, (1, 1, 1), xyz, 2)


def test_spread_open_axis_offset_box():
    """a non-periodic z axis and a box away from the origin"""
    rng = np.random.default_rng(3)
    lo, L, nm = (-11.0, 5.0, 100.0), (36.0, 30.0, 24.0), (24, 20, 16)
    xyz = np.asarray(lo) + rng.uniform(0, 1, (1200, 3)) * np.asarray(L)
    _check(lo, L, nm, (1, 1, 0), xyz, 3)


def test_spread_dense_staging_in_several_passes():
    """more particles in a brick's dilated region than one shared-memory
    pass holds (512 FP32 / 256 FP64 records): the passes add up"""
    rng = np.random.default_rng(4)
    L = 40.0
    xyz = rng.uniform(0, L, (6400, 3))
    _check((0, 0, 0), (L,) * 3, (28, 28, 28), (1, 1, 1), xyz, 4)


def test_spread_wide_stencil_compact_bitmap():
    """elements of h = 0.55 under the spread's search radius (0.5 h + 8):
    offsets up to 15 elements, so the stencil (31 per axis) plus twice the
    2-element brick exceeds 32 and the kernel reads the compact stencil
    bitmap instead of the padded one (an open box, whose frames are clipped
    to the mesh, keeps the case small)"""
    rng = np.random.default_rng(6)
    L = 12 * 0.55
    _check((0, 0, 0), (L,) * 3, (12, 12, 12), (0, 0, 0), rng.uniform(0, L, (60, 3)), 5)
