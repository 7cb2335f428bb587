"""Degenerate inputs through the C ABI, against the FP64 oracle: a context
without particles, a single bead (the self term alone, whose mobility is a
multiple of the identity), and coincident and near-coincident beads (the
reference's r < 1e-6 branch of green_tensor_local_regularized,
ggem_stokes.C:304-357, and the pair list's r = 0 entries)."""
import ctypes as C

import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.parametrize("prec", [G.FP32, G.FP64])
def test_empty_context_then_particles(prec):
    """no particles: the build, the matvec and both series return without
    work (the series reported converged at degree 0), the field at given
    points is zero, Lanczos refuses; the same context then takes particles
    and matches the oracle"""
    L = 30.0
    lib = G.lib()
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
        ctx.set_particles(np.zeros((0, 3)))
        ctx.build_cells()
        if prec == G.FP32:
            assert ctx.pair_count() == 0
        off, ids = ctx.neighbors()
        assert off.tolist() == [0] and len(ids) == 0
        u = ctx.local_matvec(np.zeros((0, 3)))
        assert u.shape == (0, 3)
        reps = (G.ChebReport * 2)()
        rc = lib.ggem_brownian_displacement(ctx.h, 2, 30, 0.5, 2.0, 1e-3, 0, None, None, reps)
        assert rc == 0
        for r in reps:
            assert (r.converged, r.n_terms, r.n_matvecs) == (1, 0, 0)
        reps = (G.ChebReport * 1)()
        rc = lib.ggem_cheb_inv_sqrt(ctx.h, 1, 30, 0.5, 2.0, 1e-3, 1, None, reps)
        assert rc == 0 and reps[0].converged == 1 and reps[0].n_matvecs == 0
        # the Python binding over the same calls
        rc, dw, r = ctx.brownian_displacement(np.zeros((3, 0, 3)), 30, 0.5, 2.0, 1e-3)
        assert rc == 0 and dw.shape == (3, 0, 3) and len(r) == 3 and r[0]["converged"] == 1
        y, r = ctx.cheb_inv_sqrt(np.zeros((0, 3)), 30, 0.5, 2.0, 1e-3)
        assert y.shape == (0, 3) and len(r) == 1 and r[0]["n_matvecs"] == 0
        targets = np.random.default_rng(1).uniform(0, L, (5, 3))
        assert np.array_equal(ctx.local_field(targets, np.zeros((0, 3))), np.zeros((5, 3)))
        with pytest.raises(G.GGEMError):
            ctx.lanczos_bounds(k=8)
        # the same context, now with particles
        xyz = np.random.default_rng(2).uniform(0, L, (200, 3))
        f = np.random.default_rng(3).standard_normal((200, 3))
        ctx.set_particles(xyz)
        ctx.build_cells()
        box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
        nb = O.neighbors_cutoff(box, xyz, 7.0)
        want = O.local_matvec(O.constants(alpha=0.5), box, xyz, nb, f[None], O.SELF_BEAD)
        got = ctx.local_matvec(f, G.SELF_BEAD)
        assert rel(got, want[0]) <= (FP64_TOL if prec == G.FP64 else FP32_TOL)


@pytest.mark.parametrize("prec", [G.FP32, G.FP64])
@pytest.mark.parametrize("check_every", [0, 1])
def test_single_bead(prec, check_every):
    """one bead: M = c I with c the self coefficient, so the Brownian
    displacement is sqrt(c) xi to the series' tolerance"""
    L = 30.0
    xyz = np.array([[3.0, 17.0, 29.5]])
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.array([[0.3, -1.2, 0.7]])
    want = O.local_matvec(O.constants(alpha=0.5), box, xyz, nb, f[None], O.SELF_BEAD)[0]
    c = want[0, 0] / f[0, 0]
    assert np.allclose(want, c * f, rtol=1e-14, atol=0)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.local_matvec(f, G.SELF_BEAD)
        assert rel(got, want) <= (FP64_TOL if prec == G.FP64 else FP32_TOL)
        xi = np.array([[0.9, 0.1, -1.4]])
        rc, dw, reps = ctx.brownian_displacement(xi, 30, c / 1.05, c * 1.05, 1e-3,
                                                 check_every=check_every)
        assert rc == 0 and reps[0]["converged"] == 1, (rc, reps)
        assert rel(dw.reshape(1, 3), np.sqrt(c) * xi) <= 2e-3, (dw, np.sqrt(c) * xi)


@pytest.mark.parametrize("prec", [G.FP32, G.FP64])
def test_coincident_and_near_coincident_beads(prec):
    """two beads at one point (r = 0), two 4e-7 apart (inside the
    reference's r < 1e-6 branch, G = coeff_2 I), a pair across a periodic
    face and a few ordinary ones: lists bit-exact, velocities within the
    precision's tolerance of the oracle"""
    L = 30.0
    xyz = np.array([
        [5.0, 5.0, 5.0], [5.0, 5.0, 5.0],            # coincident
        [12.0, 5.0, 5.0], [12.0 + 4e-7, 5.0, 5.0],   # near-coincident
        [0.5, 10.0, 10.0], [29.7, 10.0, 10.0],       # across the x face
        [20.0, 20.0, 20.0], [24.5, 22.0, 19.0], [8.0, 6.0, 4.0], [15.0, 25.0, 12.0],
    ])
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(5).standard_normal((2, len(xyz), 3))
    want = O.local_matvec(O.constants(alpha=0.5), box, xyz, nb, f, O.SELF_BEAD)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        off, ids = ctx.neighbors()
        assert np.array_equal(off, nb.offsets)
        assert np.array_equal(ids, nb.ids)
        got = ctx.local_matvec(f, G.SELF_BEAD)
        tol = FP64_TOL if prec == G.FP64 else FP32_TOL
        assert rel(got, want) <= tol
        # the coincident pair's velocities: both beads see the same sources
        g2 = ctx.local_matvec(np.ascontiguousarray(f[0]), G.SELF_BEAD)
        w2 = want[0]
        assert rel(g2[:2], w2[:2]) <= tol
        assert rel(g2[2:4], w2[2:4]) <= tol
