"""Parity of the CUDA library (through the C ABI) with the FP64 oracle.

Tolerances (spec contract):
  * neighbour and cell lists: bit-exact as sorted index sets;
  * FP64 results: 1e-12 relative (norm-wise);
  * FP32 pair sum: 1e-6 relative velocity error (norm-wise), the per-component
    error is reported against the largest component;
  * Chebyshev: reference-faithful mode reproduces the oracle's terms and
    stopping decisions on the same xi.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"

FP64_TOL = 1e-12
FP32_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def suspension(n, phi, seed):
    xyz, L = G.make_suspension(seed, n, phi)
    return xyz, L


def test_golden_velocity_profile_local_field():
    """The reference's PointParticle_Stokes_GGEM golden profiles through
    ggem_local_field (cut-off at search_radius_p = 4/alpha, copss.C:1074)."""
    g = json.loads((GOLD / "ggem_profile_3P.json").read_text())
    lo, hi = g["box"]
    with G.Context(alpha=g["alpha"], box_lo=(lo,) * 3, box_hi=(hi,) * 3, periodic=(0, 0, 0),
                   rc=4.0 / g["alpha"], precision=G.FP64) as ctx:
        ctx.set_particles(np.array(g["beads"]))
        ctx.build_cells()
        f = np.array([g["force"]] * 3)
        tol = 0.5 * 10.0 ** (-g["print_decimals"]) + 1e-12
        for ax, name in enumerate("xyz"):
            A = g["axes"][name]
            pts = np.zeros((len(A["coord"]), 3))
            pts[:, ax] = A["coord"]
            u = ctx.local_field(pts, f)
            assert np.abs(u - np.array(A["local"])).max() <= tol


def test_constants_and_green_tensor_match_oracle():
    with G.Context(alpha=0.5, box_hi=(30.0,) * 3, precision=G.FP64) as ctx:
        k = ctx.constants()
        c = O.constants(alpha=0.5)
        for name in ("ksi", "coeff_1", "coeff_2", "one_eight_pi_mu", "alpha3_pi_23"):
            assert getattr(k, name) == getattr(c, name)
        rng = np.random.default_rng(0)
        x = rng.normal(size=(200, 3)) * 3
        x[0] = 0.0
        x[1] = [1e-7, 0, 0]
        Gd = ctx.green_tensor_local(x)
        Go = np.array([O.green_local(c, v) for v in x])
        assert np.abs(Gd - Go).max() <= 1e-14 * np.abs(Go).max()


@pytest.mark.parametrize("prec", [G.FP64, G.FP32])
@pytest.mark.parametrize("cell_div", [1, 2])
def test_cutoff_neighbor_lists_bit_exact(prec, cell_div):
    if prec == G.FP64 and cell_div == 2:
        pytest.skip("FP64 sweeps rc-sized cells")
    xyz, L = suspension(3000, 0.1, 11)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec, cell_div=cell_div) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        off, ids = ctx.neighbors()
        want = O.neighbors_cutoff(O.make_box([0] * 3, [L] * 3, [1, 1, 1]), xyz, 7.0)
        assert np.array_equal(off, want.offsets)
        assert np.array_equal(ids, want.ids)
        assert ctx.pair_count() == want.offsets[-1]


@pytest.mark.parametrize("n", [1500, 5000])
def test_crowded_cells_lists_bit_exact_over_rebuilds(n):
    """Cells of ~55 particles (ranked in registers, two chunks) and of ~185
    (the in-place path): the cell order, the neighbour lists and the matvec
    are the oracle's, and stay so over rebuilds that reuse the zeroed cell
    counters, across a particle-count change and back."""
    rng = np.random.default_rng(n)
    L = 21.0  # three cells of side 7 per axis
    xyz = rng.uniform(0, L, (n, 3))
    other = rng.uniform(0, L, (n // 3, 3))
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    want = O.neighbors_cutoff(box, xyz, 7.0)
    cells = np.minimum(np.floor(xyz / 7.0).astype(int), 2)
    cell_want = cells[:, 0] + 3 * (cells[:, 1] + 3 * cells[:, 2])
    for prec in (G.FP64, G.FP32):
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
            for cfg in (xyz, xyz, other, xyz):
                ctx.set_particles(cfg)
                ctx.build_cells()
                if cfg is other:
                    continue
                assert np.array_equal(ctx.cell_of_particles(), cell_want)
                off, ids = ctx.neighbors()
                assert np.array_equal(off, want.offsets) and np.array_equal(ids, want.ids)


def test_cutoff_lists_with_boundary_pairs_bit_exact():
    """Pairs placed at |r| = rc within rounding: the FP32 filter must defer
    to the exact FP64 predicate."""
    rng = np.random.default_rng(5)
    L = 40.0
    base = rng.uniform(0, L, (400, 3))
    d = rng.normal(size=(400, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    eps = rng.choice([-1, 0, 1], size=(400, 1)) * 1e-14
    other = np.mod(base + d * (7.0 + eps), L)
    xyz = np.concatenate([base, other])
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    want = O.neighbors_cutoff(box, xyz, 7.0)
    for prec in (G.FP64, G.FP32):
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
            ctx.set_particles(xyz)
            ctx.build_cells()
            off, ids = ctx.neighbors()
            assert np.array_equal(off, want.offsets) and np.array_equal(ids, want.ids)


def test_reference_mode_lists_bit_exact():
    xyz, L = suspension(600, 0.05, 3)
    nm = 16
    h = L / nm
    sre = 0.5 * h + 4.0 / 0.5 + 1e-3
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    mesh = O.make_mesh(nm, nm, nm, sre)
    want = O.neighbors_reference(box, mesh, xyz)
    with G.Context(box_hi=(L,) * 3, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                   search_radius_e=sre, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        off, ids = ctx.neighbors()
        wl = [np.sort(x) for x in want.lists()]
        assert np.array_equal(off, np.concatenate([[0], np.cumsum([len(x) for x in wl])]))
        assert np.array_equal(ids, np.concatenate(wl))
        _, eop = O.elem_lists(box, mesh, xyz)
        assert np.array_equal(ctx.cell_of_particles(), eop)


def _face_points(lo, L, nm, seed):
    """Beads on every element face of every axis and 1 and 3 ulps either
    side of it, plus uniform beads, all inside [lo, lo + L)."""
    rng = np.random.default_rng(seed)
    lo, L = np.asarray(lo, float), np.asarray(L, float)
    h = L / nm
    pts = []
    for k in range(nm + 1):
        for d in range(3):
            for s in (-3, -1, 0, 1, 3):
                p = lo + rng.uniform(0.05, 0.95, 3) * L
                x = lo[d] + k * h[d]
                for _ in range(abs(s)):
                    x = np.nextafter(x, np.inf if s > 0 else -np.inf)
                p[d] = x
                pts.append(p)
    pts = np.array(pts)
    pts = pts[np.all((pts >= lo) & (pts < lo + L), axis=1)]
    return np.concatenate([pts, lo + rng.uniform(0, 1, (2000, 3)) * L])


@pytest.mark.parametrize("lo", [(0.0, 0.0, 0.0), (-10.3, 1000.0, 0.1), (-7.0, 3.3, -1e4)])
def test_element_index_at_element_faces_matches_oracle(lo):
    """The cell index takes an FP32 shortcut away from the box and element
    faces; beads on the faces and a few ulps off them, in boxes away from the
    origin, must still land in the oracle's element."""
    nm, L = 16, 21.0
    xyz = _face_points(lo, (L,) * 3, nm, 7)
    hi = tuple(x + L for x in lo)
    box = O.make_box(lo, hi, [1, 1, 1])
    sre = 0.5 * L / nm + 4.0 / 0.5 + 1e-3
    _, eop = O.elem_lists(box, O.make_mesh(nm, nm, nm, sre), xyz)
    with G.Context(box_lo=lo, box_hi=hi, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                   search_radius_e=sre, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        assert np.array_equal(ctx.cell_of_particles(), eop)


@pytest.mark.parametrize("self_mode", [G.SELF_NONE, G.SELF_BEAD, G.SELF_LAGRANGIAN])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_fp64_matvec_cutoff(self_mode, nrhs):
    xyz, L = suspension(2000, 0.1, 21)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(2).standard_normal((nrhs, len(xyz), 3))
    want = O.local_matvec(c, box, xyz, nb, f, self_mode)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.local_matvec(f, self_mode)
    assert rel(got, want) <= FP64_TOL


def test_fp64_matvec_reference_mode_non_periodic_axis():
    rng = np.random.default_rng(4)
    L = np.array([36.0, 36.0, 20.0])
    xyz = rng.uniform(0, 1, (700, 3)) * L
    nm = (12, 12, 7)
    sre = 0.5 * 3.0 + 4.0 / 0.5 + 1e-3
    box = O.make_box([0] * 3, L, [1, 1, 0])
    mesh = O.make_mesh(*nm, sre)
    c = O.constants(alpha=0.5)
    nb = O.neighbors_reference(box, mesh, xyz)
    f = rng.standard_normal((len(xyz), 3))
    want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD)
    with G.Context(box_hi=tuple(L), periodic=(1, 1, 0), nb_mode=G.NB_REFERENCE, n_mesh=nm,
                   search_radius_e=sre, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.local_matvec(f, G.SELF_BEAD)
    assert rel(got, want) <= FP64_TOL


@pytest.mark.parametrize("nrhs", [1, 5, 8, 20, 64, 70])
@pytest.mark.parametrize("cell_div", [1, 2])
def test_fp32_matvec_error(nrhs, cell_div):
    xyz, L = suspension(5000, 0.1, 31)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(3).standard_normal((nrhs, len(xyz), 3))
    want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=8)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32, cell_div=cell_div) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.local_matvec(f, G.SELF_BEAD)
    err = rel(got, want)
    comp = np.abs(got - want).max() / np.abs(want).max()
    print(f"FP32 nrhs={nrhs} div={cell_div}: norm-wise {err:.2e}, max component {comp:.2e}")
    assert err <= FP32_TOL
    assert comp <= 10 * FP32_TOL


@pytest.mark.parametrize("cell_div", [1, 2])
def test_fp32_matvec_symmetric_pairs(cell_div):
    """Each unordered pair evaluated once from the half list, its source side
    scattered by vector atomics: the oracle's velocities within the FP32
    tolerance on consecutive matvecs (the accumulators are cleared between
    uses) and across a rebuild."""
    xyz, L = suspension(5000, 0.1, 31)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    rng = np.random.default_rng(3)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32, cell_div=cell_div) as ctx:
        ctx.set_pair_tensors(False)
        ctx.set_symmetric_pairs(True)
        for rebuild in range(2):
            ctx.set_particles(xyz)
            ctx.build_cells()
            for _ in range(2):
                f = rng.standard_normal((len(xyz), 3))
                want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=8)
                got = ctx.local_matvec(f, G.SELF_BEAD)
                err = rel(got, want)
                comp = np.abs(got - want).max() / np.abs(want).max()
                print(f"symmetric FP32 div={cell_div}: norm-wise {err:.2e}, max component {comp:.2e}")
                assert err <= FP32_TOL and comp <= 10 * FP32_TOL


def test_fp32_matvec_chains_short_bonds():
    xyz, L = G.make_chains(4, 150, 20, 2.0, 0.05)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(6).standard_normal((len(xyz), 3))
    want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        assert rel(ctx.local_matvec(f, G.SELF_BEAD), want) <= FP32_TOL


def test_spread_and_element_rhs_reference_mode():
    rng = np.random.default_rng(8)
    L = 24.0
    nm = 6
    xyz = rng.uniform(0, L, (150, 3))
    f = rng.standard_normal((150, 3))
    sre = 0.5 * (L / nm) + 4.0 / 0.5 + 1e-3
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    mesh = O.make_mesh(nm, nm, nm, sre)
    c = O.constants(alpha=0.5)
    enb, _ = O.elem_lists(box, mesh, xyz)
    ne, nq, nu = nm ** 3, 8, 20
    # 2x2x2 Gauss points inside each element
    g1 = 0.5 - 0.5 / np.sqrt(3.0)
    h = L / nm
    q = []
    for e in range(ne):
        ix, iy, iz = e % nm, (e // nm) % nm, e // (nm * nm)
        for a in (g1, 1 - g1):
            for b in (g1, 1 - g1):
                for cc in (g1, 1 - g1):
                    q.append([(ix + cc) * h, (iy + b) * h, (iz + a) * h])
    q = np.array(q)
    qe = np.repeat(np.arange(ne), nq).astype(np.int32)
    IF = rng.standard_normal((ne, nu * nq))
    rho_o = O.spread_qp(c, box, enb, xyz, f, q, qe)
    Fe_o = O.element_rhs(c, box, enb, xyz, f, ne, nq, nu, q, IF)
    with G.Context(box_hi=(L,) * 3, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                   search_radius_e=sre, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        rho = ctx.spread_qp(q, f, qe)
        Fe = ctx.element_rhs(ne, nq, nu, q, IF, f)
    assert rel(rho, rho_o) <= FP64_TOL
    assert rel(Fe, Fe_o) <= FP64_TOL


def test_spread_cutoff_mode():
    xyz, L = suspension(800, 0.1, 13)
    f = np.random.default_rng(1).standard_normal((len(xyz), 3))
    q = np.random.default_rng(2).uniform(0, L, (3000, 3))
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    want = O.spread_qp(c, box, None, xyz, f, q, None, rc=8.0)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.spread_qp(q, f, None, spread_rc=8.0)
    assert rel(got, want) <= FP64_TOL


def _dense(c, box, xyz, nb):
    n = len(xyz)
    E = np.eye(3 * n).reshape(3 * n, n, 3)
    return O.local_matvec(c, box, xyz, nb, E, O.SELF_BEAD, nthreads=8).reshape(3 * n, 3 * n).T


def test_chebyshev_faithful_matches_oracle_fp64():
    xyz, L = suspension(400, 0.1, 41)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    M = _dense(c, box, xyz, nb)
    w = np.linalg.eigvalsh(M)
    lmin, lmax = w[0] / 1.05, w[-1] * 1.05
    xi = O.std_normal_vector(123456789, 3 * len(xyz))
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 1))
    for tol in (1e-2, 1e-3):
        y_o, rep_o = O.cheb_inv_sqrt(op, xi, 30, lmin, lmax, tol)
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as ctx:
            ctx.set_particles(xyz)
            ctx.build_cells()
            y, rep = ctx.cheb_inv_sqrt(xi, 30, lmin, lmax, tol)
        r = rep[0]
        assert r["converged"] == rep_o.converged and r["n_terms"] == rep_o.n_terms
        assert r["n_matvecs"] == rep_o.n_matvecs
        assert r["err1"] == pytest.approx(rep_o.err1, rel=1e-8)
        assert r["err2"] == pytest.approx(rep_o.err2, rel=1e-8)
        assert rel(y, y_o) <= 1e-11


def test_chebyshev_faithful_fp32_matches_oracle():
    """The FP32 context's reference-faithful series (check after every term,
    FP64 estimator sums; each term writes the pair records of its new x and
    dw for the next matvecs, and the next term runs speculatively while the
    host waits for a check) against the FP64 oracle's series: the same
    terms, matvecs and stopping decision, err1 / err2 within the FP32 pair
    sums' effect, y and dw = M y within 1e-5; dw is the library's own M y of
    the returned y; a second call repeats the first bit for bit."""
    xyz, L = suspension(3000, 0.1, 43)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    xi = O.std_normal_vector(987654321, 3 * len(xyz))
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=24, seed=5)
        lo, hi = lo / 1.05, hi * 1.05
        y_o, rep_o = O.cheb_inv_sqrt(op, xi, 50, lo, hi, 1e-3)
        y, rep = ctx.cheb_inv_sqrt(xi, 50, lo, hi, 1e-3, check_every=1)
        rc, dw, rep_b = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=1)
        rc2, dw2, _ = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=1)
        # dw is M of the y the series stopped at (not of a speculative next term's)
        My = ctx.local_matvec(y, G.SELF_BEAD)
    assert rel(dw, My) <= 1e-12
    r = rep[0]
    assert r["converged"] == rep_o.converged and r["n_terms"] == rep_o.n_terms
    assert r["n_matvecs"] == rep_o.n_matvecs
    assert r["err1"] == pytest.approx(rep_o.err1, rel=5e-2)
    assert r["err2"] == pytest.approx(rep_o.err2, rel=1e-3)
    assert rel(y, y_o) <= 1e-5
    assert rc == 0 and rep_b[0]["n_terms"] == r["n_terms"]
    My_o = O.local_matvec(c, box, xyz, nb, y_o, O.SELF_BEAD, nthreads=8)
    assert rel(dw, My_o) <= 1e-5
    assert rc2 == 0 and np.array_equal(dw, dw2)
    print(f"FP32 faithful: {r['n_terms']} terms, err1 {r['err1']:.4e} (oracle "
          f"{rep_o.err1:.4e}), y {rel(y, y_o):.2e}, dw {rel(dw, My_o):.2e}")


def test_chebyshev_fp32_batched_rhs_accuracy():
    xyz, L = suspension(1500, 0.1, 43)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
    xi = np.random.default_rng(7).standard_normal((4, 3 * len(xyz)))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=40, seed=5)
        y, reps = ctx.cheb_inv_sqrt(xi, 50, lo / 1.05, hi * 1.05, 1e-3, check_every=1)
    for r in range(4):
        y_o, rep_o = O.cheb_inv_sqrt(op, xi[r], 50, lo / 1.05, hi * 1.05, 1e-3)
        assert reps[r]["converged"] == 1
        assert rel(y.reshape(4, -1)[r], y_o) <= 1e-5


def test_lanczos_bounds_vs_dense_eigenvalues():
    xyz, L = suspension(160, 0.05, 51)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    w = np.linalg.eigvalsh(_dense(c, box, xyz, nb))
    for prec, tol in ((G.FP64, 1e-9), (G.FP32, 1e-5)):
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=prec) as ctx:
            ctx.set_particles(xyz)
            ctx.build_cells()
            lo, hi = ctx.lanczos_bounds(k=3 * len(xyz), seed=1)
            assert lo == pytest.approx(w[0], rel=tol) and hi == pytest.approx(w[-1], rel=tol)
            lo30, hi30 = ctx.lanczos_bounds(k=30, seed=1)
            assert w[0] * (1 - tol) <= lo30 and hi30 <= w[-1] * (1 + tol)
            it, lam = ctx.power_iteration(tol=1e-3, maxits=5000)
            assert lam == pytest.approx(w[-1], rel=2e-3)


def test_philox_noise_matches_oracle():
    import torch
    n = 10001
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    with G.Context(box_hi=(30.0,) * 3) as ctx:
        ctx.philox_normals_dev(99, 7, n, d.data_ptr())
        ctx.synchronize()
    got = d.cpu().numpy()
    want = O.philox_normals(99, 7, n)
    # counter words bit-exact; the FP32 transform within a few FP32 ulps
    assert np.all(np.abs(got - want) <= 1e-6 * (1.0 + np.abs(want)))
    assert abs(got.mean()) < 0.05 and abs(got.std() - 1) < 0.05


def test_non_finite_position_reported_by_the_build():
    xyz, L = suspension(500, 0.05, 9)
    bad = xyz.copy()
    bad[3, 1] = np.nan
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(bad)
        with pytest.raises(G.GGEMError) as ei:
            ctx.build_cells()
        assert ei.value.code == G.ERR_BAD_ARG
        ctx.set_particles(xyz)  # the context stays usable
        ctx.build_cells()
        assert ctx.pair_count() > 0


def test_integer_double_to_float_conversion_matches_hardware():
    """the library's bit-field double -> float rounding (used on the hot
    paths) equals __double2float_rn bit for bit, ties and edges included"""
    import torch
    rng = np.random.default_rng(12)
    vals = [rng.standard_normal(200000), rng.standard_normal(20000) * 1e30,
            rng.standard_normal(20000) * 1e-30, np.exp(rng.uniform(-700, 700, 20000))]
    # exact ties between two floats, both parities, and values next to them
    f = rng.standard_normal(20000).astype(np.float32)
    up = np.nextafter(f, np.float32(np.inf))
    mid = (f.astype(np.float64) + up.astype(np.float64)) / 2.0
    vals += [mid, np.nextafter(mid, np.inf), np.nextafter(mid, -np.inf)]
    vals.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38,
                          3.4028236e38, 1e39, -1e39, 1.1754943508222875e-38, 1e-45, 1e-320]))
    x = np.concatenate(vals)
    d = torch.from_numpy(x).cuda()
    out = torch.empty(len(x), dtype=torch.float32, device="cuda")
    ref = torch.empty_like(out)
    with G.Context(box_hi=(30.0,) * 3) as ctx:
        ctx._check(G.lib().ggem_diag_convert_f32(ctx.h, len(x), d.data_ptr(), out.data_ptr(),
                                                 ref.data_ptr()))
    a = out.cpu().numpy().view(np.uint32)
    b = ref.cpu().numpy().view(np.uint32)
    nan = np.isnan(x)
    assert np.array_equal(a[~nan], b[~nan])
    assert np.all(np.isnan(out.cpu().numpy()[nan]))


def test_errors_are_reported_not_raised_on_device():
    with G.Context(box_hi=(20.0,) * 3, periodic=(0, 0, 0), precision=G.FP64) as ctx:
        ctx.set_particles(np.array([[1.0, 1.0, 1.0], [25.0, 1.0, 1.0]]))
        with pytest.raises(G.GGEMError) as e:
            ctx.build_cells()
        assert e.value.code == G.ERR_OUT_OF_DOMAIN
    with pytest.raises(G.GGEMError) as e:
        G.Context(box_hi=(15.0,) * 3, rc=7.0)  # periodic edge < 3 rc
    assert e.value.code == G.ERR_BAD_ARG
    xyz, L = suspension(200, 0.05, 2)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        with pytest.raises(G.GGEMError) as e:
            ctx.cheb_inv_sqrt(np.ones(3 * len(xyz)), 10, 2.0, 1.0, 0.1)
        assert e.value.code == G.ERR_INVALID_RANGE


def test_device_pointer_matvec_with_torch_stream():
    import torch
    xyz, L = suspension(1000, 0.1, 61)
    f = np.random.default_rng(0).standard_normal((2, len(xyz), 3))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        want = ctx.local_matvec(f, G.SELF_BEAD)
        s = torch.cuda.Stream()
        df = torch.from_numpy(f).cuda()
        du = torch.empty_like(df)
        ctx.set_stream(s.cuda_stream)
        torch.cuda.current_stream().synchronize()
        ctx.local_matvec_dev(df.data_ptr(), du.data_ptr(), 2, G.SELF_BEAD)
        s.synchronize()
        ctx.set_stream(0)
        assert np.array_equal(du.cpu().numpy(), want)


@pytest.mark.parametrize("check_every", [0, 3])
def test_chebyshev_sparse_checks_and_displacement(check_every):
    """Sparse error checks return a y whose reported err1 is its own and a
    Brownian displacement dw = M y equal to an explicit matvec of y."""
    xyz, L = suspension(3000, 0.1, 47)
    xi = np.random.default_rng(12).standard_normal(3 * len(xyz))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=24, seed=5)
        y_ref, rep_ref = ctx.cheb_inv_sqrt(xi, 50, lo / 1.05, hi * 1.05, 1e-3, check_every=1)
        for _ in range(3):  # the adaptive mode learns the degree across calls
            rc, dw, rep = ctx.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05, 1e-3,
                                                    check_every=check_every)
            assert rc == 0 and rep[0]["converged"] and rep[0]["err1"] <= 1e-3
            assert rep[0]["n_terms"] >= rep_ref[0]["n_terms"]
        y, rep2 = ctx.cheb_inv_sqrt(xi, 50, lo / 1.05, hi * 1.05, 1e-3, check_every=check_every)
        assert rep2[0]["n_terms"] == rep[0]["n_terms"] or check_every == 0
        My = ctx.local_matvec(y, G.SELF_BEAD)
        if rep2[0]["n_terms"] == rep[0]["n_terms"]:
            assert rel(dw, My) <= 1e-12
        assert rel(y, y_ref) <= 5e-3


def test_fused_chebyshev_terms_match_unfused_path():
    """Terms without an error check run as one fused pair-sum + recurrence
    kernel on the FP32 single-RHS path; its y equals the unfused path's and
    the FP64 oracle's within the FP32 pair-sum tolerance."""
    xyz, L = suspension(2000, 0.1, 53)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
    xi = np.random.default_rng(21).standard_normal(3 * len(xyz))
    N = 12
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=30, seed=3)
        lo, hi = lo / 1.05, hi * 1.05
        y1, r1 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=1)
        ctx.set_kernel_timing(True)
        y2, r2 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=N - 1)
        fused_ms, fused_n = ctx.kernel_timing(G.KERNEL_PAIR_CHEB)
        ctx.set_kernel_timing(False)
    assert r1[0]["n_terms"] == r2[0]["n_terms"] == N
    assert fused_n == N - 2  # terms 1 .. N-2; the last term is checked
    assert rel(y2, y1) <= 1e-12
    y_o, rep_o = O.cheb_inv_sqrt(op, xi, N, lo, hi, 0.0)
    assert rep_o.n_terms == N
    assert rel(y2, y_o) <= 1e-5
    # err1 = sqrt(|y.M.M.y - xi.M.xi| / xi.M.xi) cancels to ~1e-9 relative
    # here, below the FP32 pair-sum error, so only the FP32 runs agree closely
    assert r2[0]["err1"] == pytest.approx(r1[0]["err1"], rel=1e-6)
    assert 0.5 * rep_o.err1 <= r2[0]["err1"] <= 2.0 * rep_o.err1


def test_fused_series_estimators_match_unfused_path():
    """Per-matvec pair tensors: the whole series is fused, and the
    estimator sums (xi.M.xi, the checked term's norms, |M dw|^2) come from
    the pair kernels as float-float partials without FP64 arithmetic; err1,
    err2 and y agree with the path that checks every term in FP64 vector
    kernels, and the adaptive series stops at the same degree."""
    xyz, L = suspension(4000, 0.1, 57)
    xi = np.random.default_rng(23).standard_normal(3 * len(xyz))
    # err1 = sqrt(|y.M.M.y - xi.M.xi| / xi.M.xi): at 8 terms err1 ~ 1e-3, so
    # the sums' ~1e-14 relative error moves err1 by ~1e-8 relative (deeper
    # series cancel more: at err1 ~ 2e-5 it is ~1e-5)
    N = 8
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_pair_tensors(False)
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=30, seed=3)
        lo, hi = lo / 1.05, hi * 1.05
        y1, r1 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=1)
        y2, r2 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=N - 1)
        rc, dw_a, ra = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=1)
        rc2, dw_b, rb = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=0)
        rc3, dw_c, rc_ = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=0)
    assert rel(y2, y1) <= 1e-12
    assert r2[0]["err1"] == pytest.approx(r1[0]["err1"], rel=1e-6)
    assert r2[0]["err2"] == pytest.approx(r1[0]["err2"], rel=1e-9)
    assert rc == rc2 == rc3 == 0
    # the adaptive (fused) series converges at the degree the every-term
    # check finds, with the same err1
    assert rb[0]["n_terms"] == ra[0]["n_terms"] or rc_[0]["n_terms"] == ra[0]["n_terms"]
    same = rc_ if rc_[0]["n_terms"] == ra[0]["n_terms"] else rb
    dw_s = dw_c if same is rc_ else dw_b
    assert same[0]["err1"] == pytest.approx(ra[0]["err1"], rel=1e-6)
    assert rel(dw_s, dw_a) <= 1e-12


def test_fused_batched_chebyshev_terms_match_unfused_path():
    """16 .. 64 right-hand sides: unchecked terms run as one batched kernel
    (pair sum, recurrence and the next term's FP32 staging); the series
    equals the one that checks every term (unfused) to rounding."""
    xyz, L = G.make_chains(5, 60, 20, 2.0, 0.05)
    n = len(xyz)
    xi = np.random.default_rng(31).standard_normal((40, 3 * n))
    N = 12
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_pair_tensors(False)
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=30, seed=3)
        lo, hi = lo / 1.05, hi * 1.05
        y1, r1 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=1)
        ctx.set_kernel_timing(True)
        y2, r2 = ctx.cheb_inv_sqrt(xi, N, lo, hi, 0.0, check_every=N - 1)
        fused_ms, fused_n = ctx.kernel_timing(G.KERNEL_PAIR_CHEB)
        ctx.set_kernel_timing(False)
    assert all(r["n_terms"] == N for r in r1 + r2)
    assert fused_n == N - 2  # terms 1 .. N-2; the last term is checked
    assert rel(y2, y1) <= 1e-12
    # the FP32 series' estimator sums are float-float (~1e-15 relative here);
    # err1 = sqrt(|a1 - a2| / a2) divides that by err1^2 ~ 7.6e-7
    for a, b in zip(r1, r2):
        assert b["err1"] == pytest.approx(a["err1"], rel=1e-7)


def test_batched_64_rhs_chains_matvec_and_chebyshev():
    """The polymer workload's shape at a small size: 20-bead chains, phi=0.05,
    64 noise right-hand sides through the batched pair kernel (lanes over
    right-hand sides) and the adaptive Chebyshev; each checked against the
    FP64 oracle."""
    xyz, L = G.make_chains(11, 100, 20, 2.0, 0.05)
    n = len(xyz)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(9).standard_normal((64, n, 3))
    want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=8)
    xi = np.random.default_rng(10).standard_normal((64, 3 * n))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.local_matvec(f, G.SELF_BEAD)
        lo, hi = ctx.lanczos_bounds(k=40, seed=2)
        y, reps = ctx.cheb_inv_sqrt(xi, 50, lo / 1.05, hi * 1.05, 1e-3, check_every=0)
    assert rel(got, want) <= FP32_TOL
    for r in range(64):
        assert rel(got[r], want[r]) <= FP32_TOL
    assert all(rp["converged"] and rp["err1"] <= 1e-3 for rp in reps)
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
    for r in (0, 31, 63):
        # the oracle checks every term and may stop earlier than the adaptive
        # schedule; both series meet err1 <= 1e-3
        y_o, rep_o = O.cheb_inv_sqrt(op, xi[r], 50, lo / 1.05, hi * 1.05, 1e-3)
        assert rep_o.converged and rep_o.n_terms <= reps[r]["n_terms"]
        assert rel(y.reshape(64, -1)[r], y_o) <= 5e-3


@pytest.mark.parametrize("stored,variant", [(False, 0), (False, 1), (True, 0), (True, 1),
                                            (True, 2), (True, 3)])
def test_pair_tensor_storage_modes(stored, variant):
    """Stored per-pair tensors (streamed) and per-matvec tensors (computed)
    give the same velocities within the FP32 contract, and the same
    fused-Chebyshev displacement."""
    xyz, L = suspension(4000, 0.1, 71)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    f = np.random.default_rng(8).standard_normal((1, len(xyz), 3))
    want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=8)
    xi = np.random.default_rng(9).standard_normal(3 * len(xyz))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_pair_tensors(stored)
        ctx.set_pair_variant(computed=0 if stored else variant,
                             stored=variant if stored else 0)
        ctx.set_particles(xyz)
        ctx.build_cells()
        W, st = ctx.pair_storage()
        assert st == stored and W % 8 == 0
        got = ctx.local_matvec(f, G.SELF_BEAD)
        lo, hi = ctx.lanczos_bounds(k=30, seed=3)
        y, rep = ctx.cheb_inv_sqrt(xi, 12, lo / 1.05, hi * 1.05, 0.0, check_every=11)
    assert rel(got, want) <= FP32_TOL
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
    y_o, _ = O.cheb_inv_sqrt(op, xi, 12, lo / 1.05, hi * 1.05, 0.0)
    assert rel(y, y_o) <= 1e-5


@pytest.mark.parametrize("mode", ["cutoff", "reference"])
def test_excluded_volume_forces_match_oracle(mode):
    xyz, L = suspension(3000, 0.1, 81)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c1, c2 = 0.37, 0.21
    if mode == "cutoff":
        nb = O.neighbors_cutoff(box, xyz, 7.0)
        kw = dict(rc=7.0, precision=G.FP64)
    else:
        nm = 12
        sre = 0.5 * L / nm + 8.0 + 1e-3
        nb = O.neighbors_reference(box, O.make_mesh(nm, nm, nm, sre), xyz)
        kw = dict(nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3, search_radius_e=sre,
                  precision=G.FP64)
    want = O.ev_gaussian(box, xyz, nb, c1, c2)
    with G.Context(box_hi=(L,) * 3, **kw) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        got = ctx.ev_gaussian_forces(c1, c2)
        base = np.ones_like(got)
        got2 = ctx.ev_gaussian_forces(c1, c2, f=base)
    assert rel(got, want) <= 1e-12
    assert rel(got2 - base, want) <= 1e-12


@pytest.mark.parametrize("kind", [G.SPRING_WLS, G.SPRING_FENE, G.SPRING_UD, G.SPRING_LHS])
def test_spring_forces_match_oracle(kind):
    n_chains, beads = 60, 20
    xyz, L = G.make_chains(17, n_chains, beads, 2.0, 0.05)
    bonds = np.array([[c * beads + k, c * beads + k + 1] for c in range(n_chains)
                      for k in range(beads - 1)])
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    params = {G.SPRING_WLS: (0.25, 4.0), G.SPRING_FENE: (0.8, 3.0), G.SPRING_UD: (0.05, 5.0),
              G.SPRING_LHS: (1.9, 2.5)}[kind]
    want = O.spring_forces(box, xyz, bonds, kind, *params)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        ctx.set_bonds(bonds)
        got = ctx.spring_forces(kind, *params)
    assert rel(got, want) <= 1e-12


def test_fp64_and_fp32_bead_velocity_vs_reference_ggem_stokes_outputs():
    """The CUDA matvec against outputs of the reference's own GGEMStokes
    (src/ggem_stokes.C compiled into oracle/_ref, stored in
    tests/golden/ref_ggem_local.json): local_solution_bead - self exclusion
    + f for beads (pm_system_stokes.C:446-455), local_solution_bead with
    G(0) f for Lagrangian points (ggem_stokes.C:485-499).  FP64 within
    1e-12, FP32 within 1e-6 (norm-wise)."""
    d = json.loads((GOLD / "ref_ggem_local.json").read_text())

    def unhex(a):
        return np.array([float.fromhex(x) for x in a]).reshape(-1, 3)

    for b in d["beads"]:
        kw = {k: b[k] for k in ("ibm_beta", "hmin") if k in b}
        lag = b["point_type"] == G.LAGRANGIAN_POINT
        xyz, f = unhex(b["xyz"]), unhex(b["f"])
        ul, us = unhex(b["u_local"]), unhex(b["u_self"])
        want = ul if lag else ul - us + f
        mode = G.SELF_LAGRANGIAN if lag else G.SELF_BEAD
        for prec, tol in ((G.FP64, FP64_TOL), (G.FP32, FP32_TOL)):
            with G.Context(alpha=b["alpha"], point_type=b["point_type"], box_hi=(b["L"],) * 3,
                           periodic=b["periodic"], rc=b["rc"], precision=prec, **kw) as ctx:
                ctx.set_particles(xyz)
                ctx.build_cells()
                got = ctx.local_matvec(f, mode)
            err = rel(got, want)
            print(f"{b['case']} precision={prec}: {err:.2e}")
            assert err <= tol, (b["case"], prec)
