"""The FP64 oracle against the reference's golden vectors and known answers.

Pins: the PointParticle_Stokes_GGEM golden profiles (pair kernel in field
mode and the unbounded xi-smoothed Green's function), the reference's own
chebyshev.C (bit-exact), closed-form Chebyshev / spectral known answers and
dense-matrix eigenvalues for the Lanczos bounds.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _build():
    O.build_oracle(with_ref=True)


def test_constants_match_reference_formulas():
    c = O.constants(alpha=0.5)
    # ggem_stokes.C:44, :59, :81, :112 with mu = 1/(6 pi), br0 = 1
    assert c.one_eight_pi_mu == pytest.approx(0.75, rel=1e-15)
    assert c.ksi == pytest.approx(np.sqrt(np.pi) / 3, rel=1e-15)
    assert c.coeff_1 == pytest.approx(0.75 * 4 * 0.5 / np.sqrt(np.pi), rel=1e-15)
    assert c.coeff_2 == pytest.approx(0.75 * 4 * (c.ksi - 0.5) / np.sqrt(np.pi), rel=1e-15)
    # bead self mobility 1 - coeff_1 equals G_local(0) = coeff_2 when br0 = 1
    assert 1 - c.coeff_1 == pytest.approx(c.coeff_2, rel=1e-14)
    lag = O.constants(alpha=0.5, point_type=O.LAGRANGIAN_POINT, ibm_beta=0.75, hmin=2.0)
    assert lag.ksi == pytest.approx(1 / 1.5, rel=1e-15)


@pytest.mark.parametrize("axis", ["x", "y", "z"])
def test_golden_velocity_profile(axis):
    """Local GGEM velocity at the reference profile points, 3 beads, alpha 0.35.

    The golden files were produced with the point-centred neighbour search of
    radius search_radius_p = 4/alpha (copss.C:1074); the cut-off field
    evaluation at that radius reproduces them to the printed 9 decimals.
    """
    g = json.loads((GOLD / "ggem_profile_3P.json").read_text())
    c = O.constants(alpha=g["alpha"])
    box = O.make_box([g["box"][0]] * 3, [g["box"][1]] * 3, [0, 0, 0])
    xyz = np.array(g["beads"])
    f = np.array([g["force"]] * 3)
    ax = "xyz".index(axis)
    A = g["axes"][axis]
    pts = np.zeros((len(A["coord"]), 3))
    pts[:, ax] = A["coord"]
    ul = O.local_field_cutoff(c, box, xyz, f, pts, 4.0 / g["alpha"])
    ue = O.exact_unbounded(c, xyz, f, pts)
    tol = 0.5 * 10.0 ** (-g["print_decimals"]) + 1e-12
    assert np.abs(ul - np.array(A["local"])).max() <= tol
    assert np.abs(ue - np.array(A["exact"])).max() <= tol


def test_chebyshev_coefficients_bit_exact_vs_reference_source():
    d = json.loads((GOLD / "ref_chebyshev_coeffs.json").read_text())
    for cs in d["cases"]:
        c = O.cheb_coeffs(cs["N"], float.fromhex(cs["da"]), float.fromhex(cs["db"]),
                          cs["method"])
        ref = np.array([float.fromhex(x) for x in cs["coef"]])
        assert np.array_equal(c, ref), (cs["N"], cs["method"])


def test_chebyshev_coefficients_live_reference_build():
    if O.ref_lib() is None:
        pytest.skip("reference source tree not present on this machine")
    rng = np.random.default_rng(3)
    for _ in range(20):
        N = int(rng.integers(2, 60))
        lmin = float(rng.uniform(0.01, 1.0))
        lmax = lmin * float(rng.uniform(1.1, 50.0))
        d = lmax - lmin
        for m in (0, 1, 2):
            a = O.cheb_coeffs(N, 2 / d, -(lmax + lmin) / d, m)
            b = O.ref_cheb_coeffs(N, 2 / d, -(lmax + lmin) / d, m)
            assert np.array_equal(a, b)


def test_chebyshev_diagonal_operator_known_answer():
    """brownian_system.C:1181-1211 test operator M = diag(1..n): the Chebyshev
    series must reproduce M^{-1/2} xi within the stated error estimate."""
    n = 12
    op = O.Operator("diag", dim=n)
    xi = np.random.default_rng(0).standard_normal(n)
    # err1 = sqrt(|y.M^2.y - xi.M.xi| / xi.M.xi) scales like the square root
    # of the relative error of y, so tol 1e-4 asks for ~1e-8 accuracy
    y, rep = O.cheb_inv_sqrt(op, xi, 50, 1.0 / 1.05, n * 1.05, 1e-4)
    assert rep.converged == 1
    exact = xi / np.sqrt(np.arange(1, n + 1))
    assert np.abs(y - exact).max() / np.abs(exact).max() < 1e-6
    assert rep.n_matvecs == 2 + 2 * (rep.n_terms - 1)
    # an unreachable tolerance stops on the err2 <= 1e-9 rule unconverged
    y2, rep2 = O.cheb_inv_sqrt(op, xi, 50, 1.0 / 1.05, n * 1.05, 1e-7)
    assert rep2.converged == 0 and rep2.err2 <= 1e-9 and rep2.n_terms < 50


def _suspension(n, phi, seed):
    rng = np.random.default_rng(seed)
    L = (n * 4.0 / 3.0 * np.pi / phi) ** (1 / 3)
    pts = []
    while len(pts) < n:
        p = rng.uniform(0, L, 3)
        ok = True
        for q in pts:
            d = p - q
            d -= L * np.round(d / L)
            if d @ d < 4.0:
                ok = False
                break
        if ok:
            pts.append(p)
    return np.array(pts), L


def test_cutoff_lists_match_brute_force():
    xyz, L = _suspension(300, 0.1, 1)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    for i, lst in enumerate(nb.lists()):
        d = xyz - xyz[i]
        d -= L * np.round(d / L)
        r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        want = np.nonzero(r2 < 49.0)[0]
        want = want[want != i]
        assert np.array_equal(np.sort(lst), want)


def test_reference_lists_self_removed_and_symmetric_within_cell():
    xyz, L = _suspension(200, 0.05, 2)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    mesh = O.make_mesh(12, 12, 12, 0.5 * L / 12 + 8.0)
    nb = O.neighbors_reference(box, mesh, xyz)
    for i, lst in enumerate(nb.lists()):
        assert i not in set(lst.tolist())
        assert len(set(lst.tolist())) == len(lst)


def test_local_mobility_spd_and_lanczos_bounds():
    xyz, L = _suspension(120, 0.1, 4)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    n = len(xyz)
    M = np.zeros((3 * n, 3 * n))
    for k in range(3 * n):
        e = np.zeros(3 * n)
        e[k] = 1
        M[:, k] = O.local_matvec(c, box, xyz, nb, e, O.SELF_BEAD)
    assert np.abs(M - M.T).max() < 1e-14
    ev = np.linalg.eigvalsh(M)
    assert ev[0] > 0
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 1))
    lo, hi, a, b = O.lanczos(op, np.random.default_rng(1).standard_normal(3 * n), 3 * n)
    assert lo == pytest.approx(ev[0], rel=1e-8)
    assert hi == pytest.approx(ev[-1], rel=1e-8)
    lo30, hi30, _, _ = O.lanczos(op, np.random.default_rng(1).standard_normal(3 * n), 30)
    assert ev[0] <= lo30 + 1e-12 and hi30 <= ev[-1] + 1e-12
    # brownian_system.C:846-920 defaults: tol 1e-3 on the iterate change
    it, lam = O.power_iteration(op, 3 * n, tol=1e-3, maxits=5000)
    assert it >= 0 and lam <= ev[-1] * (1 + 1e-12) and lam == pytest.approx(ev[-1], rel=1e-3)


def test_chebyshev_on_local_mobility_matches_dense_inverse_sqrt():
    xyz, L = _suspension(80, 0.1, 5)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    nb = O.neighbors_cutoff(box, xyz, 7.0)
    n = len(xyz)
    M = np.zeros((3 * n, 3 * n))
    for k in range(3 * n):
        e = np.zeros(3 * n)
        e[k] = 1
        M[:, k] = O.local_matvec(c, box, xyz, nb, e, O.SELF_BEAD)
    w, V = np.linalg.eigh(M)
    xi = np.random.default_rng(9).standard_normal(3 * n)
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 1))
    y, rep = O.cheb_inv_sqrt(op, xi, 50, w[0] / 1.05, w[-1] * 1.05, 1e-4)
    exact = V @ ((V.T @ xi) / np.sqrt(w))
    assert rep.converged
    # err1 is a first-order, sign-averaged estimate of the error of y, so the
    # true error is checked at a looser level than err1**2
    assert np.linalg.norm(y - exact) / np.linalg.norm(exact) < 1e-4
    # err1 definition, brownian_system.C:1117-1125
    My = M @ y
    err1 = np.sqrt(abs(My @ My - xi @ (M @ xi)) / (xi @ (M @ xi)))
    assert err1 == pytest.approx(rep.err1, rel=1e-6, abs=1e-12)


def test_spread_and_element_rhs_consistent():
    rng = np.random.default_rng(7)
    L = 20.0
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    xyz = rng.uniform(0, L, (40, 3))
    f = rng.standard_normal((40, 3))
    mesh = O.make_mesh(5, 5, 5, 0.5 * 4 + 8.0)
    enb, _ = O.elem_lists(box, mesh, xyz)
    ne, nq, nu = 125, 8, 20
    q = rng.uniform(0, L, (ne * nq, 3))
    qe = np.repeat(np.arange(ne), nq).astype(np.int32)
    IF = rng.standard_normal((ne, nu * nq))
    rho = O.spread_qp(c, box, enb, xyz, f, q, qe)
    Fe = O.element_rhs(c, box, enb, xyz, f, ne, nq, nu, q, IF)
    want = np.zeros((ne, 3 * nu))
    for e in range(ne):
        for qp in range(nq):
            for j in range(3):
                want[e, j * nu:(j + 1) * nu] += IF[e].reshape(nu, nq)[:, qp] * rho[e * nq + qp, j]
    assert np.abs(Fe - want).max() < 1e-12
    # direct evaluation of smoothed_force_exp for one point
    e0 = 0
    lst = enb.lists()[e0]
    r = 0.0
    for j in lst:
        d = xyz[j] - q[0]
        d -= L * np.round(d / L)
        r += O.smoothed_force_exp(c, d) * f[j, 0]
    assert rho[0, 0] == pytest.approx(r, rel=1e-13)


def test_std_normal_stream_is_reproducible_and_normal():
    a = O.std_normal_vector(123456789, 30000)
    b = O.std_normal_vector(123456789, 30000)
    assert np.array_equal(a, b)
    assert abs(a.mean()) < 0.03 and abs(a.std() - 1) < 0.03
    skipped = O.std_normal_vector(123456789, 3000, skip_vectors=2)
    assert not np.array_equal(skipped, a[:3000])


def test_philox_known_answer():
    # Philox4x32-10 known-answer vector (Random123 kat_vectors: counter 0,
    # key 0 -> 6627e8d5 e169c58d bc57ac4c 9b00dbd8)
    out = O.philox_normals(0, 0, 4)
    words = [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    for h in range(2):
        u1 = float(np.float32(np.float32(words[2 * h]) * np.float32(2.0 ** -32)
                              + np.float32(2.0 ** -33)))
        u2 = float(np.float32((words[2 * h + 1] >> 9) * 2.0 ** -23 + 2.0 ** -24))
        r = np.sqrt(-2 * np.log(u1))
        assert out[2 * h] == pytest.approx(r * np.cos(2 * np.pi * u2), rel=1e-14)
        assert out[2 * h + 1] == pytest.approx(r * np.sin(2 * np.pi * u2), rel=1e-14)


def test_mlp_oracle_gradient_matches_finite_differences():
    """The network oracle's backward formulas, in exact float64 arithmetic,
    against central differences of its own loss."""
    import mlp_oracle as M
    rng = np.random.default_rng(4)
    n = 7
    P = (rng.standard_normal(55808) * 0.05)
    X = rng.standard_normal((n, M.IN))
    Y = rng.standard_normal((n, M.OUT))
    norm = np.concatenate([np.zeros(M.IN), np.ones(M.IN), np.zeros(2), np.ones(2)])
    loss, g = M.loss_and_grad(P, norm, X, Y, exact=True)
    # a sample of parameters from every layer (weights and biases)
    offs = [0, 48 * 128, 48 * 128 + 128, 48 * 128 + 128 + 16384, 48 * 128 + 256 + 2 * 16384,
            48 * 128 + 384 + 3 * 16384]
    picks = [offs[0] + 5, offs[0] + 130, offs[1] + 3, offs[2] + 777, offs[3] + 11,
             offs[4] + 129, offs[4] + 5, offs[5] + 1]
    for k in picks:
        h = 1e-6
        Pp, Pm = P.copy(), P.copy()
        Pp[k] += h
        Pm[k] -= h
        fd = (M.loss_and_grad(Pp, norm, X, Y, exact=True)[0] -
              M.loss_and_grad(Pm, norm, X, Y, exact=True)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), (k, fd, g[k])


def test_bf16_rounding_is_nearest_even():
    import mlp_oracle as M
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 0.0],
                 dtype=np.float32)
    got = M.bf16(x)
    want = np.array([1.0, 1.0, 1.0 + 4 * 2 ** -8, 1.0, -2.5, 0.0], dtype=np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1
    assert np.array_equal(got, want)


def test_force_oracle_laws_and_action_reaction():
    """The spring laws of the force fixes (fix_base.C:55-148) on known
    points, and Newton's third law of the pairwise oracle forces."""
    import oracle as O
    O.build_oracle(with_ref=False)
    box = O.make_box([0] * 3, [30.0] * 3, [1, 1, 1])
    # LHS: zero at the rest length, k0 (R - l0) along R beyond it
    xyz = np.array([[1.0, 1.0, 1.0], [4.0, 1.0, 1.0]])
    f = O.spring_forces(box, xyz, [[0, 1]], 3, 2.0, 5.0)
    assert np.allclose(f[0], [5.0, 0, 0]) and np.allclose(f[1], [-5.0, 0, 0])
    f = O.spring_forces(box, xyz, [[0, 1]], 3, 3.0, 5.0)
    assert np.allclose(f, 0.0)
    # WLS at R/Ls = 1/2: c1 (1/(1/2)^2 - 1 + 2) = 5 c1 along R
    f = O.spring_forces(box, xyz, [[0, 1]], 0, 0.7, 6.0)
    assert np.allclose(f[0], [0.7 * 5.0, 0, 0])
    # minimum image: the partner across the boundary pulls backwards
    xyz2 = np.array([[0.5, 1.0, 1.0], [29.0, 1.0, 1.0]])
    f = O.spring_forces(box, xyz2, [[0, 1]], 3, 0.0, 1.0)
    assert np.allclose(f[0], [-1.5, 0, 0])
    rng = np.random.default_rng(2)
    pts = rng.uniform(0, 30.0, (300, 3))
    nb = O.neighbors_cutoff(box, pts, 7.0)
    ev = O.ev_gaussian(box, pts, nb, 0.3, 0.2)
    assert np.abs(ev.sum(axis=0)).max() < 1e-12 * np.abs(ev).max() * len(pts)
    bonds = np.stack([np.arange(299), np.arange(1, 300)], 1)
    for kind in range(4):
        sp = O.spring_forces(box, pts, bonds, kind, 0.2, 40.0)
        assert np.abs(sp.sum(axis=0)).max() < 1e-9 * max(1.0, np.abs(sp).max())


def test_hex20_shape_functions_kronecker_partition_and_quadratics():
    """the serendipity element: N_i(node_j) = delta_ij, sum N = 1, and the
    20-node space reproduces every quadratic polynomial exactly"""
    from fem_mesh import HEX20
    for j, node in enumerate(HEX20):
        n = O.hex20_shape(node.astype(float))
        assert np.allclose(n, np.eye(20)[j], atol=1e-15)
    rng = np.random.default_rng(0)
    for xi in rng.uniform(-1, 1, (50, 3)):
        n = O.hex20_shape(xi)
        assert abs(n.sum() - 1.0) < 1e-14
        for mono in (lambda p: p[..., 0] * p[..., 1], lambda p: p[..., 2] ** 2,
                     lambda p: p[..., 1] - 0.5 * p[..., 0] * p[..., 2]):
            assert abs(n @ mono(HEX20.astype(float)) - mono(xi)) < 1e-14


def test_fem_point_values_oracle_reproduces_quadratic_fields():
    from fem_mesh import hex20_mesh, quadratic
    ne, lo, hi = (4, 3, 5), (-2.0, 0.0, 1.0), (6.0, 3.0, 11.0)
    dofs, nd, dpos, dvar = hex20_mesh(ne, lo, hi, seed=1)
    sol = np.array([quadratic(dpos[k], dvar[k]) for k in range(nd)])
    pts = np.random.default_rng(2).uniform(lo, hi, (300, 3))
    u, outside = O.fem_point_values(pts, ne, lo, hi, (0, 0, 0), dofs, sol)
    assert outside == 0
    want = np.stack([quadratic(pts, v) for v in range(3)], axis=1)
    assert np.abs(u - want).max() <= 1e-12 * np.abs(want).max()


# ---------------------------------------------------------------------------
# the reference's own GGEMStokes (src/ggem_stokes.C through oracle/_ref)
# ---------------------------------------------------------------------------
def _unhex(a, shape=None):
    v = np.array([float.fromhex(x) for x in a])
    return v.reshape(shape) if shape is not None else v


def _ggem_gold():
    return json.loads((GOLD / "ref_ggem_local.json").read_text())


def test_green_tensor_bit_exact_vs_reference_ggem_stokes():
    """green_tensor_local_regularized (ggem_stokes.C:304-352) for bead,
    Lagrangian and point-particle constants, r = 0, r < r_eps and generic r"""
    d = _ggem_gold()
    vecs = _unhex(d["vectors"], (-1, 3))
    for g in d["green"]:
        kw = {k: g[k] for k in ("ibm_beta", "hmin") if k in g}
        c = O.constants(alpha=g["alpha"], point_type=g["point_type"], **kw)
        want = _unhex(g["G"], (-1, 3, 3))
        got = np.stack([O.green_local(c, x) for x in vecs])
        assert np.array_equal(got, want), g["type"]


def _bead_case(b):
    kw = {k: b[k] for k in ("ibm_beta", "hmin") if k in b}
    c = O.constants(alpha=b["alpha"], point_type=b["point_type"], **kw)
    L = b["L"]
    box = O.make_box((0, 0, 0), (L, L, L), b["periodic"])
    xyz = _unhex(b["xyz"], (-1, 3))
    f = _unhex(b["f"], (-1, 3))
    return c, box, xyz, f, kw


def test_bead_local_sums_bit_exact_vs_reference_ggem_stokes():
    """local_solution_bead (ggem_stokes.C:426-503) with global_self_exclusion
    (:506-521) and the bead velocity of pm_system_stokes.C:446-455:
    the oracle's SELF_NONE / SELF_BEAD / SELF_LAGRANGIAN sums equal the
    reference's own outputs bit for bit, over the same cut-off lists"""
    for b in _ggem_gold()["beads"]:
        c, box, xyz, f, _ = _bead_case(b)
        nb = O.neighbors_cutoff(box, xyz, b["rc"])
        assert np.array_equal(nb.offsets, b["offsets"]) and np.array_equal(nb.ids, b["ids"])
        ul = _unhex(b["u_local"], (-1, 3))
        us = _unhex(b["u_self"], (-1, 3))
        if b["point_type"] == O.LAGRANGIAN_POINT:
            # the reference adds G(0) f inside local_solution_bead (:485-499)
            got = O.local_matvec(c, box, xyz, nb, f, O.SELF_LAGRANGIAN)
            assert np.array_equal(got, ul), b["case"]
        else:
            assert np.array_equal(O.local_matvec(c, box, xyz, nb, f, O.SELF_NONE), ul), b["case"]
            got = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD)
            assert np.array_equal(got, ul - us + f), b["case"]
        assert np.array_equal(us, c.coeff_1 * f)


def test_field_local_sums_bit_exact_vs_reference_ggem_stokes():
    """local_solution_field (ggem_stokes.C:358-423) over the element
    point-neighbour lists, at targets inside the elements"""
    fd = _ggem_gold()["field"]
    L, nm = fd["L"], fd["n_mesh"]
    c = O.constants(alpha=fd["alpha"])
    box = O.make_box((0, 0, 0), (L, L, L), fd["periodic"])
    mesh = O.make_mesh(nm, nm, nm, fd["search_radius_e"])
    xyz = _unhex(fd["xyz"], (-1, 3))
    f = _unhex(fd["f"], (-1, 3))
    enb, _ = O.elem_lists(box, mesh, xyz)
    targets = _unhex(fd["targets"], (-1, 3))
    got = O.local_field_reference(c, box, mesh, enb, xyz, f, targets)
    assert np.array_equal(got, _unhex(fd["u"], (-1, 3)))


def test_live_reference_ggem_stokes_build():
    """fresh cases through the reference's GGEMStokes compiled here"""
    if O.ref_ggem_lib() is None:
        pytest.skip("reference source tree not present on this machine")
    rng = np.random.default_rng(11)
    for pt, kw in ((O.POLYMER_BEAD, {}), (O.LAGRANGIAN_POINT, {"ibm_beta": 0.6, "hmin": 1.5})):
        c = O.constants(alpha=0.4, point_type=pt, **kw)
        for x in rng.standard_normal((50, 3)) * 4:
            assert np.array_equal(O.green_local(c, x), O.ref_green_local(c, x, pt, **kw))
        L = 11.0
        box = O.make_box((-3, 0, 2), (L - 3, L, L + 2), (1, 0, 1))
        xyz = np.array([-3, 0, 2]) + rng.uniform(0, L, (120, 3))
        f = rng.standard_normal((120, 3))
        nb = O.neighbors_cutoff(box, xyz, 5.5)
        ul, us = O.ref_local_bead(c, box, xyz, f, nb, pt, **kw)
        if pt == O.LAGRANGIAN_POINT:
            assert np.array_equal(O.local_matvec(c, box, xyz, nb, f, O.SELF_LAGRANGIAN), ul)
        else:
            assert np.array_equal(O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD), ul - us + f)
