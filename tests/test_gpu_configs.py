"""Parity at the benchmark's own configurations, against the FP64 oracle.

Each test builds one of the five workloads at its full size (seeded,
synthetic: the reference ships none of them) and compares the CUDA path,
through the C ABI, with the oracle restatement of the reference:

  * N = 1000 beads, phi = 0.05, order 30 with Lanczos bounds, in both
    neighbour modes (element lists of point_mesh.C:293-848 and the rc = 7
    cut-off): lists bit-exact, FP64 u within 1e-12, the reference-faithful
    series (brownian_system.C:967-1178) with the oracle's terms, matvec
    count, err1/err2 and y;
  * N = 200k, phi = 0.1: lists bit-exact, FP64 u within 1e-12, FP32 u
    within 1e-6 norm-wise (per-component error printed);
  * 5000 chains x 20 beads (N = 100k), 64 right-hand sides: every
    right-hand side's FP32 u within 1e-6, and the adaptive batched series
    on a sample of right-hand sides against the oracle's series run to the
    same number of terms;
  * 512 uneven suspensions x 8 right-hand sides: every suspension's u
    within 1e-6, and the batched series of the smallest, the largest and
    the densest suspension against the oracle's series;
  * the shipped eigen-interval network on the 2000 held-out configurations
    of its training run: the fraction of intervals that contain both
    Lanczos bounds.
"""
import os
import time

import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-6
ALPHA, RC = 0.5, 7.0
THREADS = max(1, min(64, os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _timed(label, t0):
    print(f"{label}: {time.perf_counter() - t0:.1f} s")


def cheb_fixed_terms(matvec, xi, N, eig_min, eig_max, n_terms):
    """The series of brownian_system.C:1036-1108 for right-hand sides xi
    [r][3n], stopped after n_terms terms (the report's n_terms: y holds the
    coefficients 0 .. n_terms), with the order-N coefficients of
    chebyshev.C:44-151 (Gauss).  matvec maps [r][3n] -> [r][3n].
    Returns y and err1 = sqrt(|M y|^2 - xi . M xi| / xi . M xi) per
    right-hand side (brownian_system.C:1117-1125)."""
    d = eig_max - eig_min
    da, db = 2.0 / d, -(eig_max + eig_min) / d
    X = O.cheb_coeffs(N, da, db)
    x0 = xi.copy()
    m0 = matvec(x0)
    aux2 = np.sum(m0 * x0, axis=-1)
    x1 = db * x0 + da * m0
    y = X[0] * x0 + X[1] * x1
    for i in range(1, n_terms):
        xm = 2.0 * db * x1 + 2.0 * da * matvec(x1) - x0
        y = y + X[i + 1] * xm
        x0, x1 = x1, xm
    my = matvec(y)
    err1 = np.sqrt(np.abs(np.sum(my * my, axis=-1) - aux2) / aux2)
    return y, err1, my


# --------------------------------------------------------------------------
# N = 1000 beads, phi = 0.05, order 30, Lanczos bounds
# --------------------------------------------------------------------------
CFG1_N, CFG1_PHI, CFG1_ORDER, CFG1_SEED = 1000, 0.05, 30, 1001


def _dense(c, box, xyz, nb):
    n = len(xyz)
    E = np.eye(3 * n).reshape(3 * n, n, 3)
    return O.local_matvec(c, box, xyz, nb, E, O.SELF_BEAD, nthreads=THREADS).reshape(
        3 * n, 3 * n).T


def _cfg1_mode(mode):
    xyz, L = G.make_suspension(CFG1_SEED, CFG1_N, CFG1_PHI)
    assert abs(L - 43.75) < 0.05
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    if mode == "cutoff":
        nb = O.neighbors_cutoff(box, xyz, RC)
        kw = dict(rc=RC)
        want_off, want_ids = nb.offsets, nb.ids
    else:
        # element mesh of side h = L / floor(L / 1.414) (h <= 1/(sqrt(2) alpha)
        # of the reference's tutorial, rounded to whole elements) and the
        # element search radius 0.5 hmax + 4/alpha with hmax the longest edge
        # (copss.C:989-992, :1074-1075)
        nm = int(np.floor(L / 1.414))
        h = L / nm
        sre = 0.5 * h + 4.0 / ALPHA
        mesh = O.make_mesh(nm, nm, nm, sre)
        nb = O.neighbors_reference(box, mesh, xyz)
        kw = dict(nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3, search_radius_e=sre)
        wl = [np.sort(x) for x in nb.lists()]
        want_off = np.concatenate([[0], np.cumsum([len(x) for x in wl])])
        want_ids = np.concatenate(wl)
    return xyz, L, box, nb, kw, want_off, want_ids


@pytest.mark.parametrize("mode", ["cutoff", "reference", "cutoff-list"])
def test_cfg1_lists_matvec_and_faithful_series(mode):
    t0 = time.perf_counter()
    xyz, L, box, nb, kw, want_off, want_ids = _cfg1_mode(mode.split("-")[0])
    c = O.constants(alpha=ALPHA)
    n = len(xyz)
    f = np.random.default_rng(5).standard_normal((n, 3))
    u_o = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=THREADS)
    w = np.linalg.eigvalsh(_dense(c, box, xyz, nb))
    assert w[0] > 0
    # the reference's noise stream (random_generator.C:43-67)
    xi = O.std_normal_vector(123456789, 3 * n)
    with G.Context(alpha=ALPHA, box_hi=(L,) * 3, precision=G.FP64, **kw) as ctx:
        if mode == "cutoff-list":  # the FP64 pair kernel over the exact list
            ctx.set_fp64_pair_list(True)
        ctx.set_particles(xyz)
        ctx.build_cells()
        off, ids = ctx.neighbors()
        assert np.array_equal(off, want_off) and np.array_equal(ids, want_ids)
        u = ctx.local_matvec(f, G.SELF_BEAD)
        assert rel(u, u_o) <= FP64_TOL
        lo, hi = ctx.lanczos_bounds(k=60, seed=3)
        # Ritz values lie inside the spectrum, near its ends
        print(f"cfg1 {mode}: Lanczos(60) [{lo:.6f}, {hi:.6f}], dense [{w[0]:.6f}, {w[-1]:.6f}]")
        assert w[0] * (1 - 1e-9) <= lo <= w[0] * 1.25
        assert w[-1] * (1 - 1e-2) <= hi <= w[-1] * (1 + 1e-9)
        lmin, lmax = lo / 1.05, hi * 1.05  # eig_factor widening (copss.C:1607)
        y, rep = ctx.cheb_inv_sqrt(xi, CFG1_ORDER, lmin, lmax, 1e-3, check_every=1)
        rc, dw, rep_dw = ctx.brownian_displacement(xi, CFG1_ORDER, lmin, lmax, 1e-3,
                                                   check_every=1)
        assert rc == 0
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, THREADS))
    y_o, rep_o = O.cheb_inv_sqrt(op, xi, CFG1_ORDER, lmin, lmax, 1e-3)
    r = rep[0]
    print(f"cfg1 {mode}: {r}, oracle terms {rep_o.n_terms} err1 {rep_o.err1:.3e}")
    assert rep_o.converged == 1
    assert r["converged"] == rep_o.converged and r["n_terms"] == rep_o.n_terms
    assert r["n_matvecs"] == rep_o.n_matvecs
    # err1^2 = |M y|^2 / xi.M xi - 1 is the difference of two nearly equal
    # FP64 sums: whatever the summation order its absolute error is ~1e-15,
    # so err1 carries ~1e-15 / (2 err1) (2e-12 at err1 = 3e-4)
    assert abs(r["err1"] - rep_o.err1) <= max(1e-8 * rep_o.err1, 1e-13 / rep_o.err1)
    assert r["err2"] == pytest.approx(rep_o.err2, rel=1e-8)
    assert rel(y, y_o) <= 1e-11
    # hi_ewald: dw = M y (copss.C:1686)
    dw_o = O.local_matvec(c, box, xyz, nb, y_o, O.SELF_BEAD, nthreads=THREADS)
    assert rel(dw, dw_o) <= 1e-11
    _timed(f"cfg1 {mode}", t0)


def test_cfg1_fp32_series_against_oracle():
    """The same workload on the FP32 pair sum with the adaptive single check
    (the benchmark's mode): y within the FP32 operator's error of the
    oracle's series run to the same number of terms."""
    xyz, L, box, nb, kw, _, _ = _cfg1_mode("cutoff")
    c = O.constants(alpha=ALPHA)
    n = len(xyz)
    xi = O.std_normal_vector(987654321, 3 * n)
    with G.Context(alpha=ALPHA, box_hi=(L,) * 3, precision=G.FP32, **kw) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=60, seed=3)
        lmin, lmax = lo / 1.05, hi * 1.05
        rc, dw, rep = ctx.brownian_displacement(xi, CFG1_ORDER, lmin, lmax, 1e-3, check_every=0)
        assert rc == 0
    T = rep[0]["n_terms"]

    def mv(v):
        return O.local_matvec(c, box, xyz, nb, v.reshape(-1, n, 3), O.SELF_BEAD,
                              nthreads=THREADS).reshape(v.shape)

    y_o, err1_o, dw_o = cheb_fixed_terms(mv, xi.reshape(1, -1), CFG1_ORDER, lmin, lmax, T)
    print(f"cfg1 FP32 adaptive: {rep[0]}, oracle err1 at {T} terms {err1_o[0]:.3e}")
    assert rep[0]["err1"] <= 1e-3 and err1_o[0] <= 1e-3
    assert abs(rep[0]["err1"] - err1_o[0]) <= 2e-4
    assert rel(dw.reshape(-1), dw_o.reshape(-1)) <= 1e-5


# --------------------------------------------------------------------------
# N = 200k beads, phi = 0.1
# --------------------------------------------------------------------------
def test_cfg2_N200k_lists_fp64_and_fp32_matvecs():
    t0 = time.perf_counter()
    xyz, L = G.make_suspension(20261203, 200_000, 0.1)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=ALPHA)
    nb = O.neighbors_cutoff(box, xyz, RC)
    f = np.random.default_rng(17).standard_normal((len(xyz), 3))
    u_o = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=THREADS)
    _timed("cfg2 oracle", t0)
    # FP64 with the cell sweep, FP64 over the exact pair list, FP32
    for prec, f64_list in ((G.FP64, False), (G.FP64, True), (G.FP32, False)):
        with G.Context(alpha=ALPHA, box_hi=(L,) * 3, rc=RC, precision=prec) as ctx:
            if f64_list:
                ctx.set_fp64_pair_list(True)
            ctx.set_particles(xyz)
            ctx.build_cells()
            off, ids = ctx.neighbors()
            assert np.array_equal(off, nb.offsets) and np.array_equal(ids, nb.ids)
            assert ctx.pair_count() == nb.offsets[-1]
            u = ctx.local_matvec(f, G.SELF_BEAD)
        err = rel(u, u_o)
        comp = np.abs(u - u_o).max() / np.abs(u_o).max()
        per = np.abs(u - u_o) / np.maximum(np.abs(u_o), 1e-300)
        print(f"cfg2 precision {prec} (pair list {f64_list or prec == G.FP32}): "
              f"pairs {nb.offsets[-1]}, norm-wise {err:.2e}, "
              f"max component {comp:.2e} of the largest, median per-component relative "
              f"{np.median(per):.2e}, 99.9th percentile {np.percentile(per, 99.9):.2e}")
        assert err <= (FP64_TOL if prec == G.FP64 else FP32_TOL)
    _timed("cfg2", t0)


# --------------------------------------------------------------------------
# 5000 chains x 20 beads, 64 right-hand sides
# --------------------------------------------------------------------------
def test_cfg3_chains_64rhs_matvec_and_adaptive_series():
    t0 = time.perf_counter()
    xyz, L = G.make_chains(20261210, 5000, 20, 2.0, 0.05)
    n = len(xyz)
    assert n == 100_000
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=ALPHA)
    nb = O.neighbors_cutoff(box, xyz, RC)
    R = 64
    rng = np.random.default_rng(23)
    f = rng.standard_normal((R, n, 3))
    u_o = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=THREADS)
    xi = rng.standard_normal((R, 3 * n))
    with G.Context(alpha=ALPHA, box_hi=(L,) * 3, rc=RC, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        off, ids = ctx.neighbors()
        assert np.array_equal(off, nb.offsets) and np.array_equal(ids, nb.ids)
        u = ctx.local_matvec(f, G.SELF_BEAD)
        errs = [rel(u[r], u_o[r]) for r in range(R)]
        print(f"cfg3 64-RHS matvec: worst right-hand side {max(errs):.2e}")
        assert max(errs) <= FP32_TOL
        lo, hi = ctx.lanczos_bounds(k=24, seed=7)
        lmin, lmax = lo / 1.05, hi * 1.05
        for _ in range(2):  # the adaptive schedule learns the degree, as in a run
            rc, dw, rep = ctx.brownian_displacement(xi, 50, lmin, lmax, 1e-3, check_every=0)
            assert rc == 0
    assert all(r["converged"] and r["err1"] <= 1e-3 for r in rep)
    sample = [0, 21, 42, 63]

    def mv(v):
        return O.local_matvec(c, box, xyz, nb, v.reshape(-1, n, 3), O.SELF_BEAD,
                              nthreads=THREADS).reshape(v.shape)

    dwr = dw.reshape(R, -1)
    for r in sample:
        T = rep[r]["n_terms"]
        y_o, err1_o, dw_o = cheb_fixed_terms(mv, xi[r:r + 1], 50, lmin, lmax, T)
        e = rel(dwr[r], dw_o[0])
        print(f"cfg3 series rhs {r}: {T} terms, err1 {rep[r]['err1']:.3e} "
              f"(oracle {err1_o[0]:.3e}), dw error {e:.2e}")
        assert abs(rep[r]["err1"] - err1_o[0]) <= 2e-4
        assert e <= 1e-5
    _timed("cfg3", t0)


# --------------------------------------------------------------------------
# 512 uneven suspensions x 8 right-hand sides
# --------------------------------------------------------------------------
def _cfg4_suspensions(seed=20261214, K=512):
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(500), np.log(20000), K)).astype(np.int64)
    phis = rng.uniform(0.02, 0.2, K)
    with ThreadPoolExecutor(THREADS) as ex:
        sus = list(ex.map(lambda b: G.make_suspension(seed * 7 + b, int(ns[b]), float(phis[b])),
                          range(K)))
    return sus, ns, phis


def test_cfg4_all_512_suspensions_matvec_and_series():
    import torch
    from concurrent.futures import ThreadPoolExecutor
    t0 = time.perf_counter()
    sus, ns, phis = _cfg4_suspensions()
    K, R = len(sus), 8
    c = O.constants(alpha=ALPHA)
    rng = np.random.default_rng(29)
    f = rng.standard_normal((int(ns.sum()), R, 3))
    xi = rng.standard_normal((int(ns.sum()), R, 3))
    off = np.concatenate([[0], np.cumsum(ns)])
    pick = {"smallest": int(np.argmin(ns)), "largest": int(np.argmax(ns)),
            "densest": int(np.argmax(phis))}
    with G.Ensemble([L for _, L in sus]) as ens:
        d_xyz = torch.from_numpy(np.concatenate([x for x, _ in sus]).reshape(-1)).cuda()
        ens.set_particles_dev(ns, d_xyz.data_ptr())
        d_f = torch.from_numpy(f.reshape(-1)).cuda()
        d_u = torch.empty_like(d_f)
        ens.matvec_dev(R, d_f.data_ptr(), d_u.data_ptr(), G.SELF_BEAD)
        u = d_u.cpu().numpy().reshape(-1, R, 3)
        bounds = [ens.lanczos(b, 24, 7) for b in range(K)]
        lo = np.array([x[0] for x in bounds]) / 1.05
        hi = np.array([x[1] for x in bounds]) * 1.05
        d_xi = torch.from_numpy(xi.reshape(-1)).cuda()
        d_dw = torch.empty_like(d_xi)
        for _ in range(2):
            rc, reps = ens.brownian_dev(R, 50, lo, hi, 1e-3, d_xi.data_ptr(), d_dw.data_ptr())
            assert rc == 0
        dw = d_dw.cpu().numpy().reshape(-1, R, 3)
    _timed("cfg4 device", t0)

    def check(b):
        xyz, L = sus[b]
        n = len(xyz)
        box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
        nb = O.neighbors_cutoff(box, xyz, RC)
        fb = np.transpose(f[off[b]:off[b + 1]], (1, 0, 2))
        want = O.local_matvec(c, box, xyz, nb, fb, O.SELF_BEAD, nthreads=1)
        got = np.transpose(u[off[b]:off[b + 1]], (1, 0, 2))
        return b, max(rel(got[r], want[r]) for r in range(R))

    with ThreadPoolExecutor(THREADS) as ex:
        worst = list(ex.map(check, range(K)))
    e_max = max(e for _, e in worst)
    print(f"cfg4 matvec: {K} suspensions, {int(ns.sum())} beads, worst right-hand side "
          f"{e_max:.2e} (suspension {max(worst, key=lambda t: t[1])[0]})")
    assert e_max <= FP32_TOL
    for name, b in pick.items():
        xyz, L = sus[b]
        n = len(xyz)
        box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
        nb = O.neighbors_cutoff(box, xyz, RC)

        def mv(v, xyz=xyz, box=box, nb=nb, n=n):
            return O.local_matvec(c, box, xyz, nb, v.reshape(-1, n, 3), O.SELF_BEAD,
                                  nthreads=THREADS).reshape(v.shape)

        assert all(r["converged"] for r in reps[b])
        xib = np.transpose(xi[off[b]:off[b + 1]], (1, 0, 2)).reshape(R, -1)
        got = np.transpose(dw[off[b]:off[b + 1]], (1, 0, 2)).reshape(R, -1)
        e, d1 = 0.0, 0.0
        for T in sorted({r["n_terms"] for r in reps[b]}):
            rs = [r for r in range(R) if reps[b][r]["n_terms"] == T]
            _, err1_o, dw_o = cheb_fixed_terms(mv, xib[rs], 50, lo[b], hi[b], T)
            for k, r in enumerate(rs):
                e = max(e, rel(got[r], dw_o[k]))
                d1 = max(d1, abs(reps[b][r]["err1"] - err1_o[k]))
        terms = [r["n_terms"] for r in reps[b]]
        print(f"cfg4 series, {name} suspension {b} (N={n}, phi={phis[b]:.3f}): terms {terms}, "
              f"dw error {e:.2e}, err1 difference {d1:.1e}")
        assert e <= 1e-5 and d1 <= 2e-4
    _timed("cfg4", t0)


# --------------------------------------------------------------------------
# the shipped eigen-interval network on its held-out configurations
# --------------------------------------------------------------------------
def test_cfg5_shipped_network_held_out_coverage():
    from ggem_gb300 import surrogate_data as SD
    loaded = SD.load_default()
    if loaded is None:
        pytest.fail("the trained network is not shipped")
    sur, margins, summary = loaded
    t0 = time.perf_counter()
    total, hold = summary["configs"], summary["n_holdout"]
    cfgs = SD.sample_configs(total, summary["seed"], **SD.range_kwargs(summary))[total - hold:]
    X, Y = SD.label(cfgs, k=summary["lanczos_k"], threads=THREADS)
    P = sur.predict(X)
    inside = (P[:, 0] - margins[0] <= Y[:, 0]) & (P[:, 1] + margins[1] >= Y[:, 1])
    cover = float(inside.mean())
    rmse = np.sqrt(((P - Y) ** 2).mean(axis=0))
    print(f"cfg5: {hold} held-out configurations, coverage {cover:.4f} "
          f"(training run: {summary['holdout_coverage']:.4f}), RMSE {rmse}")
    assert cover >= summary["holdout_coverage"] - 0.005
    assert cover >= 0.97
    sur.close()
    _timed("cfg5", t0)
