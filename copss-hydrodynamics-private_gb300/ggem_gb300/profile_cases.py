"""Small, self-contained runs of single kernels, for profiling.

Each case builds one workload, launches the kernel it is named after a few
times (the first launch is a warm-up that ``ncu -s 1`` skips) and exits 0.
The cases are sized so that a full ``ncu --set full`` capture of one launch
finishes in a minute or two while the inputs stay larger than L2.

    python copss-hydrodynamics-private_gb300/ggem_gb300/profile_cases.py <case>

cases:
  pair_cheb   k_pair_first / k_pair_cheb: two Brownian steps of a 200k-bead
              suspension (phi = 0.1, rc = 7), 10-ish fused Chebyshev terms each,
              tensors evaluated per pair
  pair_tv     k_pair_first / k_pair_cheb_tv: the same with stored pair tensors
  pair_r1     k_pair_r1: 6 plain FP32 matvecs of the same suspension
  list        k_pair_list_warp: 3 list builds of the same suspension
  pair_f64    k_pair_list_f64: 3 FP64 matvecs over the exact pair list
  spread      k_spread_brick: FP32, FP32, FP64 element spreads of 25k beads
              onto the 8 Gauss points of each of 72^3 HEX20 elements
  mlp         k_mlp_forward: 3 predictions of 512 rows of the eigen network
  ens         k_ens_series: 3 ensemble steps of 64 suspensions, 8 RHS each
  ens_term    k_ens_pair: the same steps as one launch per term
  all         every kernel family of the library once, on a 20k-bead suspension
              (and small ensemble / network / FEM cases), for a per-kernel
              counter table
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import ggem_gb300 as G  # noqa: E402
from ggem_gb300 import build as B  # noqa: E402

N_BENCH, PHI_BENCH, SEED_BENCH = 200_000, 0.1, 20261203


def _torch():
    import torch
    return torch


def _bench_suspension():
    return G.make_suspension(SEED_BENCH, N_BENCH, PHI_BENCH)


def pair_cheb() -> None:
    torch = _torch()
    xyz, L = _bench_suspension()
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    ctx.set_pair_tensors(False)  # tensors per pair, the form the bench's autotuner keeps
    ctx.set_particles(xyz)
    ctx.build_cells()
    lo, hi = ctx.lanczos_bounds(k=24, seed=7)
    xi = torch.randn(3 * len(xyz), dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    for _ in range(2):
        rc, rep = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), 1, 50, lo / 1.05,
                                                hi * 1.05, 1e-3, check_every=0)
    ctx.synchronize()
    print("rc", rc, rep)


def pair_tv() -> None:
    torch = _torch()
    xyz, L = _bench_suspension()
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    ctx.set_pair_tensors(True)
    ctx.set_particles(xyz)
    ctx.build_cells()
    lo, hi = ctx.lanczos_bounds(k=24, seed=7)
    xi = torch.randn(3 * len(xyz), dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    for _ in range(2):
        rc, rep = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), 1, 50, lo / 1.05,
                                                hi * 1.05, 1e-3, check_every=0)
    ctx.synchronize()
    print("rc", rc, rep)


def pair_r1() -> None:
    torch = _torch()
    xyz, L = _bench_suspension()
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    ctx.set_pair_tensors(False)
    ctx.set_particles(xyz)
    ctx.build_cells()
    f = torch.randn(3 * len(xyz), dtype=torch.float64, device="cuda")
    u = torch.empty_like(f)
    for _ in range(6):
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
    ctx.synchronize()
    print("ok")


def list_build() -> None:
    xyz, L = _bench_suspension()
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    for _ in range(3):
        ctx.set_particles(xyz)
        ctx.build_cells()
    ctx.synchronize()
    print("pairs", ctx.pair_count())


def pair_f64() -> None:
    torch = _torch()
    xyz, L = _bench_suspension()
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64)
    ctx.set_fp64_pair_list(True)
    ctx.set_particles(xyz)
    ctx.build_cells()
    f = torch.randn(3 * len(xyz), dtype=torch.float64, device="cuda")
    u = torch.empty_like(f)
    for _ in range(3):
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
    ctx.synchronize()
    print("ok")


def spread() -> None:
    torch = _torch()
    xyz, L = G.make_suspension(3, 25000, 0.1)
    nm = int(np.ceil(L / 1.414))
    h = L / nm
    ctx = G.Context(box_hi=(L,) * 3, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                    search_radius_e=0.5 * h + 8.0, precision=G.FP64)
    ctx.set_particles(xyz)
    ctx.build_cells()
    g = [0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)]
    loc = np.array([[g[a], g[b], g[c]] for c in range(2) for b in range(2) for a in range(2)])
    ez, ey, ex = np.meshgrid(np.arange(nm), np.arange(nm), np.arange(nm), indexing="ij")
    base = np.stack([ex.ravel(), ey.ravel(), ez.ravel()], axis=1)
    q = ((base[:, None, :] + loc[None]) * h).reshape(-1, 3)
    ctx.set_quadrature(q, 8)
    f = torch.randn(3 * len(xyz), dtype=torch.float64, device="cuda")
    rho = torch.empty(3 * len(q), dtype=torch.float64, device="cuda")
    for prec in (G.FP32, G.FP32, G.FP64):
        ctx.spread_elements_dev(f.data_ptr(), rho.data_ptr(), prec)
    ctx.synchronize()
    print("nm", nm, "points", len(q))


def mlp() -> None:
    sur = G.Surrogate(seed=3)
    X = np.random.default_rng(1).standard_normal((512, 35)).astype(np.float32)
    for _ in range(3):
        sur.predict(X)
    print("ok")


def ens(persistent=True) -> None:
    torch = _torch()
    rng = np.random.default_rng(5)
    K = 64
    ns = np.exp(rng.uniform(np.log(500), np.log(20000), K)).astype(np.int64)
    phis = rng.uniform(0.02, 0.2, K)
    sus = [G.make_suspension(100 + b, int(ns[b]), float(phis[b])) for b in range(K)]
    e = G.Ensemble([L for _, L in sus])
    d_xyz = torch.from_numpy(np.concatenate([x for x, _ in sus]).reshape(-1)).cuda()
    e.set_particles_dev(ns, d_xyz.data_ptr())
    e.set_series_mode(persistent=persistent)
    beads, pairs = e.sizes()
    lz = [e.lanczos(b, 24, 7) for b in range(K)]
    lo = np.array([x[0] for x in lz]) / 1.05
    hi = np.array([x[1] for x in lz]) * 1.05
    xi = torch.randn(beads * 8 * 3, dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    for _ in range(3):
        rc, _ = e.brownian_dev(8, 50, lo, hi, 1e-3, xi.data_ptr(), dw.data_ptr())
    torch.cuda.synchronize()
    print("beads", beads, "pairs", pairs, "rc", rc)


def all_kernels() -> None:
    torch = _torch()
    import ctypes as C
    rng = np.random.default_rng(1)
    xyz, L = G.make_suspension(11, 20000, 0.1)
    n = len(xyz)
    f = rng.standard_normal((n, 3))
    failures = []

    def run(name, fn):
        try:
            fn()
        except Exception as exc:  # keep going: the table lists what ran
            failures.append(f"{name}: {exc}")

    # FP32 cut-off context: cell build, pair list, the pair kernels of 1, 8
    # and 64 right-hand sides, both Chebyshev schedules, Lanczos, power
    # iteration, Philox, network features, forces
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as c:
        c.set_pair_tensors(False)
        c.set_particles(xyz)
        c.build_cells()
        run("matvec 1", lambda: c.local_matvec(f))
        run("matvec 8", lambda: c.local_matvec(rng.standard_normal((8, n, 3))))
        run("matvec 64", lambda: c.local_matvec(rng.standard_normal((64, n, 3))))
        lo, hi = c.lanczos_bounds(k=24, seed=7)
        xi = rng.standard_normal(3 * n)
        run("series adaptive", lambda: c.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05, 1e-3,
                                                               check_every=0))
        run("series faithful", lambda: c.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05,
                                                               1e-3, check_every=1))
        run("series 64", lambda: c.cheb_inv_sqrt(rng.standard_normal(64 * 3 * n), 50,
                                                 lo / 1.05, hi * 1.05, 1e-3, check_every=0))
        run("power", lambda: c.power_iteration(tol=1e-2, maxits=200))
        run("features", lambda: c.surrogate_features())
        d = torch.empty(3 * n, dtype=torch.float64, device="cuda")
        run("philox", lambda: c.philox_normals_dev(1, 2, 3 * n, d.data_ptr()))
        run("ev forces", lambda: c.ev_gaussian_forces(0.37, 0.21))
        c.set_pair_tensors(True)
        c.build_cells()
        run("stored", lambda: c.local_matvec(f))
        c.synchronize()
    # chains: spring forces
    cxyz, cL = G.make_chains(5, 500, 20)
    with G.Context(box_hi=(cL,) * 3, rc=7.0, precision=G.FP64) as c:
        c.set_particles(cxyz)
        c.build_cells()
        bonds = np.array([(20 * k + j, 20 * k + j + 1) for k in range(500) for j in range(19)])
        c.set_bonds(bonds)
        run("springs", lambda: c.spring_forces(G.SPRING_FENE, 1.0, 3.0))
    # FP64 cut-off context: the cell sweep, the exact-list kernel, the field
    # points, the per-point spread and element right-hand sides
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as c:
        c.set_particles(xyz)
        c.build_cells()
        run("fp64 sweep", lambda: c.local_matvec(f))
        c.set_fp64_pair_list(True)
        c.build_cells()
        run("fp64 list", lambda: c.local_matvec(f))
        t = rng.uniform(0, L, (20000, 3))
        run("field", lambda: c.local_field(t, f))
        run("spread qp", lambda: c.spread_qp(t, f, spread_rc=8.0))
    # reference mode: the element spread (FP32 and FP64 bricks)
    nm = int(np.ceil(L / 1.414))
    h = L / nm
    with G.Context(box_hi=(L,) * 3, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                   search_radius_e=0.5 * h + 8.0, precision=G.FP64) as c:
        c.set_particles(xyz)
        c.build_cells()
        g = [0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)]
        loc = np.array([[g[a], g[b], g[cc]] for cc in range(2) for b in range(2) for a in range(2)])
        ez, ey, ex = np.meshgrid(np.arange(nm), np.arange(nm), np.arange(nm), indexing="ij")
        base = np.stack([ex.ravel(), ey.ravel(), ez.ravel()], axis=1)
        q = ((base[:, None, :] + loc[None]) * h).reshape(-1, 3)
        c.set_quadrature(q, 8)
        run("spread fp32", lambda: c.spread_elements(f, G.FP32))
        run("spread fp64", lambda: c.spread_elements(f, G.FP64))
        run("reference matvec", lambda: c.local_matvec(f))
    # FEM values at the particles (a trivial dof map: 3 x 20 own dofs per element)
    ne = (8, 8, 8)
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP64) as c:
        c.set_particles(xyz)
        ne_tot = int(np.prod(ne))
        dofs = np.arange(60 * ne_tot, dtype=np.int64).reshape(ne_tot, 3, 20)
        sol = rng.standard_normal(60 * ne_tot)

        def fem():
            with G.Fem(c, ne, (0, 0, 0), (L, L, L), 60 * ne_tot, dofs) as fe:
                fe.point_values(sol)
        run("fem", fem)
    # the network: a prediction and one short training run
    sur = G.Surrogate(seed=3)
    X = rng.standard_normal((512, G.SUR_FEATURES)).astype(np.float32)
    Y = rng.standard_normal((512, G.SUR_OUTPUTS)).astype(np.float32)
    run("predict", lambda: sur.predict(X))
    run("train", lambda: sur.train(X, Y, 1, batch=256))
    sur.close()
    # a small ensemble, both step forms
    K = 8
    sus = [G.make_suspension(100 + b, 2000 + 500 * b, 0.1) for b in range(K)]
    e = G.Ensemble([Lb for _, Lb in sus])
    d_xyz = torch.from_numpy(np.concatenate([x for x, _ in sus]).reshape(-1)).cuda()
    e.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
    beads, _ = e.sizes()
    lz = [e.lanczos(b, 24, 7) for b in range(K)]
    elo = np.array([x[0] for x in lz]) / 1.05
    ehi = np.array([x[1] for x in lz]) * 1.05
    exi = torch.randn(beads * 8 * 3, dtype=torch.float64, device="cuda")
    edw = torch.empty_like(exi)
    for pers in (True, False):
        e.set_series_mode(persistent=pers)
        run(f"ensemble {pers}", lambda: e.brownian_dev(8, 50, elo, ehi, 1e-3, exi.data_ptr(),
                                                        edw.data_ptr()))
    run("ensemble matvec", lambda: e.matvec_dev(8, exi.data_ptr(), edw.data_ptr()))
    e.close()
    # the entry point without allocations
    fn = G.lib().ggem_local_matvec_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(G.Params), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p]
    sx, sL = G.make_suspension(12, 3000, 0.1)
    p = G.default_params()
    for k in range(3):
        p.box_lo[k], p.box_hi[k], p.periodic[k] = 0.0, sL, 1
    p.nb_mode, p.rc, p.precision = G.NB_CUTOFF, 7.0, G.FP64
    dx = torch.from_numpy(sx.reshape(-1)).cuda()
    df = torch.randn(3 * len(sx), dtype=torch.float64, device="cuda")
    du = torch.empty_like(df)
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    run("noalloc", lambda: fn(C.byref(p), len(sx), dx.data_ptr(), df.data_ptr(), du.data_ptr(),
                              G.SELF_BEAD, st.data_ptr(), None))
    torch.cuda.synchronize()
    print("failures:", failures if failures else "none")


CASES = {"pair_cheb": pair_cheb, "pair_tv": pair_tv, "pair_r1": pair_r1, "list": list_build,
         "pair_f64": pair_f64, "spread": spread, "mlp": mlp, "ens": ens,
         "ens_term": lambda: ens(persistent=False), "all": all_kernels}


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1 or argv[0] not in CASES:
        print(__doc__)
        return 2
    B.build()
    CASES[argv[0]]()
    return 0


if __name__ == "__main__":
    sys.exit(main())
