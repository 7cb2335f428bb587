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


CASES = {"pair_cheb": pair_cheb, "pair_tv": pair_tv, "pair_r1": pair_r1, "list": list_build,
         "pair_f64": pair_f64, "spread": spread, "mlp": mlp, "ens": ens,
         "ens_term": lambda: ens(persistent=False)}


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
