"""The fused Brownian series' prefix as a CUDA graph (ggem_set_series_graphs):
a run of steps with the graph (live first call, capture on the repeat,
replays after) gives bit-identical displacements and identical reports to
the same steps issued live, through rebuilt lists (a deferred list check in
every step), a change of eigen interval (a new key), a step that needs more
terms than the prefix holds, and with the kernel timer on.  The launch
count and the timer's launch count follow the replays."""
import numpy as np
import pytest
import torch

import ggem_gb300 as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()


def _run(graphs, timing, xyz, L, schedule):
    """schedule: list of (eig_min, eig_max, xi seed); returns dw per step,
    reports, launches, timer (ms, launches), graph stats"""
    n = len(xyz)
    ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    ctx.set_pair_tensors(False)
    ctx.set_series_graphs(graphs)
    d_xyz = torch.from_numpy(xyz.reshape(-1).copy()).cuda()
    ctx.set_particles_dev(d_xyz.data_ptr(), n)
    ctx.build_cells()
    ctx.set_deferred_checks(True)
    xi = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    out, reps = [], []
    ctx.set_kernel_timing(timing, kinds=[G.KERNEL_PAIR_CHEB] if timing else None)
    l0 = ctx.launch_count()
    for lo, hi, seed in schedule:
        ctx.set_particles_dev(d_xyz.data_ptr(), n)
        ctx.build_cells()
        ctx.philox_normals_dev(11, seed, 3 * n, xi.data_ptr())
        rc, rep = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), 1, 50, lo, hi, 1e-3,
                                                check_every=0)
        assert rc == 0, rep
        out.append(dw.cpu().numpy().copy())
        reps.append(rep[0])
    launches = ctx.launch_count() - l0
    timer = ctx.kernel_timing(G.KERNEL_PAIR_CHEB) if timing else None
    stats = ctx.series_graph_stats()
    ctx.close()
    return out, reps, launches, timer, stats


def test_series_graph_matches_live_steps():
    xyz, L = G.make_suspension(77, 20000, 0.1)
    probe = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    probe.set_particles(xyz)
    probe.build_cells()
    lo, hi = probe.lanczos_bounds(k=24, seed=7)
    probe.close()
    a, b = lo / 1.05, hi * 1.05
    # the same interval for a while (capture, replays), a wider one (a new
    # key; its first step needs more terms than the degree predicted from
    # the narrower interval, so the series runs past the prefix's check),
    # then back
    sched = [(a, b, s) for s in range(5)] + [(a / 2, b * 2, s) for s in range(5, 9)]
    sched += [(a, b, s) for s in range(9, 12)]
    for timing in (False, True):
        live = _run(False, timing, xyz, L, sched)
        graph = _run(True, timing, xyz, L, sched)
        for k, (u, v) in enumerate(zip(live[0], graph[0])):
            assert np.array_equal(u, v), (timing, k)
        assert live[1] == graph[1], timing
        assert live[2] == graph[2], (timing, live[2], graph[2])
        captures, replays = graph[4]
        assert live[4] == (0, 0)
        assert captures >= 2 and replays >= 4, graph[4]
        if timing:
            assert live[3][1] == graph[3][1], (live[3], graph[3])
            assert graph[3][0] > 0
            print(f"fused terms: live {live[3][0] / live[3][1] * 1e3:.1f} us, "
                  f"graph {graph[3][0] / graph[3][1] * 1e3:.1f} us per launch")
        terms = sorted({r["n_terms"] for r in graph[1]})
        print(f"timing={timing}: {captures} captures, {replays} replays, terms {terms}")


def test_replayed_prefix_then_live_terms():
    """a replayed prefix whose check fails (a tighter tolerance: the key does
    not hold the tolerance) continues live; the steps equal the live run's"""
    xyz, L = G.make_suspension(78, 12000, 0.1)
    probe = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
    probe.set_particles(xyz)
    probe.build_cells()
    lo, hi = probe.lanczos_bounds(k=24, seed=7)
    probe.close()
    a, b = lo / 1.05, hi * 1.05
    n = len(xyz)
    res = {}
    for graphs in (False, True):
        ctx = G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32)
        ctx.set_pair_tensors(False)
        ctx.set_series_graphs(graphs)
        d_xyz = torch.from_numpy(xyz.reshape(-1).copy()).cuda()
        xi = torch.empty(3 * n, dtype=torch.float64, device="cuda")
        dw = torch.empty_like(xi)
        outs, reps = [], []
        for seed, tol in ((0, 1e-3), (1, 1e-3), (2, 1e-3), (3, 2e-4), (4, 1e-3)):
            ctx.set_particles_dev(d_xyz.data_ptr(), n)
            ctx.build_cells()
            ctx.philox_normals_dev(5, seed, 3 * n, xi.data_ptr())
            rc, rep = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), 1, 50, a, b,
                                                    tol, check_every=0)
            assert rc == 0, rep
            outs.append(dw.cpu().numpy().copy())
            reps.append(rep[0])
        res[graphs] = (outs, reps, ctx.series_graph_stats())
        ctx.close()
    for u, v in zip(res[False][0], res[True][0]):
        assert np.array_equal(u, v)
    assert res[False][1] == res[True][1]
    # the tight step ran past the prefix's check
    assert res[True][1][3]["n_terms"] > res[True][1][2]["n_terms"], res[True][1]
    assert res[True][2][1] >= 2, res[True][2]
    print("terms", [r["n_terms"] for r in res[True][1]], "graph stats", res[True][2])
