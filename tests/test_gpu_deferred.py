"""Deferred list checks (ggem_set_deferred_checks): a rebuild that returns
without waiting for the device must give the same results as the
synchronous build, rebuild the list itself when its rows overflowed, and
report a build error at the call that reads it."""
import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def configs():
    """a dilute suspension, then a suspension eight times denser in one
    eighth of the box (rows about eight times longer, no overlaps), then the
    dilute one shifted"""
    xyz, L = G.make_suspension(91, 3000, 0.03)
    dense, _ = G.make_suspension(92, 3000, 0.24)
    return L, [xyz, dense, np.mod(xyz + 0.37, L)]


def run(ctx, xyz, xi, bounds):
    ctx.set_particles(xyz)
    ctx.build_cells()
    lo, hi = bounds
    return ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=0)


def test_deferred_matches_synchronous_and_rebuilds_overflowing_rows():
    L, cfgs = configs()
    xi = np.random.default_rng(3).standard_normal(3 * len(cfgs[0]))
    # eigenvalue intervals from a synchronous context (Lanczos reads the
    # statistics itself, so the deferred run must not call it)
    bounds = []
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        for xyz in cfgs:
            ctx.set_particles(xyz)
            ctx.build_cells()
            lo, hi = ctx.lanczos_bounds(k=30, seed=3)
            bounds.append((lo / 1.05, hi * 1.05))
    out = {}
    for deferred in (False, True):
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
            ctx.set_deferred_checks(deferred)
            res = []
            for xyz, bd in zip(cfgs, bounds):
                rc, dw, rep = run(ctx, xyz, xi, bd)
                assert rc == 0, rep
                res.append((dw, rep[0]["n_terms"], ctx.pair_count(), ctx.pair_storage()[0]))
            out[deferred] = res
    for (dw0, t0, p0, w0), (dw1, t1, p1, w1) in zip(out[False], out[True]):
        # the same row width after the overflow is repaired, so the same sums
        assert w0 == w1 and p0 == p1 and t0 == t1
        assert np.array_equal(dw0, dw1)
    # the dense configuration did overflow the dilute rows
    assert out[True][1][3] > out[True][0][3]


def test_deferred_build_then_matvec_reads_the_statistics():
    L, cfgs = configs()
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    c = O.constants(alpha=0.5)
    f = np.random.default_rng(5).standard_normal((1, len(cfgs[0]), 3))
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_deferred_checks(True)
        for xyz in cfgs:
            ctx.set_particles(xyz)
            ctx.build_cells()
            got = ctx.local_matvec(f, G.SELF_BEAD)
            nb = O.neighbors_cutoff(box, xyz, 7.0)
            assert ctx.pair_count() == nb.offsets[-1]
            want = O.local_matvec(c, box, xyz, nb, f, O.SELF_BEAD, nthreads=8)
            assert rel(got, want) <= 1e-6


def test_deferred_out_of_domain_reported_by_the_chebyshev_call():
    xyz, L = G.make_suspension(7, 800, 0.05)
    xi = np.random.default_rng(7).standard_normal(3 * len(xyz))
    with G.Context(box_hi=(L,) * 3, periodic=(1, 1, 0), rc=7.0, precision=G.FP32) as ctx:
        ctx.set_deferred_checks(True)
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=30, seed=3)
        rc, _, _ = run(ctx, xyz, xi, (lo / 1.05, hi * 1.05))
        assert rc == 0
        bad = xyz.copy()
        bad[17, 2] = L + 3.0  # outside the non-periodic axis
        ctx.set_particles(bad)
        ctx.build_cells()  # deferred: returns without the verdict
        rc, _, _ = ctx.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05, 1e-3, check_every=0)
        assert rc == G.ERR_OUT_OF_DOMAIN


def test_host_buffer_step_matches_device_step_exactly():
    """ggem_brownian_displacement copies xi on its own stream while the
    deferred cell and list build runs; the series waits for the copy.  With
    a different xi every call, the host-buffer step equals the
    device-pointer step bit for bit (a series that read the previous call's
    xi would not)."""
    import torch
    xyz, L = G.make_suspension(93, 20000, 0.1)
    n = len(xyz)
    xis = [np.random.default_rng(50 + k).standard_normal(3 * n) for k in range(4)]
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_pair_tensors(False)
        ctx.set_particles(xyz)
        ctx.build_cells()
        lo, hi = ctx.lanczos_bounds(k=24, seed=3)
        lo, hi = lo / 1.05, hi * 1.05
        ctx.set_deferred_checks(True)
        host = []
        for xi in xis:
            ctx.set_particles(xyz)
            ctx.build_cells()  # queued, not waited for
            rc, dw, rep = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=0)
            assert rc == 0, rep
            host.append(dw.copy())
        d_xyz = torch.from_numpy(xyz.reshape(-1).copy()).cuda()
        for xi, want in zip(xis, host):
            ctx.set_particles_dev(d_xyz.data_ptr(), n)
            ctx.build_cells()
            d_xi = torch.from_numpy(xi).cuda()
            d_dw = torch.empty_like(d_xi)
            rc, rep = ctx.brownian_displacement_dev(d_xi.data_ptr(), d_dw.data_ptr(), 1, 50, lo,
                                                    hi, 1e-3, 0)
            assert rc == 0, rep
            assert np.array_equal(d_dw.cpu().numpy(), want)
