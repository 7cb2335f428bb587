"""Uneven ensembles of suspensions through one block-diagonal operator,
against the FP64 oracle of every suspension."""
import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu
FP32_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _ensemble(K, seed, n_range=(500, 3000)):
    rng = np.random.default_rng(seed)
    sus = []
    for b in range(K):
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        phi = float(rng.uniform(0.02, 0.2))
        xyz, L = G.make_suspension(seed * 1000 + b, n, phi)
        sus.append((xyz, L))
    return sus


def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def test_ensemble_matvec_matches_every_suspension():
    import torch
    sus = _ensemble(6, 3)
    R = 8
    f = [np.random.default_rng(b).standard_normal((len(x), R, 3)) for b, (x, _) in enumerate(sus)]
    with G.Ensemble([L for _, L in sus]) as ens:
        d_xyz = _device(np.concatenate([x for x, _ in sus]))
        ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
        beads, pairs = ens.sizes()
        assert beads == sum(len(x) for x, _ in sus)
        d_f = _device(np.concatenate(f))
        d_u = torch.empty_like(d_f)
        ens.matvec_dev(R, d_f.data_ptr(), d_u.data_ptr(), G.SELF_BEAD)
        u = d_u.cpu().numpy()
    c = O.constants(alpha=0.5)
    off = 0
    n_pairs = 0
    for b, (xyz, L) in enumerate(sus):
        n = len(xyz)
        box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
        nb = O.neighbors_cutoff(box, xyz, 7.0)
        n_pairs += nb.offsets[-1]
        fb = np.transpose(f[b], (1, 0, 2))          # [r][n][3]
        want = O.local_matvec(c, box, xyz, nb, fb, O.SELF_BEAD, nthreads=8)
        got = np.transpose(u[off:off + n], (1, 0, 2))
        assert rel(got, want) <= FP32_TOL, b
        off += n
    assert pairs == n_pairs


def test_ensemble_brownian_matches_oracle_series():
    import torch
    sus = _ensemble(5, 7)
    R = 8
    xi = [np.random.default_rng(100 + b).standard_normal((len(x), R, 3))
          for b, (x, _) in enumerate(sus)]
    with G.Ensemble([L for _, L in sus]) as ens:
        d_xyz = _device(np.concatenate([x for x, _ in sus]))
        ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
        block, ms = ens.autotune(R)
        assert block in (128, 256, 512) and ms > 0
        bounds = [ens.lanczos(b, k=40, seed=1) for b in range(len(sus))]
        lo = np.array([x[0] for x in bounds]) / 1.05
        hi = np.array([x[1] for x in bounds]) * 1.05
        d_xi = _device(np.concatenate(xi))
        d_dw = torch.empty_like(d_xi)
        results = []
        for _ in range(3):  # the second and third calls replay the captured terms
            rc, reps = ens.brownian_dev(R, 50, lo, hi, 1e-3, d_xi.data_ptr(), d_dw.data_ptr())
            assert rc == 0
            results.append((d_dw.cpu().numpy(), reps))
    c = O.constants(alpha=0.5)
    for dw, reps in results:
        off = 0
        for b, (xyz, L) in enumerate(sus):
            n = len(xyz)
            box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
            nb = O.neighbors_cutoff(box, xyz, 7.0)
            op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, 8))
            for r in (0, 5):
                assert reps[b][r]["converged"] and reps[b][r]["err1"] <= 1e-3
                y_o, rep_o = O.cheb_inv_sqrt(op, xi[b][:, r, :].reshape(-1), 50, lo[b], hi[b],
                                             1e-3)
                dw_o = O.local_matvec(c, box, xyz, nb, y_o.reshape(1, n, 3), O.SELF_BEAD,
                                      nthreads=8)
                assert rel(dw[off:off + n, r, :], dw_o[0]) <= 5e-3, (b, r)
            off += n


def test_ensemble_intervals_from_the_network():
    """All intervals from one batched forward pass; series the check rejects
    fall back to Lanczos."""
    import torch
    from ggem_gb300 import surrogate_data as SD
    loaded = SD.load_default()
    if loaded is None:
        pytest.skip("no trained network shipped")
    sur, margins, _ = loaded
    sus = _ensemble(8, 13, n_range=(1000, 5000))
    R = 8
    with G.Ensemble([L for _, L in sus]) as ens:
        d_xyz = _device(np.concatenate([x for x, _ in sus]))
        ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
        lo, hi = ens.intervals(sur, None, margins[0], margins[1])
        assert np.all(lo > 0) and np.all(hi > lo)
        xi = np.random.default_rng(5).standard_normal((sum(len(x) for x, _ in sus), R, 3))
        d_xi = _device(xi)
        d_dw = torch.empty_like(d_xi)
        rc, reps = ens.brownian_dev(R, 50, lo, hi, 1e-3, d_xi.data_ptr(), d_dw.data_ptr())
        failed = [b for b in range(len(sus)) if not all(r["converged"] for r in reps[b])]
        for b in failed:
            lo[b], hi[b] = (v * f for v, f in zip(ens.lanczos(b, 24, 7), (1 / 1.05, 1.05)))
        if failed:
            rc, reps = ens.brownian_dev(R, 50, lo, hi, 1e-3, d_xi.data_ptr(), d_dw.data_ptr())
        assert rc == 0
        assert len(failed) <= 2
        assert all(r["converged"] for rb in reps for r in rb)
    sur.close()


def _in_box(seed, L, phi):
    """a non-overlapping suspension at volume fraction ~phi inside [0, L)^3
    (generated in the largest box L2 <= L that make_suspension gives for an
    integer bead count: its minimum-image separations only grow in L)"""
    n = int(np.floor(phi * L ** 3 * 3.0 / (4.0 * np.pi)))
    xyz, L2 = G.make_suspension(seed, n, phi)
    assert L2 <= L + 1e-12
    return xyz


def test_ensemble_reconfiguration_drops_captured_terms():
    """A Brownian step captures its unchecked terms as a graph that holds the
    bead count, the row width and the operator's buffers.  After
    set_particles on denser suspensions (more beads, wider rows, reallocated
    lists) the next step must not replay the old graph: it gives exactly
    what a fresh ensemble gives on the same configuration."""
    import torch
    boxes = [30.0, 34.0, 38.0]
    R, N, tol = 8, 4, 1e-14  # 4 terms, nothing converges: the same schedule every call
    sparse = [_in_box(10 + b, L, 0.03) for b, L in enumerate(boxes)]
    dense = [_in_box(20 + b, L, 0.2) for b, L in enumerate(boxes)]
    rng = np.random.default_rng(3)
    xi_s = _device(rng.standard_normal((sum(len(x) for x in sparse), R, 3)))
    xi_d = _device(rng.standard_normal((sum(len(x) for x in dense), R, 3)))
    lo, hi = np.full(3, 0.05), np.full(3, 2.5)
    with G.Ensemble(boxes) as fresh:
        fresh.set_particles_dev([len(x) for x in dense], _device(np.concatenate(dense)).data_ptr())
        d_want = torch.empty_like(xi_d)
        rc, rep_want = fresh.brownian_dev(R, N, lo, hi, tol, xi_d.data_ptr(), d_want.data_ptr())
        assert rc == G.ERR_CHEB_NOT_CONVERGED
        want = d_want.cpu().numpy()
        w_dense = fresh.sizes()
    with G.Ensemble(boxes) as ens:
        d_s = _device(np.concatenate(sparse))
        ens.set_particles_dev([len(x) for x in sparse], d_s.data_ptr())
        d_dw = torch.empty_like(xi_s)
        for _ in range(2):  # captures the graph, then replays it
            ens.brownian_dev(R, N, lo, hi, tol, xi_s.data_ptr(), d_dw.data_ptr())
        d_d = _device(np.concatenate(dense))
        ens.set_particles_dev([len(x) for x in dense], d_d.data_ptr())
        assert ens.sizes() == w_dense
        d_dw = torch.empty_like(xi_d)
        for _ in range(2):
            rc, reps = ens.brownian_dev(R, N, lo, hi, tol, xi_d.data_ptr(), d_dw.data_ptr())
            assert rc == G.ERR_CHEB_NOT_CONVERGED
            got = d_dw.cpu().numpy()
            assert np.array_equal(got, want)
            assert [[r["n_terms"] for r in rb] for rb in reps] == \
                [[r["n_terms"] for r in rb] for rb in rep_want]


def test_persistent_series_equals_launch_per_term():
    """The whole step in one persistent launch (device-side checks and
    stopping decisions) gives the launch-per-term path's displacements and
    reports, for every tile size, on a first call and on a second call that
    starts its checks at the learned degree (fresh ensembles, so both paths
    run the same check schedule)."""
    import torch
    sus = _ensemble(7, 21)
    R = 8
    xi = np.random.default_rng(9).standard_normal((sum(len(x) for x, _ in sus), R, 3))
    d_xyz = _device(np.concatenate([x for x, _ in sus]))
    d_xi = _device(xi)

    def run(persistent, S=0):
        out = []
        with G.Ensemble([L for _, L in sus]) as ens:
            ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
            ens.set_series_mode(persistent=persistent, slots_per_tile=S)
            bounds = [ens.lanczos(b, k=40, seed=1) for b in range(len(sus))]
            lo = np.array([x[0] for x in bounds]) / 1.05
            hi = np.array([x[1] for x in bounds]) * 1.05
            for _ in range(2):
                d_dw = torch.zeros_like(d_xi)
                rc, rep = ens.brownian_dev(R, 50, lo, hi, 1e-3, d_xi.data_ptr(), d_dw.data_ptr())
                assert rc == 0
                out.append((d_dw.cpu().numpy(), rep))
        return out

    want = run(False)
    for S in (16, 64, 256):
        got = run(True, S)
        for call, ((g, rep), (w, wrep)) in enumerate(zip(got, want)):
            assert rel(g, w) <= 1e-12, (S, call)
            for b in range(len(sus)):
                for r in range(R):
                    a, x = rep[b][r], wrep[b][r]
                    assert a["converged"] == x["converged"] and a["n_terms"] == x["n_terms"]
                    assert a["n_matvecs"] == x["n_matvecs"]
                    # err1^2 is a difference of two nearly equal FP64 sums
                    # (summed per tile here, per chunk there): ~1e-15 absolute
                    assert abs(a["err1"] - x["err1"]) <= max(1e-9 * x["err1"],
                                                             1e-13 / x["err1"])


def test_persistent_series_wait_timeout_is_reported():
    """A wait of the persistent launch that runs out (test hook: no pass is
    ever marked complete) sets the error word; every block leaves, the call
    returns GGEM_ERR_TIMEOUT and the ensemble stays usable: the next call
    gives the launch-per-term path's displacements."""
    import torch
    sus = _ensemble(3, 33)
    R = 8
    d_xyz = _device(np.concatenate([x for x, _ in sus]))
    xi = _device(np.random.default_rng(2).standard_normal((sum(len(x) for x, _ in sus), R, 3)))
    out = []
    for persistent in (True, False):
        with G.Ensemble([L for _, L in sus]) as ens:
            ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
            bounds = [ens.lanczos(b, k=40, seed=1) for b in range(len(sus))]
            lo = np.array([x[0] for x in bounds]) / 1.05
            hi = np.array([x[1] for x in bounds]) * 1.05
            dw = torch.empty_like(xi)
            if persistent:
                ens.set_series_mode(persistent=True, wait_polls=2000, never_ready=True)
                with pytest.raises(G.GGEMError) as e:
                    ens.brownian_dev(R, 50, lo, hi, 1e-3, xi.data_ptr(), dw.data_ptr())
                assert e.value.code == G.ERR_TIMEOUT
                ens.set_series_mode(persistent=True)
            else:
                ens.set_series_mode(persistent=False)
            rc, reps = ens.brownian_dev(R, 50, lo, hi, 1e-3, xi.data_ptr(), dw.data_ptr())
            assert rc == 0 and all(r["converged"] for rb in reps for r in rb)
            out.append(dw.cpu().numpy())
    assert rel(out[0], out[1]) <= 1e-12


def test_series_autotuner_and_its_cache(tmp_path):
    """The autotuner times every launch shape and tile size of the persistent
    launch, keeps the fastest and appends it to the cache file; a second
    ensemble of the same sizes reads the choice back without timing; the
    tuned launch gives the launch-per-term path's displacements."""
    import torch
    sus = _ensemble(4, 44)
    R = 8
    d_xyz = _device(np.concatenate([x for x, _ in sus]))
    xi = _device(np.random.default_rng(4).standard_normal((sum(len(x) for x, _ in sus), R, 3)))
    cache = tmp_path / "series_tune.txt"
    out = []
    for run in range(2):
        with G.Ensemble([L for _, L in sus]) as ens:
            ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
            bounds = [ens.lanczos(b, k=40, seed=1) for b in range(len(sus))]
            lo = np.array([x[0] for x in bounds]) / 1.05
            hi = np.array([x[1] for x in bounds]) * 1.05
            dw = torch.empty_like(xi)
            t0 = __import__("time").perf_counter()
            sh, S, ms = ens.autotune_series(R, 14, lo, hi, xi.data_ptr(), dw.data_ptr(),
                                            str(cache))
            dt = __import__("time").perf_counter() - t0
            assert 0 <= sh <= 3 and S in (64, 128, 256) and ms > 0  # 3: a launch per term
            lines = cache.read_text().splitlines()
            assert len(lines) == 1  # the second run reads the line, it does not add one
            out.append((sh, S, ms, dt))
            rc, _ = ens.brownian_dev(R, 50, lo, hi, 1e-3, xi.data_ptr(), dw.data_ptr())
            assert rc == 0
            got = dw.cpu().numpy()
    assert out[0][:2] == out[1][:2] and out[1][2] == pytest.approx(out[0][2], rel=1e-5)
    with G.Ensemble([L for _, L in sus]) as ens:
        ens.set_particles_dev([len(x) for x, _ in sus], d_xyz.data_ptr())
        ens.set_series_mode(persistent=False)
        dw = torch.empty_like(xi)
        rc, _ = ens.brownian_dev(R, 50, lo, hi, 1e-3, xi.data_ptr(), dw.data_ptr())
        assert rc == 0
        assert rel(got, dw.cpu().numpy()) <= 1e-12
    print(f"series autotune: shape {out[0][0]}, {out[0][1]} slots per tile, "
          f"{out[0][2]:.3f} ms per 14-term step; tuning {out[0][3]:.2f} s, cache hit {out[1][3]:.3f} s")
