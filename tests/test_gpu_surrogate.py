"""The eigen-interval network on the GPU (tcgen05 products) against the CPU
oracle, its training, and what it gains over the Lanczos bound."""
import time

import numpy as np
import pytest

import ggem_gb300 as G
import mlp_oracle as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()


def rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


def _random_net(seed, n):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, M.IN)).astype(np.float32) * 2 + 1
    Y = rng.standard_normal((n, M.OUT)).astype(np.float32)
    sur = G.Surrogate(seed=seed)
    sur.fit_norm(X, Y)
    P = sur.params
    # nonzero biases so that every term of the backward pass is exercised
    off = 0
    for d in M.IN_DIMS:
        off += 128 * d
        P[off:off + 128] = rng.standard_normal(128).astype(np.float32) * 0.1
        off += 128
    P[off - 128 + 2:off] = 0.0          # output bias padding stays zero
    sur.params = P
    return sur, X, Y


@pytest.mark.parametrize("n", [100, 256, 700])
def test_forward_matches_oracle(n):
    sur, X, _ = _random_net(1, n)
    got = sur.predict(X)
    want = M.predict(sur.params, sur.norm, X)
    assert rel(got, want) <= 2e-3
    sur.close()


@pytest.mark.parametrize("n", [200, 256, 1000])
def test_gradient_matches_oracle(n):
    """Loss and every layer's weight and bias gradient of one forward +
    backward pass (tcgen05 products: X W^T, dZ^T H, dZ W) against the
    oracle's BF16/FP32 restatement."""
    sur, X, Y = _random_net(2, n)
    loss, g = sur.gradient(X, Y)
    loss_o, g_o = M.loss_and_grad(sur.params, sur.norm, X, Y)
    assert loss == pytest.approx(loss_o, rel=1e-4)
    off = 0
    for l, d in enumerate(M.IN_DIMS):
        w = slice(off, off + 128 * d)
        b = slice(off + 128 * d, off + 128 * d + 128)
        off += 128 * d + 128
        assert rel(g[w], g_o[w]) <= 5e-3, f"layer {l} weights"
        assert rel(g[b], g_o[b]) <= 5e-3, f"layer {l} biases"
    sur.close()


def test_training_fits_a_smooth_map():
    rng = np.random.default_rng(3)
    n = 4096
    X = rng.uniform(-1, 1, (n, M.IN)).astype(np.float32)
    Y = np.stack([X[:, :5].sum(1) + 0.5 * np.sin(2 * X[:, 5] * X[:, 6]),
                  np.tanh(X[:, 7:12].sum(1)) - 0.3 * X[:, 12] ** 2], 1).astype(np.float32)
    sur = G.Surrogate(seed=5)
    sur.fit_norm(X[:3584], Y[:3584])
    loss = sur.train(X[:3584], Y[:3584], epochs=60, batch=256, lr=2e-3, seed=1)
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.05 * loss[0]
    P = sur.predict(X[3584:])
    assert rel(P, Y[3584:]) < 0.15
    sur.close()


def test_surrogate_interval_gain_over_lanczos():
    """A small training set of real configurations (features on the GPU,
    Lanczos labels), then held-out Brownian displacements: the network's
    interval (widened by the held-out error) replaces the Lanczos bound; the
    FP64 Chebyshev check judges it and Lanczos is the fallback.  The network
    must save operator applications and time."""
    from ggem_gb300 import surrogate_data as SD
    cfgs = SD.sample_configs(224, seed=11, n_range=(1000, 4000))
    X, Y = SD.label(cfgs, k=40)
    assert np.all(np.isfinite(Y)) and np.all(Y[:, 0] < Y[:, 1])
    tr, ho = slice(0, 192), slice(192, 224)
    sur, summary, loss = SD.train(X[tr], Y[tr], X[ho], Y[ho], epochs=200, batch=128, lr=2e-3)
    assert loss[-1] < 0.2 * loss[0]
    assert max(summary["holdout_rmse_log"]) < 0.25
    margins = np.maximum(np.asarray(summary["margins_log"]), 0.05)
    n_sur = n_lz = fallbacks = 0
    t_sur = t_lz = 0.0
    for i in range(192, 224):
        xyz, L = SD.positions(cfgs[i])
        xi = np.random.default_rng(i).standard_normal(3 * len(xyz))
        with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
            ctx.set_particles(xyz)
            ctx.build_cells()
            # without the network: Lanczos(24) bound, widened as copss.C:1607
            t0 = time.perf_counter()
            lo, hi = ctx.lanczos_bounds(k=24, seed=7)
            rc, dw, rep = ctx.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05, 1e-3,
                                                    check_every=1)
            t_lz += time.perf_counter() - t0
            assert rc == 0
            n_lz += 24 + rep[0]["n_matvecs"]
            # with the network, Lanczos only when the error check fails
            t0 = time.perf_counter()
            lo, hi = ctx.surrogate_interval(sur, cfgs[i]["chain_fraction"], margins[0],
                                            margins[1])
            rc, dw2, rep = ctx.brownian_displacement(xi, 50, lo, hi, 1e-3, check_every=1)
            n_sur += rep[0]["n_matvecs"]
            if rc != 0:
                fallbacks += 1
                lo, hi = ctx.lanczos_bounds(k=24, seed=7)
                rc, dw2, rep = ctx.brownian_displacement(xi, 50, lo / 1.05, hi * 1.05, 1e-3,
                                                         check_every=1)
                n_sur += 24 + rep[0]["n_matvecs"]
            t_sur += time.perf_counter() - t0
            assert rc == 0 and rep[0]["err1"] <= 1e-3
    print(f"surrogate: {n_sur} matvecs {t_sur:.3f} s, {fallbacks} fallbacks; "
          f"lanczos: {n_lz} matvecs {t_lz:.3f} s")
    assert fallbacks <= 4
    assert n_sur < 0.7 * n_lz
    assert t_sur < t_lz
    sur.close()


def test_features_on_a_known_lattice():
    """g(r) of a simple cubic lattice of spacing 2.5: only the shells at
    2.5, 3.54, 4.33, 5.0, ... are populated, and phi / log N are exact."""
    a = 2.5
    m = 12
    g1 = np.arange(m) * a + 0.3
    xyz = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)
    L = m * a
    with G.Context(box_hi=(L,) * 3, rc=7.0, precision=G.FP32) as ctx:
        ctx.set_particles(xyz)
        ctx.build_cells()
        f = ctx.surrogate_features(0.25)
    n = len(xyz)
    assert f[0] == pytest.approx(n * 4 / 3 * np.pi / L ** 3, rel=1e-6)
    assert f[1] == pytest.approx(np.log(n), rel=1e-6)
    assert f[-1] == pytest.approx(0.25)
    hist = f[2:-1]
    dr = 5.0 / 32
    edges = 2.0 + dr * np.arange(33)
    shells = np.sqrt(np.array([1, 2, 3, 4, 5, 6, 8, 9], float)) * a
    for b in range(32):
        has = np.any((shells >= edges[b]) & (shells < edges[b + 1]))
        assert (hist[b] > 0) == has, b


@pytest.mark.parametrize("n", [1, 100, 700])
def test_fused_forward_equals_layer_path(n):
    """the one-kernel forward pass (weights resident in shared memory) gives
    the layer-by-layer path's outputs: same products in the same K order,
    same bias, SiLU and BF16 rounding"""
    sur, X, _ = _random_net(4, n)
    a = sur.predict(X)
    b = sur.predict_layers(X)
    assert np.array_equal(a, b), np.abs(a - b).max()
    ms = sur.time_forward(1, 100)
    print(f"one interval prediction (1 row): {ms * 1e3:.1f} us per forward launch")
    sur.close()


def test_tensor_core_wait_timeout_is_reported_and_recovers():
    """A poll budget of zero makes the first mbarrier wait of a product give
    up at once: the kernel drains the product still in flight with its full
    window, frees TMEM and reports GGEM_ERR_TIMEOUT; the network stays
    usable and the next products are exact.  (No wait is left unbounded and
    nothing faults: the products complete within microseconds.)"""
    sur, X, Y = _random_net(5, 300)
    want = M.predict(sur.params, sur.norm, X)
    for fn in (sur.predict, sur.predict_layers):
        sur.set_poll_budget(0)
        with pytest.raises(G.GGEMError) as e:
            fn(X)
        assert e.value.code == G.ERR_TIMEOUT
        sur.set_poll_budget(1 << 22)
        assert rel(fn(X), want) <= 2e-3
    loss, g = sur.gradient(X, Y)
    loss_o, _ = M.loss_and_grad(sur.params, sur.norm, X, Y)
    assert loss == pytest.approx(loss_o, rel=1e-4)
    sur.close()
