"""The global (FEM) velocity at the particles (include/ggem_fem.h) against
the oracle's HEX20 interpolation, and exact on quadratic fields."""
import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O
from fem_mesh import HEX20, hex20_mesh, quadratic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()
    O.build_oracle(with_ref=False)


def test_hex20_shape_device_build_matches_oracle():
    rng = np.random.default_rng(1)
    for xi in np.concatenate([HEX20.astype(float), rng.uniform(-1, 1, (40, 3))]):
        assert np.abs(G.hex20_shape(xi) - O.hex20_shape(xi)).max() <= 1e-15


@pytest.mark.parametrize("periodic", [(1, 1, 1), (1, 1, 0), (0, 0, 0)])
def test_fem_point_values_match_oracle(periodic):
    ne, L = (9, 7, 8), np.array([36.0, 28.0, 32.0])
    dofs, nd, _, _ = hex20_mesh(ne, (0, 0, 0), L, seed=3)
    rng = np.random.default_rng(4)
    sol = rng.standard_normal(nd)
    xyz = rng.uniform(0, 1, (5000, 3)) * L
    if periodic[0]:
        xyz[:50, 0] += L[0] * rng.choice([-2, -1, 1], 50)  # images outside the box
    xyz[50:60] = np.floor(xyz[50:60] / (L / ne)) * (L / ne)  # on element faces
    with G.Context(box_hi=tuple(L), periodic=periodic, rc=7.0, precision=G.FP64) as ctx:
        ctx.set_particles(xyz)
        with G.Fem(ctx, ne, (0, 0, 0), L, nd, dofs) as fem:
            got = fem.point_values(sol)
            base = rng.standard_normal((len(xyz), 3))
            acc = fem.point_values(sol, u=base, accumulate=True)
    want, outside = O.fem_point_values(xyz, ne, (0, 0, 0), L, periodic, dofs, sol)
    assert outside == 0
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    assert np.abs(acc - (base + want)).max() <= 1e-12 * np.abs(base + want).max()


def test_fem_point_values_exact_on_quadratics_and_out_of_domain():
    ne, lo, hi = (5, 6, 4), (-3.0, 1.0, 0.0), (7.0, 13.0, 8.0)
    dofs, nd, dpos, dvar = hex20_mesh(ne, lo, hi, seed=5)
    sol = np.array([quadratic(dpos[k], dvar[k]) for k in range(nd)])
    pts = np.random.default_rng(6).uniform(lo, hi, (2000, 3))
    with G.Context(box_lo=lo, box_hi=hi, periodic=(0, 0, 0), rc=2.0, precision=G.FP64) as ctx:
        ctx.set_particles(pts)
        with G.Fem(ctx, ne, lo, hi, nd, dofs) as fem:
            got = fem.point_values(sol)
            want = np.stack([quadratic(pts, v) for v in range(3)], axis=1)
            assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
            bad = pts.copy()
            bad[7, 2] = hi[2] + 1.0
            ctx.set_particles(bad)
            with pytest.raises(G.GGEMError) as ei:
                fem.point_values(sol)
            assert ei.value.code == G.ERR_OUT_OF_DOMAIN
