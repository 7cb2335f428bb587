"""Regenerate the committed golden fixtures in tests/golden/.

Run on a machine that has the reference tree: GGEM_REFERENCE_ROOT, else a
checkout named "reference" beside this repository.  Two fixtures come out:

* ggem_profile_3P.json -- the reference's PointParticle_Stokes_GGEM golden
  velocity profiles (tests/integration_tests/resources/PointParticle_Stokes_GGEM/
  output/output_velocity_profile_{x,y,z}_3P.txt), reduced to the columns that
  pin the particle-side kernels: the coordinate, the three GGEM local-velocity
  columns (pair kernel in field-target mode, ggem_stokes.C:360-424) and the
  three unbounded xi-smoothed columns (ggem_stokes.C:201-251,
  analytical_solution_stokes.C:66-102).  Columns are taken by position
  (0, 7-9, 10-12); the files predate the csv writer at
  pm_system_stokes.C:669-674.
* polymer_bd_hi_data.in, polymer_bd_hi_output_0.vtk -- the reference's
  PointParticle_Polymer_BD_HI particle data file and the VTK of its initial
  configuration written by the reference (pins the particle-file formats).
* ref_chebyshev_coeffs.json -- Chebyshev coefficients produced by the
  reference's own src/chebyshev.C (compiled into oracle/_ref by
  oracle/Makefile) for a grid of orders, intervals and quadrature methods,
  stored as hex floats so the comparison is bit-exact.
* ref_ggem_local.json -- outputs of the reference's own src/ggem_stokes.C
  (GGEMStokes, compiled into oracle/_ref with the stand-in PointMesh of
  oracle/ref_shim_ggem): green_tensor_local_regularized for each point type
  and a set of vectors down to r = 0, and local_solution_bead /
  global_self_exclusion / local_solution_field of small seeded suspensions
  (periodic and open boxes, bead and Lagrangian points), inputs and outputs
  as hex floats.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_ROOT = Path(os.environ.get("GGEM_REFERENCE_ROOT", str(ROOT.parent / "reference")))
PROFILE_DIR = (REF_ROOT / "tests" / "integration_tests" / "resources"
               / "PointParticle_Stokes_GGEM")

# Chebyshev cases: (N, eig_min, eig_max) spanning the reference defaults
# (max_n_cheb 10..50, copss.C:794-797) and the BD_HI eigen interval golden
# (out.eigenvalue 0.64154 1.32335).
CHEB_CASES = [(10, 0.64154, 1.32335), (30, 0.2, 1.4), (50, 0.05, 2.0),
              (16, 1.0, 4096.0), (5, 0.9, 1.1), (40, 0.3, 1.05)]


def profiles() -> dict:
    out = {"source": "tests/integration_tests/resources/PointParticle_Stokes_GGEM",
           "alpha": 0.35, "box": [-15.0, 15.0], "n_mesh": [15, 15, 15],
           "periodic": [False, False, False],
           "beads": [[-5.0, 0.0, 0.0], [0.0, 0.0, 0.0], [5.0, 0.0, 0.0]],
           "force": [0.3333, 0.0, 0.0], "print_decimals": 9,
           "reference_tolerance": 1e-5, "axes": {}}
    for name in "xyz":
        g = np.loadtxt(PROFILE_DIR / "output" / f"output_velocity_profile_{name}_3P.txt")
        out["axes"][name] = {"coord": g[:, 0].tolist(), "local": g[:, 7:10].tolist(),
                             "exact": g[:, 10:13].tolist()}
    return out


def cheb_coeffs() -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O  # noqa: E402  (test infrastructure)

    O.build_oracle(with_ref=True)
    cases = []
    for N, lmin, lmax in CHEB_CASES:
        d = lmax - lmin
        da, db = 2.0 / d, -(lmax + lmin) / d
        for method in (0, 1, 2):
            c = O.ref_cheb_coeffs(N, da, db, method)
            if c is None:
                raise SystemExit("oracle/_ref/libref_chebyshev.so was not built")
            cases.append({"N": N, "da": da.hex(), "db": db.hex(), "method": method,
                          "coef": [float(x).hex() for x in c]})
    return {"source": "src/chebyshev.C via oracle/_ref", "cases": cases}


def _hex(a) -> list:
    return [float(x).hex() for x in np.asarray(a, float).ravel()]


def ggem_local() -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O  # noqa: E402  (test infrastructure)

    O.build_oracle(with_ref=True)
    if O.ref_ggem_lib() is None:
        raise SystemExit("oracle/_ref/libref_ggem.so was not built")
    rng = np.random.default_rng(2024)
    types = [("bead", O.POLYMER_BEAD, {}),
             ("lagrangian", O.LAGRANGIAN_POINT, {"ibm_beta": 0.75, "hmin": 2.0}),
             ("point_particle", O.POINT_PARTICLE, {})]
    vecs = np.vstack([np.zeros(3), [1e-7, 0, 0], [3e-7, 4e-7, 0], [2e-6, 0, 0],
                      rng.standard_normal((40, 3)) * 3.0])
    green = []
    for name, pt, kw in types:
        c = O.constants(alpha=0.5, point_type=pt, **kw)
        G = np.stack([O.ref_green_local(c, x, pt, **kw) for x in vecs])
        green.append({"type": name, "point_type": pt, "alpha": 0.5, **kw, "G": _hex(G)})
    beads = []
    # periodic edges of at least 3 rc, which the CUDA cut-off cell grid needs
    for name, pt, kw, L, per, n, rc in (
            ("periodic_bead", O.POLYMER_BEAD, {}, 15.0, (1, 1, 1), 120, 4.5),
            ("open_z_bead", O.POLYMER_BEAD, {}, 16.5, (1, 1, 0), 110, 5.5),
            ("periodic_lagrangian", O.LAGRANGIAN_POINT, {"ibm_beta": 0.75, "hmin": 2.0},
             12.0, (1, 1, 1), 80, 4.0)):
        c = O.constants(alpha=0.5, point_type=pt, **kw)
        box = O.make_box((0, 0, 0), (L, L, L), per)
        xyz = rng.uniform(0, L, (n, 3))
        f = rng.standard_normal((n, 3))
        nb = O.neighbors_cutoff(box, xyz, rc)
        ul, us = O.ref_local_bead(c, box, xyz, f, nb, pt, **kw)
        beads.append({"case": name, "point_type": pt, "alpha": 0.5, **kw, "L": L,
                      "periodic": list(per), "rc": rc, "xyz": _hex(xyz), "f": _hex(f),
                      "offsets": [int(v) for v in nb.offsets],
                      "ids": [int(v) for v in nb.ids],
                      "u_local": _hex(ul), "u_self": _hex(us)})
    # local_solution_field at points inside elements of a 6 x 6 x 6 mesh
    L, n, nm = 12.0, 80, 6
    c = O.constants(alpha=0.5)
    box = O.make_box((0, 0, 0), (L, L, L), (1, 1, 1))
    mesh = O.make_mesh(nm, nm, nm, 0.5 * L / nm + 4.0)
    xyz = rng.uniform(0, L, (n, 3))
    f = rng.standard_normal((n, 3))
    enb, _ = O.elem_lists(box, mesh, xyz)
    targets = rng.uniform(0, L, (50, 3))
    te = np.array([O.lib().orc_elem_of_point(O.C.byref(box), O.C.byref(mesh),
                                             O._p(np.ascontiguousarray(t)))
                   for t in targets], np.int32)
    u = O.ref_local_field(c, box, enb, xyz, f, targets, te)
    field = {"case": "periodic_field", "alpha": 0.5, "L": L, "periodic": [1, 1, 1],
             "n_mesh": nm, "search_radius_e": 0.5 * L / nm + 4.0, "xyz": _hex(xyz),
             "f": _hex(f), "targets": _hex(targets), "target_elem": te.tolist(),
             "u": _hex(u)}
    return {"source": "src/ggem_stokes.C via oracle/_ref", "vectors": _hex(vecs),
            "green": green, "beads": beads, "field": field}


POLYMER_DIR = (REF_ROOT / "tests" / "integration_tests" / "resources"
               / "PointParticle_Polymer_BD_HI")


def polymer_files() -> None:
    """The reference's PointParticle_Polymer_BD_HI input data file and the
    VTK its writer produced for that initial configuration, copied verbatim:
    a reader / writer round trip through the library must reproduce the VTK
    byte for byte (polymer_chain.C:61-226, :1096-1154)."""
    (HERE / "polymer_bd_hi_data.in").write_bytes(
        (POLYMER_DIR / "point_particle_data.in").read_bytes())
    (HERE / "polymer_bd_hi_output_0.vtk").write_bytes(
        (POLYMER_DIR / "output" / "output_polymer_0.vtk").read_bytes())


def main() -> None:
    (HERE / "ggem_profile_3P.json").write_text(json.dumps(profiles()))
    (HERE / "ref_chebyshev_coeffs.json").write_text(json.dumps(cheb_coeffs(), indent=1))
    (HERE / "ref_ggem_local.json").write_text(json.dumps(ggem_local()))
    polymer_files()
    print("wrote", HERE / "ggem_profile_3P.json", HERE / "ref_chebyshev_coeffs.json",
          HERE / "ref_ggem_local.json",
          HERE / "polymer_bd_hi_data.in", HERE / "polymer_bd_hi_output_0.vtk")


if __name__ == "__main__":
    main()
