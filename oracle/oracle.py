"""ctypes loader for the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module: it is the checker, never the product path.
``build_oracle()`` compiles ``oracle/ggem_oracle.c`` with the committed
Makefile; the reference's own ``chebyshev.C`` and ``ggem_stokes.C`` are
compiled into ``oracle/_ref`` when the reference tree is present on this
machine.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libggem_oracle.so"
REF_LIB_PATH = HERE / "_ref" / "libref_chebyshev.so"
REF_GGEM_PATH = HERE / "_ref" / "libref_ggem.so"
# the reference tree: GGEM_REFERENCE_SRC, else a checkout named "reference"
# beside this repository (absent on machines that only run the tests)
REF_SRC = Path(os.environ.get("GGEM_REFERENCE_SRC",
                              str(HERE.parent.parent / "reference" / "src")))

POLYMER_BEAD, LAGRANGIAN_POINT, POINT_PARTICLE = 0, 1, 2  # point_particle.h:36-41
SELF_NONE, SELF_BEAD, SELF_LAGRANGIAN = 0, 1, 2


class Consts(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "mu", "alpha", "ksi", "br0", "one_eight_pi_mu", "alpha2", "alpha3",
        "alpha3_pi_23", "two_alpha_sqrt_pi", "coeff_1", "ksi2", "ksi3",
        "ksi3_pi_23", "two_ksi_sqrt_pi", "coeff_2", "r_eps")]


class Box(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("periodic", C.c_int * 3)]


class NbList(C.Structure):
    _fields_ = [("n", C.c_int64), ("offsets", C.POINTER(C.c_int64)),
                ("ids", C.POINTER(C.c_int32))]


class Mesh(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("search_radius_e", C.c_double)]


class ChebReport(C.Structure):
    _fields_ = [("converged", C.c_int), ("n_terms", C.c_int),
                ("n_matvecs", C.c_int), ("err1", C.c_double),
                ("err2", C.c_double)]


class MatvecCtx(C.Structure):
    _fields_ = [("c", C.POINTER(Consts)), ("b", C.POINTER(Box)),
                ("n", C.c_int64), ("xyz", C.c_void_p),
                ("nb", C.POINTER(NbList)), ("self_mode", C.c_int),
                ("nthreads", C.c_int)]


OP_FN = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double))

_lib = None
_ref = None
_ref_ggem = None


def build_oracle(with_ref: bool = True) -> None:
    """Compile the oracle (and the reference chebyshev.C / ggem_stokes.C when
    the reference tree is available)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if with_ref and (REF_SRC / "chebyshev.C").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref",
                        f"REF_SRC={REF_SRC}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build_oracle(with_ref=False)
        L = C.CDLL(str(LIB_PATH))
        d, i64, vp = C.c_double, C.c_int64, C.c_void_p
        L.orc_set_constants.argtypes = [d, d, d, C.c_int, d, d, C.POINTER(Consts)]
        L.orc_green_local.argtypes = [C.POINTER(Consts), vp, vp]
        L.orc_green_unbounded_smoothed.argtypes = [C.POINTER(Consts), vp, d, vp]
        L.orc_smoothed_force_exp.argtypes = [C.POINTER(Consts), vp]
        L.orc_smoothed_force_exp.restype = d
        L.orc_point_vector.argtypes = [C.POINTER(Box), vp, vp, vp]
        L.orc_build_neighbors_cutoff.argtypes = [C.POINTER(Box), i64, vp, d, C.POINTER(NbList)]
        L.orc_elem_of_point.argtypes = [C.POINTER(Box), C.POINTER(Mesh), vp]
        L.orc_build_elem_lists.argtypes = [C.POINTER(Box), C.POINTER(Mesh), i64, vp,
                                           C.POINTER(NbList), vp]
        L.orc_build_neighbors_reference.argtypes = [C.POINTER(Box), C.POINTER(Mesh), i64,
                                                    vp, C.POINTER(NbList)]
        L.orc_free_nblist.argtypes = [C.POINTER(NbList)]
        L.orc_local_matvec.argtypes = [C.POINTER(Consts), C.POINTER(Box), i64, vp,
                                       C.POINTER(NbList), C.c_int, vp, vp, C.c_int, C.c_int]
        L.orc_local_field_reference.argtypes = [C.POINTER(Consts), C.POINTER(Box),
                                                C.POINTER(Mesh), C.POINTER(NbList), i64,
                                                vp, vp, i64, vp, vp]
        L.orc_local_field_cutoff.argtypes = [C.POINTER(Consts), C.POINTER(Box), i64, vp, vp,
                                             d, i64, vp, vp]
        L.orc_exact_unbounded.argtypes = [C.POINTER(Consts), i64, vp, vp, i64, vp, vp]
        L.orc_spread_qp.argtypes = [C.POINTER(Consts), C.POINTER(Box), C.POINTER(NbList),
                                    i64, vp, vp, i64, vp, vp, d, vp]
        L.orc_element_rhs.argtypes = [C.POINTER(Consts), C.POINTER(Box), C.POINTER(NbList),
                                      i64, vp, vp, i64, C.c_int, C.c_int, vp, vp, d, vp]
        L.orc_cheb_coeffs.argtypes = [C.c_int, d, d, C.c_int, vp]
        L.orc_cheb_inv_sqrt.argtypes = [OP_FN, vp, i64, C.c_int, d, d, d, vp,
                                        C.POINTER(ChebReport)]
        L.orc_lanczos.argtypes = [OP_FN, vp, i64, C.c_int, vp, vp, vp, vp, vp]
        L.orc_lanczos.restype = C.c_int
        L.orc_tridiag_extremes.argtypes = [C.c_int, vp, vp, vp, vp]
        L.orc_power_iteration.argtypes = [OP_FN, vp, i64, d, C.c_int, vp]
        L.orc_power_iteration.restype = C.c_int
        L.orc_std_normal_vector.argtypes = [C.c_uint64, i64, i64, d, d, vp]
        L.orc_philox_normals.argtypes = [C.c_uint64, C.c_uint64, i64, vp]
        L.orc_ev_gaussian.argtypes = [C.POINTER(Box), i64, vp, C.POINTER(NbList), d, d, vp]
        L.orc_spring_force.argtypes = [C.c_int, vp, d, d, vp]
        L.orc_spring_forces.argtypes = [C.POINTER(Box), i64, vp, i64, vp, C.c_int, d, d, vp]
        L.orc_hex20_shape.argtypes = [d, d, d, vp]
        L.orc_fem_point_values.restype = i64
        L.orc_fem_point_values.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own chebyshev.C (None when it was not built here)."""
    global _ref
    if _ref is None and REF_LIB_PATH.exists():
        R = C.CDLL(str(REF_LIB_PATH))
        R.ref_chebyshev_coefficients.argtypes = [C.c_int, C.c_double, C.c_double,
                                                 C.c_int, C.c_void_p]
        R.ref_chebyshev_coefficients.restype = C.c_int
        _ref = R
    return _ref


def ref_ggem_lib():
    """The reference's own GGEMStokes (ggem_stokes.C) behind the C entry
    points of oracle/ref_ggem_entry.cpp (None when it was not built here)."""
    global _ref_ggem
    if _ref_ggem is None and REF_GGEM_PATH.exists():
        R = C.CDLL(str(REF_GGEM_PATH))
        d, i64, vp = C.c_double, C.c_int64, C.c_void_p
        head = [d, d, d, C.c_int, d, d]
        R.ref_ggem_green_local.argtypes = head + [vp, vp]
        R.ref_ggem_local_bead.argtypes = head + [vp, vp, vp, i64, vp, vp, vp, vp, vp, vp]
        R.ref_ggem_local_field.argtypes = head + [vp, vp, vp, i64, vp, vp, i64, vp, vp, i64,
                                                  vp, vp, vp]
        for fn in (R.ref_ggem_green_local, R.ref_ggem_local_bead, R.ref_ggem_local_field):
            fn.restype = C.c_int
        _ref_ggem = R
    return _ref_ggem


def _ref_head(c: "Consts", point_type: int, ibm_beta: float, hmin: float):
    return (c.mu, c.alpha, c.br0, int(point_type), float(hmin), float(ibm_beta))


def ref_green_local(c, x, point_type=POLYMER_BEAD, ibm_beta=0.75, hmin=1.0):
    """green_tensor_local_regularized of the reference's own GGEMStokes"""
    x = _f64(x)
    G = np.zeros(9)
    rc = ref_ggem_lib().ref_ggem_green_local(*_ref_head(c, point_type, ibm_beta, hmin),
                                             _p(x), _p(G))
    if rc:
        raise ValueError("bad point type")
    return G.reshape(3, 3)


def _box_arrays(box: "Box"):
    lo = np.array([box.lo[d] for d in range(3)])
    hi = np.array([box.hi[d] for d in range(3)])
    per = np.array([box.periodic[d] for d in range(3)], np.int32)
    return lo, hi, per


def ref_local_bead(c, box, xyz, f, nbrs: "Neighbors", point_type=POLYMER_BEAD,
                   ibm_beta=0.75, hmin=1.0):
    """(local_solution_bead, global_self_exclusion) of every bead, from the
    reference's own GGEMStokes over the given neighbour lists"""
    xyz, f = _f64(xyz), _f64(f)
    n = len(xyz)
    off, ids = nbrs.offsets, nbrs.ids
    off = np.ascontiguousarray(off, np.int64)
    ids = np.ascontiguousarray(ids, np.int32)
    lo, hi, per = _box_arrays(box)
    ul, us = np.zeros((n, 3)), np.zeros((n, 3))
    rc = ref_ggem_lib().ref_ggem_local_bead(*_ref_head(c, point_type, ibm_beta, hmin),
                                            _p(lo), _p(hi), _p(per), n, _p(xyz), _p(f),
                                            _p(off), _p(ids), _p(ul), _p(us))
    if rc:
        raise ValueError(f"reference local_solution_bead failed ({rc})")
    return ul, us


def ref_local_field(c, box, elem_nb: "Neighbors", xyz, f, targets, target_elem,
                    point_type=POLYMER_BEAD, ibm_beta=0.75, hmin=1.0):
    """local_solution_field of the reference's own GGEMStokes at targets
    (each given with the element that holds it)"""
    xyz, f, targets = _f64(xyz), _f64(f), _f64(targets)
    off, ids = elem_nb.offsets, elem_nb.ids
    off = np.ascontiguousarray(off, np.int64)
    ids = np.ascontiguousarray(ids, np.int32)
    te = np.ascontiguousarray(target_elem, np.int32)
    lo, hi, per = _box_arrays(box)
    u = np.zeros((len(targets), 3))
    rc = ref_ggem_lib().ref_ggem_local_field(*_ref_head(c, point_type, ibm_beta, hmin),
                                             _p(lo), _p(hi), _p(per), len(xyz), _p(xyz),
                                             _p(f), len(off) - 1, _p(off), _p(ids),
                                             len(targets), _p(targets), _p(te), _p(u))
    if rc:
        raise ValueError(f"reference local_solution_field failed ({rc})")
    return u


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def constants(alpha=0.5, mu=1.0 / (6.0 * np.pi), br0=1.0, point_type=POLYMER_BEAD,
              ibm_beta=0.75, hmin=1.0) -> Consts:
    c = Consts()
    rc = lib().orc_set_constants(mu, alpha, br0, point_type, ibm_beta, hmin, C.byref(c))
    if rc:
        raise ValueError("bad point type")
    return c


def make_box(lo, hi, periodic) -> Box:
    b = Box()
    for d in range(3):
        b.lo[d], b.hi[d], b.periodic[d] = float(lo[d]), float(hi[d]), int(bool(periodic[d]))
    return b


def green_local(c: Consts, x) -> np.ndarray:
    x = _f64(x)
    G = np.zeros(9)
    lib().orc_green_local(C.byref(c), _p(x), _p(G))
    return G.reshape(3, 3)


def green_unbounded_smoothed(c: Consts, x, a) -> np.ndarray:
    x = _f64(x)
    G = np.zeros(9)
    lib().orc_green_unbounded_smoothed(C.byref(c), _p(x), float(a), _p(G))
    return G.reshape(3, 3)


def smoothed_force_exp(c: Consts, r) -> float:
    r = _f64(r)
    return lib().orc_smoothed_force_exp(C.byref(c), _p(r))


def _take_list(nb: NbList):
    n = nb.n
    off = np.ctypeslib.as_array(nb.offsets, shape=(n + 1,)).copy()
    ids = (np.ctypeslib.as_array(nb.ids, shape=(int(off[-1]),)).copy()
           if off[-1] > 0 else np.zeros(0, np.int32))
    return off, ids


class Neighbors:
    """Owning wrapper of an oracle CSR list (freed with the object)."""

    def __init__(self, nb: NbList):
        self.nb = nb
        self.offsets, self.ids = _take_list(nb)

    def __del__(self):
        try:
            lib().orc_free_nblist(C.byref(self.nb))
        except Exception:
            pass

    def lists(self):
        return [self.ids[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self.offsets) - 1)]


def neighbors_cutoff(box: Box, xyz, rc) -> Neighbors:
    xyz = _f64(xyz)
    nb = NbList()
    if lib().orc_build_neighbors_cutoff(C.byref(box), len(xyz), _p(xyz), float(rc), C.byref(nb)):
        raise RuntimeError("cutoff list build failed")
    return Neighbors(nb)


def make_mesh(nx, ny, nz, search_radius_e) -> Mesh:
    m = Mesh()
    m.nx, m.ny, m.nz, m.search_radius_e = int(nx), int(ny), int(nz), float(search_radius_e)
    return m


def neighbors_reference(box: Box, mesh: Mesh, xyz) -> Neighbors:
    xyz = _f64(xyz)
    nb = NbList()
    rc = lib().orc_build_neighbors_reference(C.byref(box), C.byref(mesh), len(xyz), _p(xyz),
                                             C.byref(nb))
    if rc:
        raise RuntimeError(f"reference list build failed ({rc})")
    return Neighbors(nb)


def elem_lists(box: Box, mesh: Mesh, xyz):
    xyz = _f64(xyz)
    nb = NbList()
    eop = np.zeros(len(xyz), np.int32)
    rc = lib().orc_build_elem_lists(C.byref(box), C.byref(mesh), len(xyz), _p(xyz),
                                    C.byref(nb), _p(eop))
    if rc:
        raise RuntimeError(f"element list build failed ({rc})")
    return Neighbors(nb), eop


def local_matvec(c: Consts, box: Box, xyz, nbrs: Neighbors, f, self_mode=SELF_BEAD,
                 nthreads=1) -> np.ndarray:
    xyz = _f64(xyz)
    f = _f64(f)
    n = len(xyz)
    nrhs = f.size // (3 * n)
    u = np.zeros_like(f)
    lib().orc_local_matvec(C.byref(c), C.byref(box), n, _p(xyz), C.byref(nbrs.nb), nrhs,
                           _p(f), _p(u), int(self_mode), int(nthreads))
    return u


def local_field_reference(c, box, mesh, elem_nb: Neighbors, xyz, f, targets):
    xyz, f, targets = _f64(xyz), _f64(f), _f64(targets)
    u = np.zeros((len(targets), 3))
    lib().orc_local_field_reference(C.byref(c), C.byref(box), C.byref(mesh),
                                    C.byref(elem_nb.nb), len(xyz), _p(xyz), _p(f),
                                    len(targets), _p(targets), _p(u))
    return u


def local_field_cutoff(c, box, xyz, f, targets, rc):
    xyz, f, targets = _f64(xyz), _f64(f), _f64(targets)
    u = np.zeros((len(targets), 3))
    lib().orc_local_field_cutoff(C.byref(c), C.byref(box), len(xyz), _p(xyz), _p(f),
                                 float(rc), len(targets), _p(targets), _p(u))
    return u


def exact_unbounded(c, xyz, f, targets):
    xyz, f, targets = _f64(xyz), _f64(f), _f64(targets)
    u = np.zeros((len(targets), 3))
    lib().orc_exact_unbounded(C.byref(c), len(xyz), _p(xyz), _p(f), len(targets),
                              _p(targets), _p(u))
    return u


def spread_qp(c, box, elem_nb, xyz, f, qxyz, qp_elem=None, rc=0.0):
    xyz, f, qxyz = _f64(xyz), _f64(f), _f64(qxyz)
    rho = np.zeros((len(qxyz), 3))
    qe = None if qp_elem is None else np.ascontiguousarray(qp_elem, np.int32)
    lib().orc_spread_qp(C.byref(c), C.byref(box),
                        C.byref(elem_nb.nb) if elem_nb is not None else None,
                        len(xyz), _p(xyz), _p(f), len(qxyz), _p(qxyz),
                        _p(qe) if qe is not None else None, float(rc), _p(rho))
    return rho


def element_rhs(c, box, elem_nb, xyz, f, n_elem, nq, n_u, qxyz, int_force, rc=0.0):
    xyz, f, qxyz, IF = _f64(xyz), _f64(f), _f64(qxyz), _f64(int_force)
    Fe = np.zeros((n_elem, 3 * n_u))
    lib().orc_element_rhs(C.byref(c), C.byref(box),
                          C.byref(elem_nb.nb) if elem_nb is not None else None,
                          len(xyz), _p(xyz), _p(f), int(n_elem), int(nq), int(n_u),
                          _p(qxyz), _p(IF), float(rc), _p(Fe))
    return Fe


def cheb_coeffs(N, da, db, method=0) -> np.ndarray:
    c = np.zeros(N + 1)
    lib().orc_cheb_coeffs(int(N), float(da), float(db), int(method), _p(c))
    return c


def ref_cheb_coeffs(N, da, db, method=0):
    R = ref_lib()
    if R is None:
        return None
    c = np.zeros(N + 1)
    if R.ref_chebyshev_coefficients(int(N), float(da), float(db), int(method), _p(c)):
        raise ValueError("bad arguments")
    return c


class Operator:
    """Wraps a python callable or the oracle matvec as an orc_op_fn."""

    def __init__(self, fn=None, matvec=None, dim=None):
        self.dim = dim
        if matvec is not None:
            c, box, xyz, nbrs, self_mode, nthreads = matvec
            self._keep = (c, box, _f64(xyz), nbrs)
            self.ctx = MatvecCtx(C.pointer(c), C.pointer(box), len(xyz),
                                 self._keep[2].ctypes.data, C.pointer(nbrs.nb),
                                 int(self_mode), int(nthreads))
            self.fn = C.cast(lib().orc_matvec_op, OP_FN)
            self.ctx_p = C.cast(C.pointer(self.ctx), C.c_void_p)
            self.dim = 3 * len(xyz)
        elif fn == "diag":
            self._dim = C.c_int64(dim)
            self.fn = C.cast(lib().orc_diag_test_op, OP_FN)
            self.ctx_p = C.cast(C.pointer(self._dim), C.c_void_p)
        else:
            def _cb(ctx, f, u, _fn=fn, _dim=dim):
                fa = np.ctypeslib.as_array(f, shape=(_dim,))
                ua = np.ctypeslib.as_array(u, shape=(_dim,))
                ua[:] = _fn(fa.copy())
            self.fn = OP_FN(_cb)
            self.ctx_p = None


def cheb_inv_sqrt(op: Operator, dw, N, eig_min, eig_max, tol):
    dw = _f64(dw).copy()
    rep = ChebReport()
    lib().orc_cheb_inv_sqrt(op.fn, op.ctx_p, len(dw), int(N), float(eig_min), float(eig_max),
                            float(tol), _p(dw), C.byref(rep))
    return dw, rep


def lanczos(op: Operator, v0, k):
    v0 = _f64(v0)
    lmin, lmax = C.c_double(), C.c_double()
    a = np.zeros(k)
    b = np.zeros(k)
    m = lib().orc_lanczos(op.fn, op.ctx_p, len(v0), int(k), _p(v0), C.byref(lmin),
                          C.byref(lmax), _p(a), _p(b))
    return lmin.value, lmax.value, a[:m], b[:m]


def tridiag_extremes(a, b):
    a, b = _f64(a), _f64(b)
    lo, hi = C.c_double(), C.c_double()
    lib().orc_tridiag_extremes(len(a), _p(a), _p(b), C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def power_iteration(op: Operator, dim, tol=1e-3, maxits=50):
    eig = C.c_double()
    it = lib().orc_power_iteration(op.fn, op.ctx_p, int(dim), float(tol), int(maxits),
                                   C.byref(eig))
    return it, eig.value


def std_normal_vector(seed, n, mean=0.0, std=1.0, skip_vectors=0):
    out = np.zeros(n)
    lib().orc_std_normal_vector(int(seed), int(skip_vectors), int(n), float(mean), float(std),
                                _p(out))
    return out


def philox_normals(seed, stream, n):
    out = np.zeros(n)
    lib().orc_philox_normals(int(seed), int(stream), int(n), _p(out))
    return out


def ev_gaussian(box: Box, xyz, nbrs: "Neighbors", c1, c2) -> np.ndarray:
    """excluded-volume forces [n][3] (fix_point_gaussian_dna.C:69-84)"""
    xyz = _f64(xyz)
    f = np.zeros_like(xyz)
    lib().orc_ev_gaussian(C.byref(box), len(xyz), _p(xyz), C.byref(nbrs.nb), float(c1),
                          float(c2), _p(f))
    return f


def spring_forces(box: Box, xyz, bonds, kind, c1, Ls) -> np.ndarray:
    """bonded spring forces [n][3] (fix_point_wls.C:66-92 with the law `kind`)"""
    xyz = _f64(xyz)
    b = np.ascontiguousarray(bonds, dtype=np.int64)
    f = np.zeros_like(xyz)
    lib().orc_spring_forces(C.byref(box), len(xyz), _p(xyz), len(b), _p(b), int(kind),
                            float(c1), float(Ls), _p(f))
    return f


def hex20_shape(xi):
    """the 20 serendipity shape functions at reference point xi (Hex20 order)"""
    n = np.zeros(20)
    lib().orc_hex20_shape(float(xi[0]), float(xi[1]), float(xi[2]), _p(n))
    return n


def fem_point_values(xyz, n_elem, lo, hi, periodic, elem_dofs, solution):
    """(U_global [n][3], number of points outside a non-periodic axis):
    point_value of u, v, w on the HEX20 mesh (pm_system_stokes.C:437-441)"""
    xyz = _f64(xyz)
    ne = np.ascontiguousarray(n_elem, dtype=np.int32)
    lo = _f64(lo)
    hi = _f64(hi)
    per = np.ascontiguousarray(periodic, dtype=np.int32)
    dofs = np.ascontiguousarray(elem_dofs, dtype=np.int64)
    sol = _f64(solution)
    u = np.zeros((len(xyz), 3))
    out = lib().orc_fem_point_values(len(xyz), _p(xyz), _p(ne), _p(lo), _p(hi), _p(per),
                                     _p(dofs), _p(sol), _p(u))
    return u, int(out)
