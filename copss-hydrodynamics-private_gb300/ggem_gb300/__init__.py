"""Python binding of the GB300 GGEM library (ctypes over the C ABI).

The compute path is ``_lib/libggem_gb300.so`` (hand-written CUDA for
sm_103a); this module only marshals arguments.  There is no CPU fallback:
if the library is missing, :func:`lib` raises.

Layout conventions follow the reference's PETSc vectors
(brownian_system.C:72-75): forces and velocities are ``[nrhs, n, 3]``
float64, positions ``[n, 3]`` float64.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libggem_gb300.so"

GGEM_OK = 0
POLYMER_BEAD, LAGRANGIAN_POINT, POINT_PARTICLE = 0, 1, 2  # point_particle.h:36-41
SELF_NONE, SELF_BEAD, SELF_LAGRANGIAN = 0, 1, 2
NB_REFERENCE, NB_CUTOFF = 0, 1
FP64, FP32 = 0, 1
CHEB_GAUSS, CHEB_GAUSS_RADAU, CHEB_GAUSS_LOBATTO = 0, 1, 2
ERR_BAD_ARG, ERR_CUDA, ERR_CELL_OVERFLOW, ERR_TIMEOUT = -1, -2, -3, -4
ERR_NOT_SPD, ERR_CHEB_NOT_CONVERGED, ERR_SURROGATE_REJECTED = -5, -6, -7
ERR_OUT_OF_DOMAIN, ERR_NO_DEVICE, ERR_OOM, ERR_INVALID_RANGE = -8, -9, -10, -11
KERNEL_PAIR_FP32, KERNEL_PAIR_FP64, KERNEL_CHEB_TERM, KERNEL_LIST_BUILD, KERNEL_PAIR_CHEB = (
    0, 1, 2, 3, 4)
SPRING_WLS, SPRING_FENE, SPRING_UD, SPRING_LHS = 0, 1, 2, 3


class Params(C.Structure):
    _fields_ = [("mu", C.c_double), ("alpha", C.c_double), ("br0", C.c_double),
                ("point_type", C.c_int), ("ibm_beta", C.c_double), ("hmin", C.c_double),
                ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3),
                ("periodic", C.c_int * 3), ("nb_mode", C.c_int), ("rc", C.c_double),
                ("n_mesh", C.c_int * 3), ("search_radius_e", C.c_double),
                ("precision", C.c_int), ("cell_div", C.c_int), ("device", C.c_int)]


class Constants(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "mu", "alpha", "ksi", "br0", "one_eight_pi_mu", "alpha2", "alpha3",
        "alpha3_pi_23", "two_alpha_sqrt_pi", "coeff_1", "ksi2", "ksi3",
        "ksi3_pi_23", "two_ksi_sqrt_pi", "coeff_2", "r_eps")]


class ChebReport(C.Structure):
    _fields_ = [("converged", C.c_int), ("n_terms", C.c_int), ("n_matvecs", C.c_int),
                ("err1", C.c_double), ("err2", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PolymerData(C.Structure):
    _fields_ = [("n_beads", C.c_int64), ("n_bonds", C.c_int64), ("n_bead_types", C.c_int),
                ("n_bond_types", C.c_int), ("n_chains", C.c_int), ("has_box", C.c_int),
                ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3),
                ("xyz", C.POINTER(C.c_double)), ("chain_id", C.POINTER(C.c_int32)),
                ("bead_type", C.POINTER(C.c_int32)), ("rot", C.POINTER(C.c_double)),
                ("const_force", C.POINTER(C.c_double)), ("charge", C.POINTER(C.c_double)),
                ("mass", C.POINTER(C.c_double)), ("bonds", C.POINTER(C.c_int64)),
                ("bond_type", C.POINTER(C.c_int32))]


class GGEMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ggem error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run ggem_gb300.build.build() first "
                           "(the GGEM path has no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    vp, i64, d, i = C.c_void_p, C.c_int64, C.c_double, C.c_int
    P = C.POINTER
    sig = {
        "ggem_default_params": (None, [P(Params)]),
        "ggem_create": (i, [P(Params), P(vp)]),
        "ggem_destroy": (None, [vp]),
        "ggem_strerror": (C.c_char_p, [i]),
        "ggem_last_error": (C.c_char_p, [vp]),
        "ggem_get_constants": (i, [vp, P(Constants)]),
        "ggem_set_stream": (i, [vp, vp]),
        "ggem_synchronize": (i, [vp]),
        "ggem_set_particles": (i, [vp, i64, vp]),
        "ggem_set_particles_dev": (i, [vp, i64, vp]),
        "ggem_build_cells": (i, [vp]),
        "ggem_set_deferred_checks": (i, [vp, i]),
        "ggem_neighbor_pair_count": (i, [vp, P(i64)]),
        "ggem_get_neighbors": (i, [vp, vp, vp, i64]),
        "ggem_get_cell_of_particles": (i, [vp, vp]),
        "ggem_local_matvec": (i, [vp, i, vp, vp, i]),
        "ggem_local_matvec_dev": (i, [vp, i, vp, vp, i]),
        "ggem_green_tensor_local": (i, [vp, i64, vp, vp]),
        "ggem_local_field": (i, [vp, i64, vp, vp, vp]),
        "ggem_spread_qp": (i, [vp, i64, vp, vp, vp, d, vp]),
        "ggem_element_rhs": (i, [vp, i64, i, i, vp, vp, vp, d, vp]),
        "ggem_spread_qp_dev": (i, [vp, i64, vp, vp, vp, d, vp]),
        "ggem_set_quadrature": (i, [vp, i, vp]),
        "ggem_set_quadrature_dev": (i, [vp, i, vp]),
        "ggem_spread_elements": (i, [vp, i, vp, vp]),
        "ggem_spread_elements_dev": (i, [vp, i, vp, vp, P(i64)]),
        "ggem_cheb_coeffs": (i, [i, d, d, i, vp]),
        "ggem_cheb_inv_sqrt": (i, [vp, i, i, d, d, d, i, vp, P(ChebReport)]),
        "ggem_cheb_inv_sqrt_dev": (i, [vp, i, i, d, d, d, i, vp, P(ChebReport)]),
        "ggem_brownian_displacement": (i, [vp, i, i, d, d, d, i, vp, vp, P(ChebReport)]),
        "ggem_brownian_displacement_dev": (i, [vp, i, i, d, d, d, i, vp, vp, P(ChebReport)]),
        "ggem_get_launch_count": (i, [vp, P(i64)]),
        "ggem_get_pair_count": (i, [vp, P(i64)]),
        "ggem_get_pair_storage": (i, [vp, P(i), P(i)]),
        "ggem_set_pair_tensors": (i, [vp, i]),
        "ggem_set_fp64_pair_list": (i, [vp, i]),
        "ggem_set_symmetric_pairs": (i, [vp, i]),
        "ggem_autotune_pair_storage": (i, [vp, i, d, P(i), P(d), P(d), P(i)]),
        "ggem_set_pair_variant": (i, [vp, i, i]),
        "ggem_probe_fp32_peak": (i, [vp, P(d)]),
        "ggem_set_kernel_timing": (i, [vp, i]),
        "ggem_set_kernel_timing_kinds": (i, [vp, i, C.c_uint]),
        "ggem_set_series_graphs": (i, [vp, i]),
        "ggem_get_series_graph_stats": (i, [vp, P(i64), P(i64)]),
        "ggem_set_launch_trace": (i, [vp, i]),
        "ggem_diag_convert_f32": (i, [vp, i64, vp, vp, vp]),
        "ggem_get_launch_trace": (i, [vp, i64, vp, vp, P(i64)]),
        "ggem_get_kernel_timing": (i, [vp, i, P(d), P(i64)]),
        "ggem_lanczos_bounds": (i, [vp, i, C.c_uint64, P(d), P(d)]),
        "ggem_power_iteration": (i, [vp, d, i, P(d)]),
        "ggem_std_random_vector": (i, [C.c_uint64, i64, i64, d, d, vp]),
        "ggem_philox_normals_dev": (i, [vp, C.c_uint64, C.c_uint64, i64, vp]),
        "ggem_make_suspension": (i, [C.c_uint64, i64, d, d, vp, P(d)]),
        "ggem_make_chains": (i, [C.c_uint64, i64, i, d, d, d, vp, P(d)]),
        "ggem_make_normals": (i, [C.c_uint64, i64, vp]),
        "ggem_make_mixture": (i, [C.c_uint64, i64, i, i64, d, d, d, vp, P(d)]),
        "ggem_surrogate_create": (vp, [i, C.c_uint64]),
        "ggem_surrogate_destroy": (None, [vp]),
        "ggem_surrogate_last_error": (C.c_char_p, [vp]),
        "ggem_surrogate_set_norm": (i, [vp, vp]),
        "ggem_surrogate_get_norm": (i, [vp, vp]),
        "ggem_surrogate_set_params": (i, [vp, vp]),
        "ggem_surrogate_get_params": (i, [vp, vp]),
        "ggem_surrogate_train": (i, [vp, vp, vp, i64, i, i, C.c_float, C.c_uint64, vp]),
        "ggem_surrogate_predict": (i, [vp, vp, i64, vp]),
        "ggem_surrogate_predict_layers": (i, [vp, vp, i64, vp]),
        "ggem_surrogate_set_poll_budget": (i, [vp, C.c_uint32]),
        "ggem_surrogate_time_forward": (i, [vp, i64, i, P(d)]),
        "ggem_surrogate_gradient": (i, [vp, vp, vp, i64, P(C.c_float), vp]),
        "ggem_surrogate_features": (i, [vp, d, vp]),
        "ggem_surrogate_interval": (i, [vp, vp, d, d, d, P(d), P(d)]),
        "ggem_ev_gaussian_forces": (i, [vp, d, d, vp, i]),
        "ggem_ev_gaussian_forces_dev": (i, [vp, d, d, vp, i]),
        "ggem_set_bonds": (i, [vp, i64, vp]),
        "ggem_spring_forces": (i, [vp, i, d, d, vp, i]),
        "ggem_spring_forces_dev": (i, [vp, i, d, d, vp, i]),
        "ggem_read_polymer_data": (i, [C.c_char_p, P(PolymerData)]),
        "ggem_read_polymer_vtk": (i, [C.c_char_p, P(PolymerData)]),
        "ggem_free_polymer_data": (None, [P(PolymerData)]),
        "ggem_write_polymer_vtk": (i, [C.c_char_p, i64, vp, i64, vp, vp, i]),
        "ggem_write_bead_csv": (i, [C.c_char_p, i64, vp, vp, vp, i]),
        "ggem_write_petsc_vec": (i, [C.c_char_p, i64, vp]),
        "ggem_read_petsc_vec": (i, [C.c_char_p, i64, vp, P(i64)]),
        "ggem_fem_create": (i, [vp, vp, vp, vp, i64, vp, P(vp)]),
        "ggem_fem_destroy": (None, [vp]),
        "ggem_fem_point_values": (i, [vp, vp, vp, i]),
        "ggem_fem_point_values_dev": (i, [vp, vp, vp, i]),
        "ggem_fem_hex20_shape": (None, [vp, vp]),
        "ggem_ensemble_create": (i, [P(Params), i, vp, P(vp)]),
        "ggem_ensemble_destroy": (None, [vp]),
        "ggem_ensemble_last_error": (C.c_char_p, [vp]),
        "ggem_ensemble_set_particles_dev": (i, [vp, vp, vp]),
        "ggem_ensemble_sizes": (i, [vp, P(i64), P(i64)]),
        "ggem_ensemble_matvec_dev": (i, [vp, i, vp, vp, i]),
        "ggem_ensemble_brownian_dev": (i, [vp, i, i, vp, vp, d, vp, vp, P(ChebReport)]),
        "ggem_ensemble_intervals": (i, [vp, vp, vp, d, d, vp, vp]),
        "ggem_ensemble_lanczos": (i, [vp, i, i, C.c_uint64, P(d), P(d)]),
        "ggem_ensemble_autotune": (i, [vp, i, P(i), P(d)]),
        "ggem_ensemble_set_series_mode": (i, [vp, i, i, C.c_uint32, i]),
        "ggem_ensemble_autotune_series": (i, [vp, i, i, vp, vp, d, vp, vp, C.c_char_p, P(i),
                                              P(i), P(d)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _nrhs(x: np.ndarray, n: int) -> int:
    """right-hand sides in x ([nrhs][n][3] or [n][3]); for a context without
    particles the leading dimension of a 3-D array, else one"""
    if n:
        return x.size // (3 * n)
    return x.shape[0] if x.ndim == 3 else 1


def cheb_coeffs(N, da, db, method=CHEB_GAUSS) -> np.ndarray:
    c = np.zeros(N + 1)
    rc = lib().ggem_cheb_coeffs(int(N), float(da), float(db), int(method), _p(c))
    if rc:
        raise GGEMError(rc, lib().ggem_strerror(rc).decode())
    return c


def std_random_vector(seed, n, mean=0.0, std=1.0, skip_vectors=0) -> np.ndarray:
    out = np.zeros(n)
    rc = lib().ggem_std_random_vector(int(seed), int(skip_vectors), int(n), float(mean),
                                      float(std), _p(out))
    if rc:
        raise GGEMError(rc, "bad arguments")
    return out


def make_suspension(seed, n, phi, radius=1.0):
    xyz = np.zeros((n, 3))
    L = C.c_double()
    rc = lib().ggem_make_suspension(int(seed), int(n), float(phi), float(radius), _p(xyz),
                                    C.byref(L))
    if rc:
        raise GGEMError(rc, "suspension generation failed")
    return xyz, L.value


def make_mixture(seed, n_chains, beads, n_free, bond=2.0, phi=0.05, radius=1.0):
    """n_chains chains of `beads` beads followed by n_free free beads."""
    xyz = np.zeros((n_chains * beads + n_free, 3))
    L = C.c_double()
    rc = lib().ggem_make_mixture(int(seed), int(n_chains), int(beads), int(n_free), float(bond),
                                 float(phi), float(radius), _p(xyz), C.byref(L))
    if rc:
        raise GGEMError(rc, "mixture generation failed")
    return xyz, L.value


SUR_FEATURES, SUR_OUTPUTS, SUR_HIST_BINS = 35, 2, 32
SUR_PARAMS = 128 * 48 + 128 + 3 * (128 * 128 + 128)
SUR_NORM = 2 * SUR_FEATURES + 2 * SUR_OUTPUTS


class Surrogate:
    """The eigen-interval network (include/ggem_surrogate.h): BF16 MLP
    35 -> 128 -> 128 -> 128 -> 2 trained and evaluated by the library's
    tensor-core kernels."""

    def __init__(self, device=0, seed=1):
        self.h = lib().ggem_surrogate_create(int(device), int(seed))
        if not self.h:
            raise GGEMError(ERR_NO_DEVICE, "surrogate: no usable CUDA device")

    def close(self):
        if self.h:
            lib().ggem_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise GGEMError(rc, (lib().ggem_surrogate_last_error(self.h) or b"").decode())

    @property
    def norm(self) -> np.ndarray:
        out = np.zeros(SUR_NORM, dtype=np.float32)
        self._check(lib().ggem_surrogate_get_norm(self.h, _p(out)))
        return out

    @norm.setter
    def norm(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        assert v.size == SUR_NORM
        self._check(lib().ggem_surrogate_set_norm(self.h, _p(v)))

    def fit_norm(self, X, Y):
        """Feature and output mean / std from a training set."""
        X = np.asarray(X, dtype=np.float64)
        Y = np.asarray(Y, dtype=np.float64)
        sd = X.std(axis=0)
        sd[sd < 1e-6] = 1.0
        ysd = Y.std(axis=0)
        ysd[ysd < 1e-6] = 1.0
        self.norm = np.concatenate([X.mean(axis=0), sd, Y.mean(axis=0), ysd])

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(SUR_PARAMS, dtype=np.float32)
        self._check(lib().ggem_surrogate_get_params(self.h, _p(out)))
        return out

    @params.setter
    def params(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        assert v.size == SUR_PARAMS
        self._check(lib().ggem_surrogate_set_params(self.h, _p(v)))

    def train(self, X, Y, epochs, batch=256, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = np.zeros(epochs, dtype=np.float32)
        self._check(lib().ggem_surrogate_train(self.h, _p(X), _p(Y), len(X), int(epochs),
                                               int(batch), float(lr), int(seed), _p(loss)))
        return loss

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float32)
        Y = np.zeros((len(X), SUR_OUTPUTS), dtype=np.float32)
        self._check(lib().ggem_surrogate_predict(self.h, _p(X), len(X), _p(Y)))
        return Y

    def predict_layers(self, X) -> np.ndarray:
        """the layer-by-layer path of training (one product per layer)"""
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float32)
        Y = np.zeros((len(X), SUR_OUTPUTS), dtype=np.float32)
        self._check(lib().ggem_surrogate_predict_layers(self.h, _p(X), len(X), _p(Y)))
        return Y

    def set_poll_budget(self, polls):
        """test hook: polls of the first mbarrier wait of every product"""
        self._check(lib().ggem_surrogate_set_poll_budget(self.h, int(polls)))

    def time_forward(self, n, reps=50):
        """mean ms of the one-kernel forward pass over n rows"""
        ms = C.c_double()
        self._check(lib().ggem_surrogate_time_forward(self.h, int(n), int(reps), C.byref(ms)))
        return ms.value

    def gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.zeros(SUR_PARAMS, dtype=np.float32)
        loss = C.c_float()
        self._check(lib().ggem_surrogate_gradient(self.h, _p(X), _p(Y), len(X), C.byref(loss),
                                                  _p(g)))
        return loss.value, g

    def save(self, path):
        np.savez(path, params=self.params, norm=self.norm)

    def load(self, path):
        d = np.load(path)
        self.norm = d["norm"]
        self.params = d["params"]


def make_chains(seed, n_chains, beads, bond=2.0, phi=0.05, radius=1.0):
    xyz = np.zeros((n_chains * beads, 3))
    L = C.c_double()
    rc = lib().ggem_make_chains(int(seed), int(n_chains), int(beads), float(bond), float(phi),
                                float(radius), _p(xyz), C.byref(L))
    if rc:
        raise GGEMError(rc, "chain generation failed")
    return xyz, L.value


def make_normals(seed, n) -> np.ndarray:
    out = np.zeros(n)
    rc = lib().ggem_make_normals(int(seed), int(n), _p(out))
    if rc:
        raise GGEMError(rc, "bad arguments")
    return out


def default_params() -> Params:
    p = Params()
    lib().ggem_default_params(C.byref(p))
    return p


class Context:
    """One GGEM context: constants, box, cell lists and device workspaces."""

    def __init__(self, *, alpha=0.5, mu=None, br0=1.0, point_type=POLYMER_BEAD,
                 ibm_beta=0.75, hmin=1.0, box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0),
                 periodic=(1, 1, 1), nb_mode=NB_CUTOFF, rc=7.0, n_mesh=(1, 1, 1),
                 search_radius_e=0.0, precision=FP32, cell_div=0, device=0):
        p = default_params()
        if mu is not None:
            p.mu = float(mu)
        p.alpha, p.br0, p.point_type = float(alpha), float(br0), int(point_type)
        p.ibm_beta, p.hmin = float(ibm_beta), float(hmin)
        for k in range(3):
            p.box_lo[k], p.box_hi[k] = float(box_lo[k]), float(box_hi[k])
            p.periodic[k] = int(bool(periodic[k]))
            p.n_mesh[k] = int(n_mesh[k])
        p.nb_mode, p.rc, p.search_radius_e = int(nb_mode), float(rc), float(search_radius_e)
        p.precision, p.cell_div, p.device = int(precision), int(cell_div), int(device)
        self.params = p
        h = C.c_void_p()
        rc_ = lib().ggem_create(C.byref(p), C.byref(h))
        if rc_:
            raise GGEMError(rc_, lib().ggem_strerror(rc_).decode())
        self.h = h
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            lib().ggem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc < 0:
            raise GGEMError(rc, lib().ggem_last_error(self.h).decode())
        return rc

    def constants(self) -> Constants:
        c = Constants()
        self._check(lib().ggem_get_constants(self.h, C.byref(c)))
        return c

    def set_stream(self, stream_ptr):
        self._check(lib().ggem_set_stream(self.h, C.c_void_p(stream_ptr or None)))

    def synchronize(self):
        self._check(lib().ggem_synchronize(self.h))

    def set_particles(self, xyz):
        xyz = _f64(xyz).reshape(-1, 3)
        self._check(lib().ggem_set_particles(self.h, len(xyz), _p(xyz)))
        self.n = len(xyz)

    def set_particles_dev(self, d_ptr, n):
        self._check(lib().ggem_set_particles_dev(self.h, int(n), C.c_void_p(d_ptr)))
        self.n = int(n)

    def build_cells(self):
        self._check(lib().ggem_build_cells(self.h))

    def set_deferred_checks(self, enable: bool):
        """builds after the first keep the row width and return without
        waiting; their statistics are read by the next synchronising call"""
        self._check(lib().ggem_set_deferred_checks(self.h, 1 if enable else 0))

    def pair_count(self) -> int:
        v = C.c_int64()
        self._check(lib().ggem_neighbor_pair_count(self.h, C.byref(v)))
        return v.value

    def neighbors(self):
        off = np.zeros(self.n + 1, np.int64)
        self._check(lib().ggem_get_neighbors(self.h, _p(off), None, 0))
        ids = np.zeros(max(int(off[-1]), 1), np.int32)
        self._check(lib().ggem_get_neighbors(self.h, _p(off), _p(ids), len(ids)))
        return off, ids[:off[-1]]

    def cell_of_particles(self):
        out = np.zeros(self.n, np.int32)
        self._check(lib().ggem_get_cell_of_particles(self.h, _p(out)))
        return out

    def local_matvec(self, f, self_mode=SELF_BEAD):
        f = _f64(f)
        nrhs = f.size // (3 * self.n) if self.n else 1
        u = np.zeros_like(f)
        self._check(lib().ggem_local_matvec(self.h, nrhs, _p(f), _p(u), int(self_mode)))
        return u

    def local_matvec_dev(self, d_f, d_u, nrhs=1, self_mode=SELF_BEAD):
        self._check(lib().ggem_local_matvec_dev(self.h, int(nrhs), C.c_void_p(d_f),
                                                C.c_void_p(d_u), int(self_mode)))

    def green_tensor_local(self, x):
        x = _f64(x).reshape(-1, 3)
        G = np.zeros((len(x), 3, 3))
        self._check(lib().ggem_green_tensor_local(self.h, len(x), _p(x), _p(G)))
        return G

    def local_field(self, targets, f):
        t = _f64(targets).reshape(-1, 3)
        f = _f64(f)
        u = np.zeros_like(t)
        self._check(lib().ggem_local_field(self.h, len(t), _p(t), _p(f), _p(u)))
        return u

    def spread_qp(self, qxyz, f, qp_elem=None, spread_rc=0.0):
        q = _f64(qxyz).reshape(-1, 3)
        f = _f64(f)
        rho = np.zeros_like(q)
        qe = None if qp_elem is None else np.ascontiguousarray(qp_elem, np.int32)
        self._check(lib().ggem_spread_qp(self.h, len(q), _p(q), _p(qe) if qe is not None else None,
                                         _p(f), float(spread_rc), _p(rho)))
        return rho

    def element_rhs(self, n_elem, nq, n_u, qxyz, int_force, f, spread_rc=0.0):
        q, IF, f = _f64(qxyz), _f64(int_force), _f64(f)
        Fe = np.zeros((n_elem, 3 * n_u))
        self._check(lib().ggem_element_rhs(self.h, int(n_elem), int(nq), int(n_u), _p(q), _p(IF),
                                           _p(f), float(spread_rc), _p(Fe)))
        return Fe

    def spread_qp_dev(self, nq, d_qxyz, d_qp_elem, d_f, d_rho, spread_rc=0.0):
        self._check(lib().ggem_spread_qp_dev(self.h, int(nq), C.c_void_p(d_qxyz),
                                             C.c_void_p(d_qp_elem), C.c_void_p(d_f),
                                             float(spread_rc), C.c_void_p(d_rho)))

    def set_quadrature(self, qxyz, nq_per_elem):
        """element-major quadrature points [n_elem * nq][3] (reference mode)"""
        q = _f64(qxyz).reshape(-1, 3)
        self._check(lib().ggem_set_quadrature(self.h, int(nq_per_elem), _p(q)))
        self.nq_per_elem = int(nq_per_elem)
        self.n_qp = len(q)

    def set_quadrature_dev(self, d_qxyz, nq_per_elem, n_qp):
        self._check(lib().ggem_set_quadrature_dev(self.h, int(nq_per_elem), C.c_void_p(d_qxyz)))
        self.nq_per_elem = int(nq_per_elem)
        self.n_qp = int(n_qp)

    def spread_elements(self, f, precision=FP64):
        """rho [n_elem * nq][3] at every quadrature point of every element"""
        f = _f64(f)
        rho = np.zeros((self.n_qp, 3))
        self._check(lib().ggem_spread_elements(self.h, int(precision), _p(f), _p(rho)))
        return rho

    def spread_elements_dev(self, d_f, d_rho, precision=FP64, count_pairs=False):
        """the device-pointer form; returns the (point, particle) pair count
        when count_pairs (one host synchronisation)"""
        pairs = C.c_int64(0)
        self._check(lib().ggem_spread_elements_dev(self.h, int(precision), C.c_void_p(d_f),
                                                   C.c_void_p(d_rho),
                                                   C.byref(pairs) if count_pairs else None))
        return pairs.value if count_pairs else None

    def cheb_inv_sqrt(self, xi, N, eig_min, eig_max, tol, check_every=1):
        xi = _f64(xi).copy()
        nrhs = _nrhs(xi, self.n)
        reps = (ChebReport * nrhs)()
        self._check(lib().ggem_cheb_inv_sqrt(self.h, nrhs, int(N), float(eig_min), float(eig_max),
                                             float(tol), int(check_every), _p(xi), reps))
        return xi, [r.as_dict() for r in reps]

    def cheb_inv_sqrt_dev(self, d_xi, nrhs, N, eig_min, eig_max, tol, check_every=1):
        reps = (ChebReport * nrhs)()
        self._check(lib().ggem_cheb_inv_sqrt_dev(self.h, int(nrhs), int(N), float(eig_min),
                                                 float(eig_max), float(tol), int(check_every),
                                                 C.c_void_p(d_xi), reps))
        return [r.as_dict() for r in reps]

    def brownian_displacement_dev(self, d_xi, d_dw, nrhs, N, eig_min, eig_max, tol,
                                  check_every=1):
        reps = (ChebReport * nrhs)()
        rc = lib().ggem_brownian_displacement_dev(self.h, int(nrhs), int(N), float(eig_min),
                                                  float(eig_max), float(tol), int(check_every),
                                                  C.c_void_p(d_xi), C.c_void_p(d_dw), reps)
        return rc, [r.as_dict() for r in reps]

    def brownian_displacement(self, xi, N, eig_min, eig_max, tol, check_every=1):
        xi = _f64(xi)
        nrhs = _nrhs(xi, self.n)
        dw = np.zeros_like(xi)
        reps = (ChebReport * nrhs)()
        rc = lib().ggem_brownian_displacement(self.h, nrhs, int(N), float(eig_min),
                                              float(eig_max), float(tol), int(check_every),
                                              _p(xi), _p(dw), reps)
        return rc, dw, [r.as_dict() for r in reps]

    def launch_count(self) -> int:
        v = C.c_int64()
        self._check(lib().ggem_get_launch_count(self.h, C.byref(v)))
        return v.value

    def set_kernel_timing(self, enable: bool, kinds=None):
        """CUDA-event timing of the library's kernels (totals reset); kinds,
        an iterable of KERNEL_* values, restricts it to those kernels"""
        if kinds is None:
            self._check(lib().ggem_set_kernel_timing(self.h, int(bool(enable))))
        else:
            mask = 0
            for k in kinds:
                mask |= 1 << int(k)
            self._check(lib().ggem_set_kernel_timing_kinds(self.h, int(bool(enable)), mask))

    def set_series_graphs(self, enable: bool):
        self._check(lib().ggem_set_series_graphs(self.h, int(bool(enable))))

    def series_graph_stats(self):
        """(graphs captured, replays launched) of the series prefix graph"""
        a, b = C.c_int64(), C.c_int64()
        self._check(lib().ggem_get_series_graph_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_launch_trace(self, enable: bool):
        self._check(lib().ggem_set_launch_trace(self.h, int(bool(enable))))

    def launch_trace(self, max_events=100000):
        """[(ms from the trace start, launch name)] of the traced launches"""
        t = np.zeros(max_events)
        names = (C.c_char_p * max_events)()
        n = C.c_int64()
        self._check(lib().ggem_get_launch_trace(self.h, max_events, _p(t), names, C.byref(n)))
        m = min(n.value, max_events)
        return [(float(t[k]), names[k].decode()) for k in range(m)]

    def set_fp64_pair_list(self, enable: bool):
        """FP64 cutoff contexts: walk the exact pair list instead of the cells"""
        self._check(lib().ggem_set_fp64_pair_list(self.h, 1 if enable else 0))

    def set_symmetric_pairs(self, enable: bool):
        """FP32 cutoff contexts: evaluate each unordered pair once (half list)"""
        self._check(lib().ggem_set_symmetric_pairs(self.h, 1 if enable else 0))

    def set_pair_tensors(self, enable: bool):
        self._check(lib().ggem_set_pair_tensors(self.h, 1 if enable else 0))

    def autotune_pair_storage(self, reps=10, matvecs_per_build=12.0):
        """(use_stored, ms per matvec computed, ms per matvec stored incl. the
        amortised tensor pass); the faster form and the fastest kernel shape
        of each stay selected (``pair_variants``: computed, stored)"""
        u, a, b, v = C.c_int(), C.c_double(), C.c_double(), (C.c_int * 2)()
        self._check(lib().ggem_autotune_pair_storage(self.h, int(reps), float(matvecs_per_build),
                                                     C.byref(u), C.byref(a), C.byref(b), v))
        self.pair_variants = (v[0], v[1])
        return bool(u.value), a.value, b.value

    def set_pair_variant(self, computed=0, stored=0):
        """kernel shapes: computed 0 (registers capped for 6) or 1 (for 5
        blocks per SM); stored 0 .. 3"""
        self._check(lib().ggem_set_pair_variant(self.h, int(computed), int(stored)))

    def pair_storage(self):
        """(row width, whether per-pair tensors are stored)"""
        w, t = C.c_int(), C.c_int()
        self._check(lib().ggem_get_pair_storage(self.h, C.byref(w), C.byref(t)))
        return w.value, bool(t.value)

    def kernel_timing(self, kernel: int):
        t, n = C.c_double(), C.c_int64()
        self._check(lib().ggem_get_kernel_timing(self.h, int(kernel), C.byref(t), C.byref(n)))
        return t.value, n.value

    def probe_fp32_peak(self) -> float:
        v = C.c_double()
        self._check(lib().ggem_probe_fp32_peak(self.h, C.byref(v)))
        return v.value

    def lanczos_bounds(self, k=30, seed=1):
        lo, hi = C.c_double(), C.c_double()
        self._check(lib().ggem_lanczos_bounds(self.h, int(k), int(seed), C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def ev_gaussian_forces(self, c1, c2, f=None):
        """excluded-volume forces [n][3], added to f when given"""
        out = np.zeros((self.n, 3)) if f is None else _f64(f).reshape(self.n, 3).copy()
        self._check(lib().ggem_ev_gaussian_forces(self.h, float(c1), float(c2), _p(out),
                                                  0 if f is None else 1))
        return out

    def set_bonds(self, bonds):
        b = np.ascontiguousarray(bonds, dtype=np.int64).reshape(-1, 2)
        self._check(lib().ggem_set_bonds(self.h, len(b), _p(b)))

    def spring_forces(self, kind, c1, Ls, f=None):
        """bonded spring forces [n][3], added to f when given"""
        out = np.zeros((self.n, 3)) if f is None else _f64(f).reshape(self.n, 3).copy()
        self._check(lib().ggem_spring_forces(self.h, int(kind), float(c1), float(Ls), _p(out),
                                             0 if f is None else 1))
        return out

    def surrogate_features(self, chain_fraction=0.0) -> np.ndarray:
        f = np.zeros(SUR_FEATURES, dtype=np.float32)
        self._check(lib().ggem_surrogate_features(self.h, float(chain_fraction), _p(f)))
        return f

    def surrogate_interval(self, sur, chain_fraction=0.0, margin_lo=0.0, margin_hi=0.0):
        lo, hi = C.c_double(), C.c_double()
        self._check(lib().ggem_surrogate_interval(self.h, sur.h, float(chain_fraction),
                                                  float(margin_lo), float(margin_hi),
                                                  C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def power_iteration(self, tol=1e-3, maxits=50):
        e = C.c_double()
        it = self._check(lib().ggem_power_iteration(self.h, float(tol), int(maxits), C.byref(e)))
        return it, e.value

    def philox_normals_dev(self, seed, stream, n, d_out):
        self._check(lib().ggem_philox_normals_dev(self.h, int(seed), int(stream), int(n),
                                                  C.c_void_p(d_out)))


def hex20_shape(xi):
    """the 20 serendipity shape functions at reference point xi (include/ggem_fem.h)"""
    x = np.ascontiguousarray(xi, dtype=np.float64)
    n = np.zeros(20)
    lib().ggem_fem_hex20_shape(_p(x), _p(n))
    return n


class Fem:
    """The HEX20 mesh of the FEM velocity (include/ggem_fem.h): point values
    of u, v, w at the particles of `ctx`.  elem_dofs is [n_elem][3][20]."""

    def __init__(self, ctx, n_elem, lo, hi, n_dofs, elem_dofs):
        self.ctx = ctx
        ne = np.ascontiguousarray(n_elem, dtype=np.int32)
        self._lo = np.ascontiguousarray(lo, dtype=np.float64)
        self._hi = np.ascontiguousarray(hi, dtype=np.float64)
        dofs = np.ascontiguousarray(elem_dofs, dtype=np.int64)
        self.n_dofs = int(n_dofs)
        h = C.c_void_p()
        ctx._check(lib().ggem_fem_create(ctx.h, _p(ne), _p(self._lo), _p(self._hi),
                                         self.n_dofs, _p(dofs), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ggem_fem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def point_values(self, solution, u=None, accumulate=False):
        """U_global [n][3] at the context's particles (added to u when
        accumulate)"""
        sol = _f64(solution)
        out = np.zeros((self.ctx.n, 3)) if u is None else _f64(u).reshape(self.ctx.n, 3).copy()
        self.ctx._check(lib().ggem_fem_point_values(self.h, _p(sol), _p(out),
                                                    1 if accumulate else 0))
        return out

    def point_values_dev(self, d_solution, d_u, accumulate=False):
        self.ctx._check(lib().ggem_fem_point_values_dev(self.h, C.c_void_p(d_solution),
                                                        C.c_void_p(d_u), 1 if accumulate else 0))


class Ensemble:
    """K periodic suspensions as one block-diagonal operator
    (include/ggem_ensemble.h).  Vectors are device arrays [bead][nrhs][3]
    float64 in ensemble order (the suspensions' beads concatenated)."""

    def __init__(self, box_lengths, *, alpha=0.5, mu=None, br0=1.0, point_type=POLYMER_BEAD,
                 rc=7.0, cell_div=0, device=0):
        p = default_params()
        if mu is not None:
            p.mu = float(mu)
        p.alpha, p.br0, p.point_type = float(alpha), float(br0), int(point_type)
        p.rc, p.cell_div, p.device = float(rc), int(cell_div), int(device)
        p.precision, p.nb_mode = FP32, NB_CUTOFF
        self.box = np.ascontiguousarray(box_lengths, dtype=np.float64)
        self.K = len(self.box)
        h = C.c_void_p()
        rc_ = lib().ggem_ensemble_create(C.byref(p), self.K, _p(self.box), C.byref(h))
        if rc_:
            raise GGEMError(rc_, lib().ggem_strerror(rc_).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().ggem_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            raise GGEMError(rc, (lib().ggem_ensemble_last_error(self.h) or b"").decode())
        return rc

    def set_particles_dev(self, n, d_xyz):
        self.n = np.ascontiguousarray(n, dtype=np.int64)
        self._check(lib().ggem_ensemble_set_particles_dev(self.h, _p(self.n), C.c_void_p(d_xyz)))

    def sizes(self):
        b, q = C.c_int64(), C.c_int64()
        self._check(lib().ggem_ensemble_sizes(self.h, C.byref(b), C.byref(q)))
        return b.value, q.value

    def matvec_dev(self, nrhs, d_f, d_u, self_mode=SELF_BEAD):
        self._check(lib().ggem_ensemble_matvec_dev(self.h, int(nrhs), C.c_void_p(d_f),
                                                   C.c_void_p(d_u), int(self_mode)))

    def brownian_dev(self, nrhs, N, eig_min, eig_max, tol, d_xi, d_dw):
        """(return code, reports [K][nrhs]); GGEM_ERR_CHEB_NOT_CONVERGED is
        returned, not raised, so that the caller can fall back to Lanczos"""
        lo = np.ascontiguousarray(eig_min, dtype=np.float64)
        hi = np.ascontiguousarray(eig_max, dtype=np.float64)
        reps = (ChebReport * (self.K * nrhs))()
        rc = lib().ggem_ensemble_brownian_dev(self.h, int(nrhs), int(N), _p(lo), _p(hi),
                                              float(tol), C.c_void_p(d_xi), C.c_void_p(d_dw),
                                              reps)
        if rc and rc != ERR_CHEB_NOT_CONVERGED:
            self._check(rc)
        return rc, [[reps[b * nrhs + r].as_dict() for r in range(nrhs)] for b in range(self.K)]

    def set_series_mode(self, persistent=True, slots_per_tile=0, wait_polls=0,
                        never_ready=False):
        """persistent: the whole Brownian step in one cooperative launch (the
        default) or one launch per term with host-side checks; slots per
        tile of the persistent launch (0 keeps the current); the polls of its
        bounded waits (0 = default); never_ready (test hook) makes every wait
        run out"""
        self._check(lib().ggem_ensemble_set_series_mode(self.h, 1 if persistent else 0,
                                                        int(slots_per_tile), int(wait_polls),
                                                        1 if never_ready else 0))

    def autotune_series(self, nrhs, N, eig_min, eig_max, d_xi, d_dw, cache_path=None):
        """(shape, slots per tile, ms per step) of the fastest form of the
        step: a persistent launch of shape 0, 1 or 2, or one launch per term
        (shape 3); the series mode follows the choice, and cache_path keeps
        it across runs"""
        lo = np.ascontiguousarray(eig_min, dtype=np.float64)
        hi = np.ascontiguousarray(eig_max, dtype=np.float64)
        sh, S, ms = C.c_int(), C.c_int(), C.c_double()
        self._check(lib().ggem_ensemble_autotune_series(
            self.h, int(nrhs), int(N), _p(lo), _p(hi), 0.0, C.c_void_p(d_xi), C.c_void_p(d_dw),
            cache_path.encode() if cache_path else None, C.byref(sh), C.byref(S), C.byref(ms)))
        return sh.value, S.value, ms.value

    def intervals(self, sur, chain_fraction=None, margin_lo=0.0, margin_hi=0.0):
        cf = np.zeros(self.K) if chain_fraction is None else \
            np.ascontiguousarray(chain_fraction, dtype=np.float64)
        lo, hi = np.zeros(self.K), np.zeros(self.K)
        self._check(lib().ggem_ensemble_intervals(self.h, sur.h, _p(cf), float(margin_lo),
                                                  float(margin_hi), _p(lo), _p(hi)))
        return lo, hi

    def lanczos(self, b, k=24, seed=7):
        lo, hi = C.c_double(), C.c_double()
        self._check(lib().ggem_ensemble_lanczos(self.h, int(b), int(k), int(seed), C.byref(lo),
                                                C.byref(hi)))
        return lo.value, hi.value

    def autotune(self, nrhs=8):
        t, ms = C.c_int(), C.c_double()
        self._check(lib().ggem_ensemble_autotune(self.h, int(nrhs), C.byref(t), C.byref(ms)))
        return t.value, ms.value


# ---- particle files (include/ggem_io.h) ----------------------------------
def _take_polymer(d: PolymerData) -> dict:
    n, m = d.n_beads, d.n_bonds

    def arr(ptr, count, shape=None):
        a = np.ctypeslib.as_array(ptr, shape=(count,)).copy()
        return a.reshape(shape) if shape else a
    out = {"n_beads": n, "n_bonds": m, "n_chains": d.n_chains,
           "n_bead_types": d.n_bead_types, "n_bond_types": d.n_bond_types,
           "xyz": arr(d.xyz, 3 * n, (n, 3)) if n else np.zeros((0, 3)),
           "chain_id": arr(d.chain_id, n) if n else np.zeros(0, np.int32),
           "bead_type": arr(d.bead_type, n) if n else np.zeros(0, np.int32),
           "bonds": arr(d.bonds, 2 * m, (m, 2)) if m else np.zeros((0, 2), np.int64),
           "bond_type": arr(d.bond_type, m) if m else np.zeros(0, np.int32)}
    if d.const_force and n:
        out["const_force"] = arr(d.const_force, 3 * n, (n, 3))
        out["charge"] = arr(d.charge, n)
        out["rot"] = arr(d.rot, 3 * n, (n, 3))
    if d.mass and d.n_bead_types:
        out["mass"] = arr(d.mass, d.n_bead_types)
    if d.has_box:
        out["box_lo"], out["box_hi"] = tuple(d.box_lo), tuple(d.box_hi)
    return out


def _read_polymer(fn, path) -> dict:
    d = PolymerData()
    rc = fn(str(path).encode(), C.byref(d))
    if rc:
        raise GGEMError(rc, f"cannot read {path}")
    try:
        return _take_polymer(d)
    finally:
        lib().ggem_free_polymer_data(C.byref(d))


def read_polymer_data(path) -> dict:
    """LAMMPS-style polymer data file (polymer_chain.C:61-226), 0-based ids"""
    return _read_polymer(lib().ggem_read_polymer_data, path)


def read_polymer_vtk(path) -> dict:
    """polymer VTK written by write_polymer_vtk (polymer_chain.C:396-494)"""
    return _read_polymer(lib().ggem_read_polymer_vtk, path)


def write_polymer_vtk(path, xyz, bonds, chain_id=None, precision=6):
    xyz = _f64(xyz).reshape(-1, 3)
    b = np.ascontiguousarray(bonds, dtype=np.int64).reshape(-1, 2)
    c = None if chain_id is None else np.ascontiguousarray(chain_id, dtype=np.int32)
    rc = lib().ggem_write_polymer_vtk(str(path).encode(), len(xyz), _p(xyz), len(b), _p(b),
                                      None if c is None else _p(c), int(precision))
    if rc:
        raise GGEMError(rc, f"cannot write {path}")


def write_bead_csv(path, xyz, vel=None, force=None, precision=6):
    xyz = _f64(xyz).reshape(-1, 3)
    v = None if vel is None else _f64(vel).reshape(-1, 3)
    f = None if force is None else _f64(force).reshape(-1, 3)
    rc = lib().ggem_write_bead_csv(str(path).encode(), len(xyz), _p(xyz),
                                   None if v is None else _p(v), None if f is None else _p(f),
                                   int(precision))
    if rc:
        raise GGEMError(rc, f"cannot write {path}")


def write_petsc_vec(path, v):
    v = _f64(v).reshape(-1)
    rc = lib().ggem_write_petsc_vec(str(path).encode(), len(v), _p(v))
    if rc:
        raise GGEMError(rc, f"cannot write {path}")


def read_petsc_vec(path) -> np.ndarray:
    n = C.c_int64()
    rc = lib().ggem_read_petsc_vec(str(path).encode(), -1, None, C.byref(n))
    if rc:
        raise GGEMError(rc, f"cannot read {path}")
    v = np.zeros(n.value)
    rc = lib().ggem_read_petsc_vec(str(path).encode(), n.value, _p(v), C.byref(n))
    if rc:
        raise GGEMError(rc, f"cannot read {path}")
    return v
