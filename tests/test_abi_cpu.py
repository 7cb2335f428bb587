"""CPU checks of the C ABI: the library builds, loads and exports every
declared entry point, and its host-side parts agree with the oracle."""
import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

import ggem_gb300 as G
import oracle as O
from ggem_gb300 import build as B

ROOT = Path(__file__).resolve().parent.parent
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _built():
    B.build()
    O.build_oracle(with_ref=True)


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(ggem_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = G.lib()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_cheb_coeffs_bit_exact_vs_reference_goldens():
    d = json.loads((GOLD / "ref_chebyshev_coeffs.json").read_text())
    for cs in d["cases"]:
        got = G.cheb_coeffs(cs["N"], float.fromhex(cs["da"]), float.fromhex(cs["db"]), cs["method"])
        ref = np.array([float.fromhex(x) for x in cs["coef"]])
        assert np.array_equal(got, ref), (cs["N"], cs["method"])


def test_cheb_coeffs_rejects_bad_arguments():
    c = np.zeros(4)
    assert G.lib().ggem_cheb_coeffs(0, 1.0, 0.0, 0, c.ctypes.data) == G.ERR_BAD_ARG
    assert G.lib().ggem_cheb_coeffs(3, -1.0, 0.0, 0, c.ctypes.data) == G.ERR_BAD_ARG
    assert G.lib().ggem_cheb_coeffs(3, 1.0, 0.0, 7, c.ctypes.data) == G.ERR_BAD_ARG


def test_std_random_vector_matches_reference_stream():
    for seed, skip in ((123456789, 0), (42, 3)):
        a = G.std_random_vector(seed, 999, 0.0, 1.0, skip)
        b = O.std_normal_vector(seed, 999, 0.0, 1.0, skip)
        assert np.array_equal(a, b)


def test_workload_generators_are_seeded_and_non_overlapping():
    xyz, L = G.make_suspension(5, 2000, 0.1)
    xyz2, _ = G.make_suspension(5, 2000, 0.1)
    assert np.array_equal(xyz, xyz2)
    assert L == pytest.approx((2000 * 4 / 3 * np.pi / 0.1) ** (1 / 3))
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    nb = O.neighbors_cutoff(box, xyz, 2.0)
    assert nb.offsets[-1] == 0  # nobody closer than 2a
    ch, Lc = G.make_chains(3, 50, 20, 2.0, 0.05)
    d = ch.reshape(50, 20, 3)
    b = np.diff(d, axis=1)
    b -= Lc * np.round(b / Lc)
    assert np.allclose(np.linalg.norm(b, axis=2), 2.0, atol=1e-9)
    nbc = O.neighbors_cutoff(O.make_box([0] * 3, [Lc] * 3, [1, 1, 1]), ch, 2.0 - 1e-9)
    assert nbc.offsets[-1] == 0


def test_create_without_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = G.default_params()
    h = C.c_void_p()
    assert G.lib().ggem_create(C.byref(p), C.byref(h)) == G.ERR_NO_DEVICE
    assert G.lib().ggem_strerror(G.ERR_NO_DEVICE) == b"no CUDA device"
