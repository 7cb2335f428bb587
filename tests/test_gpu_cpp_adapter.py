"""The C++ host adapter (cpp/ggem_copss.hpp) against the reference's golden
files, the way the reference's own integration test compares
output_velocity_profile_*_3P files (tests/integration_tests/src/compare.py,
cmp_df with max-abs tolerance)."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from ggem_gb300 import build as B

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def test_validation_driver_reproduces_golden_profiles(tmp_path):
    B.build()
    exe = B.OUT_DIR / "ggem_validation"
    g = json.loads((GOLD / "ggem_profile_3P.json").read_text())
    ns = [len(g["axes"][a]["coord"]) - 1 for a in "xyz"]
    args = [str(exe), str(g["alpha"]), str(g["box"][0]), str(g["box"][1]), *map(str, ns), "0",
            str(tmp_path)]
    for b in g["beads"]:
        args += [repr(v) for v in b] + [repr(v) for v in g["force"]]
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    tol = 0.5 * 10.0 ** (-g["print_decimals"]) + 1e-12
    for a in "xyz":
        out = np.loadtxt(tmp_path / f"output_velocity_profile_{a}_3P.csv", delimiter=",",
                         skiprows=1)
        A = g["axes"][a]
        assert np.allclose(out[:, 0], A["coord"], atol=1e-9)
        # the reference test's own criterion (max-abs 1e-5) and the print precision
        assert np.abs(out[:, 7:10] - np.array(A["local"])).max() <= tol
        assert np.abs(out[:, 10:13] - np.array(A["exact"])).max() <= tol
