"""Particle files in the reference's formats (host code, no GPU): the
reference's PointParticle_Polymer_BD_HI data file read by the library and
written back as VTK reproduces the reference's own output byte for byte."""
from pathlib import Path

import numpy as np
import pytest

import ggem_gb300 as G

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from ggem_gb300 import build as B
    B.build()


def test_read_reference_data_file():
    d = G.read_polymer_data(GOLD / "polymer_bd_hi_data.in")
    assert d["n_beads"] == 11 and d["n_bonds"] == 10 and d["n_chains"] == 1
    assert d["box_lo"][0] == pytest.approx(-129.872397092)
    assert d["box_hi"][2] == pytest.approx(12.9872397092)
    assert np.allclose(d["xyz"][0], [-100.493, 124.921, -9.297])
    assert np.allclose(d["xyz"][10], [-126.976, 80.933, 0.209])
    assert np.array_equal(d["bonds"], np.stack([np.arange(10), np.arange(1, 11)], 1))
    assert np.all(d["chain_id"] == 0) and np.all(d["bead_type"] == 0)
    assert d["mass"][0] == 1.0


def test_vtk_writer_matches_reference_output(tmp_path):
    d = G.read_polymer_data(GOLD / "polymer_bd_hi_data.in")
    out = tmp_path / "output_polymer_0.vtk"
    G.write_polymer_vtk(out, d["xyz"], d["bonds"], d["chain_id"], precision=6)
    assert out.read_bytes() == (GOLD / "polymer_bd_hi_output_0.vtk").read_bytes()


def test_vtk_round_trip_and_reference_vtk_read():
    d = G.read_polymer_vtk(GOLD / "polymer_bd_hi_output_0.vtk")
    ref = G.read_polymer_data(GOLD / "polymer_bd_hi_data.in")
    assert np.allclose(d["xyz"], ref["xyz"]) and np.array_equal(d["bonds"], ref["bonds"])
    assert d["n_chains"] == 1


def test_bead_csv_and_petsc_vectors(tmp_path):
    rng = np.random.default_rng(0)
    xyz = rng.normal(size=(5, 3))
    G.write_bead_csv(tmp_path / "b.csv", xyz, force=np.ones((5, 3)), precision=6)
    lines = (tmp_path / "b.csv").read_text().split("\n")
    assert lines[0].startswith("scalar x_coord")
    row = lines[1].split()
    assert row[0] == "0" and float(row[1]) == pytest.approx(xyz[0, 0], rel=1e-5)
    assert row[7:10] == ["1", "1", "1"]
    v = rng.normal(size=1234)
    G.write_petsc_vec(tmp_path / "vector_RIN.dat", v)
    raw = (tmp_path / "vector_RIN.dat").read_bytes()
    assert raw[:4] == (1211214).to_bytes(4, "big") and raw[4:8] == (1234).to_bytes(4, "big")
    assert np.frombuffer(raw[8:16], dtype=">f8")[0] == v[0]
    assert np.array_equal(G.read_petsc_vec(tmp_path / "vector_RIN.dat"), v)


def test_malformed_files_are_errors(tmp_path):
    bad = tmp_path / "bad.in"
    bad.write_text("header\n3 atoms\n2 bonds\n1 atom types\n1 bond types\n\nAtoms\n\n1 1 1 0 0 0\n")
    with pytest.raises(G.GGEMError):
        G.read_polymer_data(bad)
    with pytest.raises(G.GGEMError):
        G.read_petsc_vec(bad)
