"""Output formats of the frame writer (biospring_gb300/trajectory.py): PDB models and the energy
table laid out like the reference's CSV sampling (src/IO/CSVSampleWriter.cpp)."""

import numpy as np

from biospring_gb300 import trajectory as T


def test_pdb_model_columns():
    xyz = np.array([[1.0, -2.5, 3.25], [-123.456, 0.0, 9999.999]], np.float32)
    text = T.pdb_model(7, xyz, names=["CA", "OXT1"], resnames=["ALA", "GLY"], resids=[1, 12], chains=["B", "B"])
    lines = text.splitlines()
    assert lines[0] == "MODEL        7" and lines[-1] == "ENDMDL"
    a = lines[1]
    assert a[0:6] == "ATOM  " and int(a[6:11]) == 1 and a[12:16] == " CA " and a[17:20] == "ALA"
    assert a[21] == "B" and int(a[22:26]) == 1
    assert float(a[30:38]) == 1.0 and float(a[38:46]) == -2.5 and float(a[46:54]) == 3.25
    b = lines[2]
    assert b[12:16] == "OXT1" and int(b[22:26]) == 12
    assert abs(float(b[30:38]) - (-123.456)) < 1e-3 and abs(float(b[46:54]) - 9999.999) < 1e-3


def test_energy_table_layout():
    terms = T.enabled_terms(dict(spring_enable=1, steric_enable=1, coulomb_enable=0, impala_enable=1))
    assert terms == ["kinetic", "spring", "steric", "imp"]
    head = T.energy_header(terms)
    assert head.startswith("# Step\tFrameRate(Hz)\tKinetic energy (kJ.mol-1)\tSpring energy (kJ.mol-1)")
    row = T.energy_row(40, 12.5, [1.0, 2.0, 3.0, 4.0, 5.0, 6.0], terms).rstrip("\n").split("\t")
    assert row == ["40", "12.5", "1.0", "2.0", "3.0", "5.0"]
