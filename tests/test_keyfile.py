"""CPU: Caracal's keyword input (dynamic) and the list-directed output format."""
import numpy as np
import pytest

from caracal_gb300 import keyfile as K
from caracal_gb300.dynamic import fortran_int, fortran_real

KEY = """XYZSTART start.xyz
RPMD_BEADS 8
ENSEMBLE nvt
STEPS 40
DELTAT 0.1
TDUMP 0.5
PES ana_ch4h
E_CON
NVT {
  TEMP 300
  THERMOSTAT nose-hoover
  NOSE_DAMP 50
}
"""


def test_parse_dynamic_key():
    d = K.parse(KEY)
    assert (d.xyzstart, d.nbeads, d.ensemble, d.nstep) == ("start.xyz", 8, "NVT", 40)
    assert d.dt_fs == 0.1 and d.tdump_fs == 0.5 and d.iwrite == 5
    assert d.kelvin == 300.0 and d.thermostat == "nhc" and d.nose_damp == 50.0 and d.andersen_step == 70
    assert d.pes == "ANA_CH4H" and d.energycon and not d.unsupported


def test_defaults_and_nve():
    d = K.parse("XYZSTART a.xyz\nSTEPS 10\nPES ANA_H3\n")
    assert d.ensemble == "NVE" and d.nbeads == 1 and d.dt_fs == 1.0 and d.iwrite == 1
    assert d.thermostat == "none"


def test_fortran_nint_of_dump_interval():
    assert K.parse("STEPS 1\nDELTAT 0.4\nTDUMP 1.0\nPES ANA_H3\n").iwrite == 3   # nint(2.5) = 3
    assert K.parse("STEPS 1\nDELTAT 0.3\nTDUMP 1.0\nPES ANA_H3\n").iwrite == 3


@pytest.mark.parametrize("text,msg", [
    ("RPMD_BEADS 0\nSTEPS 1\nPES ANA_H3\n", "beads"),
    ("ENSEMBLE NVX\nSTEPS 1\nPES ANA_H3\n", "ensemble"),
    ("STEPS 0\nPES ANA_H3\n", "timesteps"),
    ("STEPS 1\nDELTAT 1e-7\nPES ANA_H3\n", "too small"),
    ("ENSEMBLE NVT\nSTEPS 1\nPES ANA_H3\nNVT {\n TEMP 300\n}\n", "THERMOSTAT"),
    ("ENSEMBLE NVT\nSTEPS 1\nPES ANA_H3\nNVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n", "delimiter"),
    ("ENSEMBLE NPT\nSTEPS 1\nPES ANA_H3\nNPT {\n TEMP 300\n THERMOSTAT ANDERSEN\n}\n", "periodic systems"),
    ("ENSEMBLE NPT\nSTEPS 1\nPES QMDFF\nPERIODIC 20 20 20\nQMDFF {\n FFNAMES a.qmdff\n}\n"
     "NPT {\n TEMP 300\n THERMOSTAT ANDERSEN\n BAROSTAT NOSE-HOOVER\n}\n", "BERENDSEN is"),
    ("ENSEMBLE NPT\nSTEPS 1\nPES QMDFF\nPERIODIC 20 20 20\nQMDFF {\n FFNAMES a.qmdff\n}\n"
     "NPT {\n TEMP 300\n PRES -1\n THERMOSTAT ANDERSEN\n}\n", "positive pressure"),
    ("STEPS 1\nPES ANA_O3\n", "not on this engine"),
    ("STEPS 1\nPES QMDFF\n", "QMDFFNAMES"),
])
def test_fatal_inputs(text, msg):
    with pytest.raises(K.KeyError_, match=msg):
        K.parse(text)


def test_qmdff_and_evb_blocks(tmp_path):
    text = ("STEPS 5\nPES de_evb\nQMDFF {\n FFNAMES a.qmdff b.qmdff\n ESHIFT -1.5 -1.4\n}\n"
            "DE_EVB {\n COUPLING sp\n}\nGPU_TRAJECTORIES 64\nSEED 9\nBOGUS 1\n")
    d = K.parse(text)
    assert d.ffnames == ["a.qmdff", "b.qmdff"] and d.eshift == [-1.5, -1.4] and d.coupling == "sp"
    assert d.ntraj == 64 and d.seed == 9 and d.unsupported == ["BOGUS"]
    (tmp_path / "evb_pars.dat").write_text("sp\n0.01\n50.0\n0.02\n30.0\n")
    assert K.read_evb_pars(str(tmp_path / "evb_pars.dat"), "sp") == dict(a=0.01, b=50.0, c=0.02, d=30.0)
    with pytest.raises(K.KeyError_):
        K.read_evb_pars(str(tmp_path / "evb_pars.dat"), "sp2d")


def test_list_directed_numbers_round_trip():
    for x in (1.0, -1.0, 0.5, 0.74, 12345.6789, 0.01, -3.2e-7, 1e20, 0.0, 2.0 / 3.0):
        s = fortran_real(x)
        assert len(s) == 26 and float(s) == x
    assert fortran_real(1.0) == "   1.0000000000000000     "
    assert fortran_real(0.01) == "   1.0000000000000000E-002"
    assert fortran_int(48) == "          48"


def test_read_vel_keyword_and_file(tmp_path):
    from caracal_gb300.dynamic import momenta_from_velocities
    key = "XYZSTART s.xyz\nRPMD_BEADS 2\nENSEMBLE NVT\nNVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n}\n" \
          "STEPS 10\nDELTAT 0.5\nTDUMP 1\nPES ana_h3\nREAD_VEL\n"
    d = K.parse(key)
    assert d.read_vel and not d.unsupported
    (tmp_path / "velocity_start.dat").write_text(
        " header\n\n 1 1  1.0d-4 -2.0E-4 3.0e-4\n 2 1 0.0 0.5d-3 0\n 3 1 1 2 3\n")
    v = K.read_velocities(str(tmp_path / "velocity_start.dat"), 3)
    assert np.allclose(v, [[1e-4, -2e-4, 3e-4], [0, 5e-4, 0], [1, 2, 3]])
    m = np.array([1.0, 2.0, 3.0])
    p = momenta_from_velocities(v, m, (4, 2, 3, 3))
    assert np.allclose(p[:, 0], -v * m[:, None]) and not p[:, 1].any()


def test_periodic_and_coulomb_keywords():
    """PERIODIC x y z (src/read_pes.f90:164-170) and the QMDFF block's
    COULOMB / COUL_CUTOFF / VDW_CUTOFF (src/read_pes.f90:1832-1863): only
    ZAHN switches the Coulomb treatment, PPPME stops the run."""
    d = K.parse("STEPS 5\nPES qmdff\nPERIODIC 27.0 27.0 30.5\nQMDFF {\n FFNAMES box.qmdff\n COULOMB zahn\n"
                " COUL_CUTOFF 9.0\n VDW_CUTOFF 8.0\n}\n")
    assert d.box == [27.0, 27.0, 30.5] and d.zahn and d.coul_cut == 9.0 and d.vdw_cut == 8.0
    assert not d.unsupported
    d = K.parse("STEPS 5\nPES qmdff\nQMDFF {\n FFNAMES a.qmdff\n}\n")
    assert d.box == [] and not d.zahn and d.coul_cut == 50.0 and d.vdw_cut == 10.0
    with pytest.raises(K.KeyError_, match="PERIODIC"):
        K.parse("STEPS 5\nPES qmdff\nPERIODIC 27.0\nQMDFF {\n FFNAMES a.qmdff\n}\n")
    d = K.parse("STEPS 5\nPES qmdff\nQMDFF {\n FFNAMES a.qmdff\n COULOMB ewald\n}\n")
    assert not d.zahn and not d.unsupported
    with pytest.raises(K.KeyError_, match="PPPME"):
        K.parse("STEPS 5\nPES qmdff\nQMDFF {\n FFNAMES a.qmdff\n COULOMB pppme\n}\n")
    with pytest.raises(K.KeyError_, match="QMDFF force fields"):
        K.parse("STEPS 5\nPES ana_h3\nPERIODIC 20 20 20\n")


@pytest.mark.parametrize("name,pes", [("ANA_H3", "h3"), ("ANA_CH4H", "ch4h"), ("ANA_CH4OH", "ch4oh"),
                                      ("ANA_OH3", "oh3"), ("ana_geh4oh", "geh4oh"), ("ANA_BRH2", "brh2")])
def test_analytic_surfaces(name, pes):
    """The analytic PES keywords built on this engine (src/read_pes.f90:413-631);
    the others stop with an error."""
    d = K.parse(f"STEPS 5\nPES {name}\n")
    assert K.ANALYTIC[d.pes] == pes
    with pytest.raises(K.KeyError_, match="not on this engine's path"):
        K.parse("STEPS 5\nPES ANA_O3\n")


def test_npt_block():
    """ENSEMBLE NPT with its block (src/dynamic.f90:478-580): temperature,
    pressure (atm), thermostat, Berendsen barostat (the default)."""
    d = K.parse("ENSEMBLE NPT\nSTEPS 10\nPES QMDFF\nPERIODIC 20 20 20\nQMDFF {\n FFNAMES a.qmdff\n}\n"
                "NPT {\n TEMP 300\n PRES 1.5\n THERMOSTAT ANDERSEN\n ANDERSEN_STEP 9\n}\n")
    assert d.ensemble == "NPT" and d.kelvin == 300.0 and d.pressure == 1.5 and d.barostat == "berendsen"
    assert d.thermostat == "andersen" and d.andersen_step == 9 and not d.unsupported
