"""GPU: `python -m caracal_gb300.dynamic` on Caracal key files (H3, QMDFF,
dE-EVB): the output files Caracal writes, and the written frames equal the
engine's own state after the same steps."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300 import qmdff as Q
from caracal_gb300.dynamic import run
from caracal_gb300.units import BOHR_ANGSTROM, angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au
from caracal_gb300.workloads import h3_collinear

pytestmark = pytest.mark.gpu


def frames(path):
    lines = open(path).read().splitlines()
    out, i = [], 0
    while i < len(lines):
        n = int(lines[i])
        out.append(np.array([[float(v) for v in ln.split()[1:4]] for ln in lines[i + 2:i + 2 + n]]))
        i += 2 + n
    return out


def test_dynamic_h3_nvt(require_gpu, tmp_path):
    xyz = h3_collinear() * BOHR_ANGSTROM
    (tmp_path / "start.xyz").write_text("3\n\n" + "".join(f"H {a} {b} {c}\n" for a, b, c in xyz))
    (tmp_path / "dynamic.key").write_text(
        "XYZSTART start.xyz\nRPMD_BEADS 4\nENSEMBLE NVT\nSTEPS 20\nDELTAT 0.1\nTDUMP 0.5\nPES ANA_H3\n"
        "E_CON\nSEED 3\nNVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n ANDERSEN_STEP 7\n}\n")
    run(str(tmp_path / "dynamic.key"), out_dir=str(tmp_path), quiet=True)
    tr = frames(tmp_path / "trajectory.xyz")
    ce = frames(tmp_path / "traj_centroid.xyz")
    en = [ln for ln in open(tmp_path / "md_energies.dat").read().splitlines()[1:]]
    assert len(tr) == 4 and all(f.shape == (12, 3) for f in tr)
    assert len(ce) == 4 and len(en) == 4
    assert [int(r.split()[0]) for r in en] == [5, 10, 15, 20]
    mass = [mass_au("H")] * 3
    eng = RPMDEngine("h3", mass, 4, 1, dt_fs_to_au(0.1), beta=beta_from_kelvin(300.0), thermostat="andersen",
                     andersen_step=7, transrot=True, seed=3)
    eng.init_positions(angstrom_to_bohr(xyz), 0.0)
    eng.init_momenta()
    eng.compute_forces()
    eng.run(20)
    q, _, _, e, _ = eng.get_state()
    assert np.allclose(tr[-1], q[0].reshape(-1, 3) * BOHR_ANGSTROM, rtol=1e-15, atol=1e-15)
    assert np.allclose(ce[-1], q[0].mean(axis=0) * BOHR_ANGSTROM, rtol=1e-15, atol=1e-15)
    assert float(en[-1].split()[1]) == pytest.approx(e[0] / 4, rel=1e-15)


def test_dynamic_qmdff_and_evb(require_gpu, tmp_path):
    ff = Q.alkane(nc=3)
    ff2 = Q.alkane_evb_partner(ff)
    Q.write_qmdff(ff, tmp_path / "a.qmdff")
    Q.write_qmdff(ff2, tmp_path / "b.qmdff")
    sym = ["C" if z == 6 else "H" for z in ff.at]
    (tmp_path / "start.xyz").write_text(f"{ff.n}\n\n" + "".join(
        f"{s} {a} {b} {c}\n" for s, (a, b, c) in zip(sym, ff.xyz * BOHR_ANGSTROM)))
    base = "XYZSTART start.xyz\nRPMD_BEADS 2\nENSEMBLE NVT\nSTEPS 6\nDELTAT 0.5\nTDUMP 1.0\nE_CON\n" \
           "NVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n}\n"
    (tmp_path / "q.key").write_text(base + "PES QMDFF\nQMDFF {\n FFNAMES a.qmdff\n ESHIFT -0.25\n}\n")
    run(str(tmp_path / "q.key"), out_dir=str(tmp_path), quiet=True)
    en = [ln.split() for ln in open(tmp_path / "md_energies.dat").read().splitlines()[1:]]
    assert len(en) == 3 and all(np.isfinite(float(v)) for r in en for v in r)
    assert float(en[0][1]) < -0.2        # E_zero from ESHIFT is in the energy
    (tmp_path / "evb_pars.dat").write_text("1g\n0.01\n50.0\n")
    (tmp_path / "e.key").write_text(base + "PES DE_EVB\nQMDFF {\n FFNAMES a.qmdff b.qmdff\n ESHIFT 0.0 0.02\n}\n"
                                    "DE_EVB {\n COUPLING 1g\n}\n")
    run(str(tmp_path / "e.key"), out_dir=str(tmp_path), quiet=True)
    assert len(frames(tmp_path / "trajectory.xyz")) == 3


def test_run_dump_callback(require_gpu):
    mass = [mass_au("H")] * 3
    kw = dict(beta=beta_from_kelvin(300.0), thermostat="andersen", andersen_step=7, seed=4)
    a = RPMDEngine("h3", mass, 4, 2, dt_fs_to_au(0.1), **kw)
    b = RPMDEngine("h3", mass, 4, 2, dt_fs_to_au(0.1), **kw)
    for e in (a, b):
        e.init_positions(h3_collinear(), 0.01)
        e.init_momenta()
        e.compute_forces()
    seen = []

    def cb(istep, q, p, epot):
        b.run(5)
        qb, pb, _, eb, _ = b.get_state()
        seen.append((istep, np.array_equal(q, qb) and np.array_equal(p, pb) and np.array_equal(epot, eb)))
        return istep >= 15          # stop after the third dump

    with pytest.raises(Exception):
        a.run_dump(40, 5, cb)
    assert seen == [(5, True), (10, True), (15, True)]


@pytest.mark.parametrize("kind", ["h3", "qmdff"])
def test_run_dump_async_frames_match_run_dump(require_gpu, kind):
    """cr_engine_run_dump_async hands over the same frames at the same steps
    as the synchronous cr_engine_run_dump and leaves the same final state,
    on the persistent kernel (H3, 4 beads) and on the graph path of a force
    field (QMDFF alkane, 8 beads)."""
    from caracal_gb300.engine import QMDFFForceField
    kw = dict(beta=beta_from_kelvin(300.0), thermostat="andersen", andersen_step=7, seed=11)
    if kind == "h3":
        mass, nb, q0, ffs = [mass_au("H")] * 3, 4, h3_collinear(), [None, None]
    else:
        ff = Q.alkane()
        mass, nb, q0 = [mass_au(Q.SYMBOLS[z - 1]) for z in ff.at], 8, ff.xyz
        ffs = [QMDFFForceField(ff), QMDFFForceField(ff)]
    engines = [RPMDEngine(f or "h3", mass, nb, 8, dt_fs_to_au(0.1), **kw) for f in ffs]
    for e in engines:
        e.init_positions(q0, 0.01)
        e.init_momenta()
        e.compute_forces()
    frames = ([], [])
    engines[0].run_dump(23, 4, lambda i, q, p, ep: frames[0].append((i, q.copy(), p.copy(), ep.copy())))
    engines[1].run_dump_async(23, 4, lambda i, q, p, ep: frames[1].append((i, q.copy(), p.copy(), ep.copy())))
    assert [f[0] for f in frames[0]] == [4, 8, 12, 16, 20] == [f[0] for f in frames[1]]
    for a, b in zip(*frames):
        assert all(np.array_equal(x, y) for x, y in zip(a[1:], b[1:]))
    sa, sb = engines[0].get_state(), engines[1].get_state()
    assert all(np.array_equal(x, y) for x, y in zip(sa, sb))
    # a truthy return stops the run with an error after that frame
    seen = []
    with pytest.raises(Exception):
        engines[1].run_dump_async(20, 2, lambda i, *_: seen.append(i) or len(seen) == 2)
    assert len(seen) == 2
    for e in engines:
        e.close()
    for f in ffs:
        if f is not None:
            f.close()


def test_dynamic_periodic_qmdff(require_gpu, tmp_path):
    """PERIODIC with a QMDFF key file: the dumped energies are the periodic
    force field's at the dumped frames (set_periodic with the key file's
    cutoffs: a 6 A dispersion cutoff removes pairs of the 11-carbon chain),
    not the free molecule's."""
    from caracal_gb300.engine import QMDFFForceField
    ff = Q.alkane(nc=11)
    Q.write_qmdff(ff, tmp_path / "a.qmdff")
    sym = ["C" if z == 6 else "H" for z in ff.at]
    (tmp_path / "start.xyz").write_text(f"{ff.n}\n\n" + "".join(
        f"{s} {a} {b} {c}\n" for s, (a, b, c) in zip(sym, ff.xyz * BOHR_ANGSTROM)))
    key = ("XYZSTART start.xyz\nRPMD_BEADS 1\nENSEMBLE NVT\nSTEPS 2\nDELTAT 0.5\nTDUMP 0.5\nE_CON\n"
           "NVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n}\nPES QMDFF\nPERIODIC 40.0 40.0 40.0\n"
           "QMDFF {\n FFNAMES a.qmdff\n VDW_CUTOFF 6.0\n}\n")
    (tmp_path / "p.key").write_text(key)
    run(str(tmp_path / "p.key"), out_dir=str(tmp_path), quiet=True)
    en = [ln.split() for ln in open(tmp_path / "md_energies.dat").read().splitlines()[1:]]
    tr = frames(tmp_path / "trajectory.xyz")
    assert len(en) == 2 and len(tr) == 2
    free = QMDFFForceField(Q.read_qmdff(str(tmp_path / "a.qmdff")))
    per = QMDFFForceField(Q.read_qmdff(str(tmp_path / "a.qmdff")))
    per.set_periodic([40.0] * 3, 50.0, 6.0)
    x = np.stack([angstrom_to_bohr(f) for f in tr])
    ef, _ = free.egrad(x, "fp64")
    ep, _ = per.egrad(x, "fp64")
    free.close()
    per.close()
    e_dump = np.array([float(r[1]) for r in en])
    # the frames are written with 17 digits: the energies agree to ~1e-12
    assert np.abs(e_dump - ep).max() < 1e-9 * max(1.0, np.abs(ep).max())
    assert np.abs(ep - ef).min() > 1e-6          # the cutoff acts on this chain


def test_dynamic_npt_berendsen(require_gpu, tmp_path, capsys):
    """ENSEMBLE NPT with the Berendsen barostat: the frames carry each dump's
    box (Angstrom) on the comment line, equal to the engine's NpT state after
    the same steps, and stdout has the NpT columns."""
    from caracal_gb300.engine import QMDFFForceField
    ff = Q.alkane(nc=4)
    Q.write_qmdff(ff, tmp_path / "a.qmdff")
    sym = ["C" if z == 6 else "H" for z in ff.at]
    (tmp_path / "start.xyz").write_text(f"{ff.n}\n\n" + "".join(
        f"{s} {a} {b} {c}\n" for s, (a, b, c) in zip(sym, ff.xyz * BOHR_ANGSTROM)))
    key = ("XYZSTART start.xyz\nRPMD_BEADS 2\nENSEMBLE NPT\nSTEPS 20\nDELTAT 0.5\nTDUMP 2.5\nE_CON\nSEED 4\n"
           "NPT {\n TEMP 300\n PRES 100.0\n THERMOSTAT ANDERSEN\n ANDERSEN_STEP 7\n}\nPES QMDFF\n"
           "PERIODIC 16.0 16.0 16.0\nQMDFF {\n FFNAMES a.qmdff\n}\n")
    (tmp_path / "p.key").write_text(key)
    run(str(tmp_path / "p.key"), out_dir=str(tmp_path), quiet=False)
    out = capsys.readouterr().out.splitlines()
    assert len(out) == 4 and all(len(ln.split()) == 6 for ln in out)
    lines = open(tmp_path / "trajectory.xyz").read().splitlines()
    n = 2 * ff.n
    boxes = [np.array([float(v) for v in lines[k * (n + 2) + 1].split()]) for k in range(4)]
    assert all(b.shape == (3,) for b in boxes) and not np.allclose(boxes[0], boxes[-1])
    # the same run through the engine
    gff = QMDFFForceField(Q.read_qmdff(str(tmp_path / "a.qmdff")))
    gff.set_periodic([16.0] * 3, 50.0, 10.0)
    mass = [mass_au(s) for s in sym]
    eng = RPMDEngine(gff, mass, 2, 1, dt_fs_to_au(0.5), beta=beta_from_kelvin(300.0), thermostat="andersen",
                     andersen_step=7, transrot=True, seed=4)
    eng.set_npt(100.0)
    eng.init_positions(ff.xyz, 0.0)
    eng.init_momenta()
    eng.compute_forces()
    eng.run(20)
    box, _, _ = eng.npt_state()
    q, _, _, _, _ = eng.get_state()
    eng.close()
    gff.close()
    assert np.allclose(boxes[-1], box[0] * BOHR_ANGSTROM, rtol=1e-15, atol=0)
    tr = frames(tmp_path / "trajectory.xyz")
    assert np.allclose(tr[-1], q[0].reshape(-1, 3) * BOHR_ANGSTROM, rtol=1e-15, atol=1e-15)
    vol = float(out[-1].split()[3])
    assert abs(vol - np.prod(box[0]) * BOHR_ANGSTROM ** 3) < 1e-3


@pytest.mark.parametrize("pes,sym,xyz_ang", [
    ("ANA_BRH2", ["H", "Br", "H"], [[0.0, 0.0, -1.9], [0.0, 0.0, 1.4145], [0.0, 0.1, 0.0]]),
    ("ANA_GEH4OH", None, None),
])
def test_dynamic_new_surfaces(require_gpu, tmp_path, pes, sym, xyz_ang):
    """PES ANA_BRH2 / ANA_GEH4OH from a key file: the last frame equals the
    engine's state after the same steps (element masses Br 78.918, Ge 72.61)."""
    from caracal_gb300.keyfile import ANALYTIC
    if sym is None:
        from caracal_gb300.workloads import geh4oh_geometry
        sym = ["H", "Ge", "H", "H", "H", "O", "H"]
        xyz_ang = geh4oh_geometry() * BOHR_ANGSTROM
    xyz_ang = np.asarray(xyz_ang, dtype=np.float64)
    (tmp_path / "start.xyz").write_text(f"{len(sym)}\n\n" + "".join(
        f"{s} {a} {b} {c}\n" for s, (a, b, c) in zip(sym, xyz_ang)))
    (tmp_path / "d.key").write_text(
        f"XYZSTART start.xyz\nRPMD_BEADS 4\nENSEMBLE NVT\nSTEPS 10\nDELTAT 0.1\nTDUMP 0.5\nPES {pes}\n"
        "SEED 2\nNVT {\n TEMP 300\n THERMOSTAT ANDERSEN\n ANDERSEN_STEP 3\n}\n")
    run(str(tmp_path / "d.key"), out_dir=str(tmp_path), quiet=True)
    tr = frames(tmp_path / "trajectory.xyz")
    mass = [mass_au(s) for s in sym]
    eng = RPMDEngine(ANALYTIC[pes], mass, 4, 1, dt_fs_to_au(0.1), beta=beta_from_kelvin(300.0),
                     thermostat="andersen", andersen_step=3, transrot=True, seed=2)
    eng.init_positions(angstrom_to_bohr(xyz_ang), 0.0)
    eng.init_momenta()
    eng.compute_forces()
    eng.run(10)
    q, _, _, _, st = eng.get_state()
    eng.close()
    assert len(tr) == 2 and not st.any()
    assert np.allclose(tr[-1], q[0].reshape(-1, 3) * BOHR_ANGSTROM, rtol=1e-15, atol=1e-15)
