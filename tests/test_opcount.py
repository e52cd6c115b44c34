"""CPU: the algorithmic operation table bench.py divides by equals the oracle's
op-counting instantiation of the reference formulas."""
import importlib.util
import os

import numpy as np

from caracal_gb300.workloads import ch4h_dividing_surface, ch4oh_geometry, h3_collinear
from conftest import ROOT
from oracle import oracle as orc


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algo_table_matches_oracle_counts():
    table = _bench().ALGO_PES_OPS
    from caracal_gb300.workloads import geh4oh_geometry, oh3_geometry
    for pes, q in (("h3", h3_collinear()), ("ch4h", ch4h_dividing_surface()), ("ch4oh", ch4oh_geometry()),
                   ("oh3", oh3_geometry()), ("geh4oh", geh4oh_geometry())):
        counted = {k: v for k, v in orc.pes_opcount(pes, q).items() if v and k != "cmp"}
        assert counted == table[pes], (pes, counted)


def test_qmdff_table_matches_oracle_counts():
    from caracal_gb300 import qmdff as Q
    ff = Q.alkane()
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    x = ff.xyz + np.random.default_rng(0).normal(0, 0.05, ff.xyz.shape)
    counted = {k: v for k, v in orc.pes_opcount("qmdff", x).items() if v and k != "cmp"}
    assert counted == _bench().ALGO_PES_OPS["qmdff"]


def test_water_table_matches_oracle_counts():
    from caracal_gb300 import water as Wt
    from caracal_gb300.workloads import water_config
    wl = water_config()
    x = wl.extra
    box, cut, za, zp = Wt.periodic_setup(x["box"], x["coul_cut"], x["zahn"])
    orc.set_water(x["nwater"], box, cut)
    q = wl.q0 + np.random.default_rng(0).normal(0, 0.05, wl.q0.shape)
    counted = {k: v for k, v in orc.pes_opcount("water", q).items() if v and k != "cmp"}
    assert counted == _bench().ALGO_PES_OPS["water"]


def test_algo_flops_positive_and_monotone_in_beads():
    b = _bench()
    w = {k: 20.0 for k in ("div", "sqrt", "exp", "pow", "log", "sin", "cos", "acos", "erf", "tanh",
                           "cosh")}
    f8 = sum(b.algo_flops_per_bead_step("h3", 3, 8, "pile", w))
    f64 = sum(b.algo_flops_per_bead_step("h3", 3, 64, "pile", w))
    assert 0 < f8 < f64
    assert np.isfinite(sum(b.algo_flops_per_bead_step("ch4h", 6, 32, "none", w, False, True)))
