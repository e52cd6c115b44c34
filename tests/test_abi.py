"""CPU: the C-ABI library builds, loads, and exports every declared symbol.

No compute call is made here (there is no GPU in the CPU run); calls that
must fail without a device are checked to fail with a status, not a crash.
"""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from conftest import ROOT, gpu_available


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(cr_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("cr_egrad_h3", "cr_engine_create", "cr_engine_run", "cr_engine_step_host",
                 "cr_engine_get_state", "cr_engine_set_state"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = L.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_strings():
    lib = L.lib()
    assert lib.cr_error_string(0) == b"ok"
    assert lib.cr_error_string(L.CR_ERR_TRAJECTORY).startswith(b"trajectory")


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_calls_without_device_fail_cleanly():
    lib = L.lib()
    q = np.zeros((1, 3, 3))
    V = np.zeros(1)
    g = np.zeros_like(q)
    info = C.c_int(7)
    rc = lib.cr_egrad_h3(L.dptr(q), 3, 1, L.dptr(V), L.dptr(g), C.byref(info))
    assert rc == L.CR_ERR_NO_DEVICE
    assert info.value == 0


def test_argument_validation_precedes_device_use():
    lib = L.lib()
    q = np.zeros((1, 4, 3))
    V = np.zeros(1)
    info = C.c_int(0)
    assert lib.cr_egrad_h3(L.dptr(q), 4, 1, L.dptr(V), L.dptr(q), C.byref(info)) == L.CR_ERR_ARG
    mass = np.ones(3)
    cfg = L.CrConfig(L.CR_PES_H3, 3, 200, 1, 0, 70, 1, 0, 1, 0, 1.0, 1.0, 0.0, L.dptr(mass))
    h = C.c_void_p()
    assert lib.cr_engine_create(C.byref(cfg), C.byref(h)) == L.CR_ERR_ARG   # nbeads > 128
    cfg = L.CrConfig(L.CR_PES_H3, 3, 16, 1, 0, 70, 1, 0, 1, 0, 1.0, float("inf"), 0.0, L.dptr(mass))
    assert lib.cr_engine_create(C.byref(cfg), C.byref(h)) == L.CR_ERR_ARG   # NVE with P > 1
    cfg = L.CrConfig(99, 3, 16, 1, 0, 70, 1, 0, 1, 0, 1.0, 1.0, 0.0, L.dptr(mass))
    assert lib.cr_engine_create(C.byref(cfg), C.byref(h)) == L.CR_ERR_UNSUPPORTED


def test_evb_fit_argument_validation():
    lib = L.lib()
    x = np.zeros(4)
    e = np.zeros(3)
    f = np.zeros(3)
    assert lib.cr_evb_fit(9, L.dptr(x), 4, 3, L.dptr(e), L.dptr(e), L.dptr(e), L.dptr(f), None) == L.CR_ERR_ARG
    assert lib.cr_evb_fit(1, L.dptr(x), 4, 3, L.dptr(e), L.dptr(e), L.dptr(e), L.dptr(f), None) == L.CR_ERR_ARG
    assert lib.cr_evb_fit(4, L.dptr(x), 4, -1, L.dptr(e), L.dptr(e), L.dptr(e), L.dptr(f), None) == L.CR_ERR_ARG
    assert lib.cr_evb_fit(4, L.dptr(x), 4, 0, None, None, None, None, None) == 0


def test_batch_argument_validation():
    lib = L.lib()
    h = C.c_void_p()
    assert lib.cr_batch_create(None, 0, 10, C.byref(h)) == L.CR_ERR_ARG
    arr = (C.c_void_p * 1)(None)
    assert lib.cr_batch_create(arr, 1, 10, C.byref(h)) == L.CR_ERR_ARG
    assert lib.cr_batch_run(None, 1) == L.CR_ERR_ARG
    assert lib.cr_batch_destroy(None) == 0


def test_qmdff_file_counts(tmp_path):
    from caracal_gb300 import qmdff as Q
    ff = Q.water_dimer()
    Q.write_qmdff(ff, tmp_path / "w.qmdff")
    n = C.c_int()
    counts = np.zeros(5, dtype=np.int32)
    assert L.lib().cr_qmdff_file_counts(str(tmp_path / "w.qmdff").encode(), C.byref(n), L.iptr(counts)) == 0
    assert n.value == ff.n
    assert counts.tolist() == [len(ff.bond), len(ff.angl), len(ff.tors), len(ff.hb), len(ff.nci)]
    assert L.lib().cr_qmdff_file_counts(str(tmp_path / "missing.qmdff").encode(), C.byref(n),
                                        L.iptr(counts)) == L.CR_ERR_ARG
