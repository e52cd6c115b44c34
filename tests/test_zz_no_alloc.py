"""GPU: cr_egrad_h3_noalloc, the allocation-free H3 gradient, against cr_egrad_h3.

The allocation-free entry point exists for callers that cannot allocate
device memory (a per-step PES call that cannot pay cudaMalloc/cudaFree's
device-wide synchronisation, or a host whose device memory is a pre-sized
pool).  Both entry points are called through the C-ABI on the same
geometries, twice in a row with different sizes so that stale contents of
the shared device array would show; they must agree within the plain-form
tolerance used elsewhere (1e-12 norm-wise relative), and both must agree
with the oracle (the CPU restatement of egrad_h3) to the same tolerance.
This file is collected last so a failure here never hides another test's
result.
"""
import ctypes as C

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from caracal_gb300.workloads import h3_collinear
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MAX_BEADS = 16384


def _noalloc_fn():
    fn = L.lib().cr_egrad_h3_noalloc
    fn.argtypes = [L.c_double_p, C.c_int, C.c_int, L.c_double_p, L.c_double_p, C.POINTER(C.c_int)]
    fn.restype = C.c_int
    return fn


def _call(fn, q):
    nb = q.shape[0]
    V = np.full(nb, np.nan)
    g = np.full_like(q, np.nan)
    info = C.c_int(-1)
    rc = fn(L.dptr(q), 3, nb, L.dptr(V), L.dptr(g), C.byref(info))
    return rc, V, g, info.value


def test_noalloc_matches_allocating_entry_point_twice(require_gpu):
    noalloc = _noalloc_fn()
    alloc = L.lib().cr_egrad_h3
    for call, nb in enumerate((MAX_BEADS, 1000)):
        rng = np.random.default_rng(700 + call)
        q = np.ascontiguousarray(h3_collinear()[None] + rng.normal(0, 0.3, (nb, 3, 3)))
        rc_a, V_a, g_a, info_a = _call(alloc, q)
        rc_n, V_n, g_n, info_n = _call(noalloc, q)
        assert rc_a == 0 and rc_n == 0
        assert info_a == 0 and info_n == 0
        assert rel_err(V_n, V_a) <= 1e-12
        assert rel_err(g_n, g_a) <= 1e-12
        sub = slice(0, 256)                  # the oracle on a sample of the geometries
        V_o, g_o = orc.egrad_h3(q[sub])
        assert rel_err(V_n[sub], V_o) <= 1e-12
        assert rel_err(g_n[sub], g_o) <= 1e-12


def test_noalloc_rejects_more_than_the_fixed_maximum(require_gpu):
    q = np.zeros((MAX_BEADS + 1, 3, 3))
    rc, _, _, _ = _call(_noalloc_fn(), q)
    assert rc == L.CR_ERR_ARG
    buf = C.create_string_buffer(512)
    L.lib().cr_last_error_detail(buf, 512)
    assert b"fixed maximum" in buf.value
