"""ctypes binding of ``libcaracal_gb300.so`` (the C-ABI in include/caracal_gb300.h).

The library is the only compute path: if it cannot be built or loaded, every
call raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)

CR_OK = 0
CR_ERR_ARG = 1
CR_ERR_CUDA = 2
CR_ERR_NO_DEVICE = 3
CR_ERR_UNSUPPORTED = 4
CR_ERR_TRAJECTORY = 5
CR_ERR_IO = 6

CR_TRAJ_NONFINITE = 1
CR_TRAJ_SINGULAR_INERTIA = 2
CR_TRAJ_SHAKE_FAILED = 4

CR_PES_H3 = 1
CR_PES_CH4H = 2
CR_PES_CH4OH = 3
CR_PES_QMDFF = 4
CR_PES_EVB = 5
CR_PES_WATER = 6
CR_PES_OH3 = 7
CR_PES_GEH4OH = 8
CR_PES_BRH2 = 9

CR_THERMO_NONE = 0
CR_THERMO_ANDERSEN = 1
CR_THERMO_NHC = 2
CR_THERMO_PILE = 3

CR_PREC_FP64 = 0
CR_PREC_MIXED = 1


class CrConfig(C.Structure):
    _fields_ = [("pes", C.c_int), ("natoms", C.c_int), ("nbeads", C.c_int), ("ntraj", C.c_int),
                ("thermostat", C.c_int), ("andersen_step", C.c_int), ("transrot", C.c_int),
                ("precision", C.c_int), ("seed", C.c_uint), ("traj0", C.c_uint),
                ("dt", C.c_double), ("beta", C.c_double), ("pile_tau0", C.c_double),
                ("mass", c_double_p), ("nose_q", C.c_double), ("nm_mode", C.c_int)]


DUMP_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                      C.POINTER(C.c_double))


class CrQmdffTables(C.Structure):
    _fields_ = [(k, C.POINTER(C.c_double)) for k in ("rad", "r0ab", "zab", "r0094", "sr42", "c6ab")]


class CrD3Reference(C.Structure):
    _fields_ = [("c6ab", C.POINTER(C.c_double)), ("maxci", C.POINTER(C.c_int)), ("rcov", C.POINTER(C.c_double))]


class CrRecross(C.Structure):
    _fields_ = [("nreac1", C.c_int), ("reac1", C.c_int * 8), ("nreac2", C.c_int),
                ("reac2", C.c_int * 8), ("bond_form", C.c_int * 2), ("bond_break", C.c_int * 2),
                ("form_ref", C.c_double), ("break_ref", C.c_double), ("r_inf", C.c_double),
                ("xi_ideal", C.c_double)]


class CrQmdffDef(C.Structure):
    _fields_ = [("natoms", C.c_int), ("at", c_int_p), ("q", c_double_p), ("rad", c_double_p),
                ("nbond", C.c_int), ("nangl", C.c_int), ("ntors", C.c_int), ("nnci", C.c_int),
                ("bond", c_int_p), ("vbond", c_double_p), ("angl", c_int_p), ("vangl", c_double_p),
                ("tors", c_int_p), ("vtors", c_double_p), ("nci", c_int_p),
                ("r0ab", c_double_p), ("zab", c_double_p), ("r0094", c_double_p), ("sr42", c_double_p),
                ("c66ab", c_double_p), ("eps1", C.c_double * 6), ("eps2", C.c_double * 6),
                ("coul_cut", C.c_double), ("zahn", C.c_int), ("zahn_a", C.c_double),
                ("zahn_par", C.c_double), ("e_zero", C.c_double), ("nhb", C.c_int), ("hb", c_int_p),
                ("vhb", c_double_p)]


class CrEvbDef(C.Structure):
    _fields_ = [("basis", C.c_int)] + [(k, C.c_double) for k in "abcdefghmn"]


class CrWaterDef(C.Structure):
    _fields_ = [("nwater", C.c_int), ("periodic", C.c_int), ("box", C.c_double * 3), ("coul_cut", C.c_double),
                ("zahn", C.c_int), ("zahn_a", C.c_double), ("zahn_par", C.c_double)]


class CaracalError(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        detail = ""
        if _lib is not None:
            buf = C.create_string_buffer(512)
            _lib.cr_last_error_detail(buf, 512)
            detail = buf.value.decode(errors="replace")
            msg = _lib.cr_error_string(code).decode()
        else:
            msg = f"status {code}"
        super().__init__(f"{where}: {msg} ({detail})")


def _sig(lib):
    d, i, v = c_double_p, c_int_p, C.c_void_p
    eng = C.c_void_p
    sigs = {
        "cr_error_string": ([C.c_int], C.c_char_p),
        "cr_last_error_detail": ([C.c_char_p, C.c_int], C.c_int),
        "cr_device_count": ([i], C.c_int),
        "cr_egrad_h3": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_egrad_h3_device": ([v, C.c_int, v, v, C.c_int, v], C.c_int),
        "cr_egrad_ch4h": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_initialize_ch4h": ([], C.c_int),
        "cr_egrad_ch4oh": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_egrad_oh3": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_initialize_ch4oh": ([], C.c_int),
        "cr_egrad_geh4oh": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_initialize_geh4oh": ([], C.c_int),
        "cr_egrad_brh2": ([d, C.c_int, C.c_int, d, d, i], C.c_int),
        "cr_initialize_brh2": ([], C.c_int),
        "cr_egrad_device": ([C.c_int, v, C.c_int, v, v, C.c_int, v], C.c_int),
        "cr_engine_create": ([C.POINTER(CrConfig), C.POINTER(C.c_void_p)], C.c_int),
        "cr_engine_destroy": ([eng], C.c_int),
        "cr_engine_init_positions": ([eng, d, C.c_double], C.c_int),
        "cr_engine_init_momenta": ([eng, C.c_int], C.c_int),
        "cr_engine_compute_forces": ([eng], C.c_int),
        "cr_engine_set_state": ([eng, d, d, d], C.c_int),
        "cr_engine_get_state": ([eng, d, d, d, d, i], C.c_int),
        "cr_engine_run": ([eng, C.c_int], C.c_int),
        "cr_engine_run_dump": ([eng, C.c_int, C.c_int, DUMP_FN, v, d, d, d], C.c_int),
        "cr_engine_run_dump_async": ([eng, C.c_int, C.c_int, DUMP_FN, v], C.c_int),
        "cr_engine_step_host": ([eng, d, d, d, d], C.c_int),
        "cr_engine_last_kernel_ms": ([eng, C.POINTER(C.c_float)], C.c_int),
        "cr_engine_launch_info": ([eng, i, i, i, i], C.c_int),
        "cr_engine_device_state": ([eng, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p)], C.c_int),
        "cr_host_alloc": ([C.POINTER(C.c_void_p), C.c_ulonglong], C.c_int),
        "cr_host_free": ([v], C.c_int),
        "cr_host_register": ([v, C.c_ulonglong], C.c_int),
        "cr_host_unregister": ([v], C.c_int),
        "cr_calibrate_op": ([C.c_int, C.c_int, C.c_int, d], C.c_int),
        "cr_engine_set_recross": ([eng, C.POINTER(CrRecross), C.c_int], C.c_int),
        "cr_engine_init_children": ([eng, d], C.c_int),
        "cr_engine_kappa": ([eng, d, d, d, i], C.c_int),
        "cr_engine_set_parent": ([eng, C.POINTER(CrRecross)], C.c_int),
        "cr_qmdff_create": ([C.POINTER(CrQmdffDef), C.POINTER(C.c_void_p)], C.c_int),
        "cr_qmdff_set_periodic": ([v, d, C.c_double, C.c_double, d], C.c_int),
        "cr_qmdff_destroy": ([v], C.c_int),
        "cr_qmdff_egrad": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_qmdff_egrad_virial": ([v, d, C.c_int, d, d, d, d, C.c_int], C.c_int),
        "cr_qmdff_egrad_device": ([v, v, C.c_int, v, v, C.c_int, v], C.c_int),
        "cr_qmdff_schedule_info": ([v, i, i], C.c_int),
        "cr_qmdff_tuning": ([v, C.c_int, i, C.POINTER(C.c_float)], C.c_int),
        "cr_engine_create_qmdff": ([C.POINTER(CrConfig), v, C.POINTER(C.c_void_p)], C.c_int),
        "cr_evb_create": ([v, v, C.POINTER(CrEvbDef), C.POINTER(C.c_void_p)], C.c_int),
        "cr_evb_destroy": ([v], C.c_int),
        "cr_evb_egrad": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_engine_create_evb": ([C.POINTER(CrConfig), v, C.POINTER(C.c_void_p)], C.c_int),
        "cr_qmdff_nparams": ([v, i], C.c_int),
        "cr_qmdff_load": ([C.c_char_p, C.POINTER(CrQmdffTables), C.c_double, C.c_int, C.c_double,
                           C.POINTER(C.c_void_p)], C.c_int),
        "cr_qmdff_file_counts": ([C.c_char_p, i, i], C.c_int),
        "cr_qmdff_eg": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_qmdff_nonb": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_qmdff_hb": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_qmdff_load_d3": ([C.c_char_p, C.POINTER(CrQmdffTables), C.POINTER(CrD3Reference), C.c_double, C.c_int,
                              C.c_double, C.POINTER(C.c_void_p)], C.c_int),
        "cr_qmdff_hvp": ([v, d, d, C.c_int, d, d, d], C.c_int),
        "cr_qmdff_param_vjp": ([v, d, d, C.c_int, d], C.c_int),
        "cr_evb_fit": ([C.c_int, d, C.c_int, C.c_int, d, d, d, d, d], C.c_int),
        "cr_evb_fit_grad": ([C.c_int, d, C.c_int, C.c_int, d, d, d, d], C.c_int),
        "cr_evb_param_vjp": ([v, d, d, C.c_int, d, d], C.c_int),
        "cr_adjoint_create": ([v, C.c_int, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
        "cr_adjoint_forward": ([v], C.c_int),
        "cr_adjoint_backward": ([v, d, d, d, d, d], C.c_int),
        "cr_adjoint_destroy": ([v], C.c_int),
        "cr_engine_set_umbrella": ([eng, C.POINTER(CrRecross), d, d, C.c_int, C.c_double, C.c_double], C.c_int),
        "cr_engine_umbrella_sampling": ([eng, C.c_int], C.c_int),
        "cr_engine_umbrella_stats": ([eng, d, d, d, C.c_int], C.c_int),
        "cr_engine_mdinit": ([eng, C.c_uint], C.c_int),
        "cr_engine_set_andersen_step": ([eng, C.c_int], C.c_int),
        "cr_engine_set_launch": ([eng, C.c_int, C.c_int], C.c_int),
        "cr_engine_set_npt": ([eng, C.c_double, d], C.c_int),
        "cr_engine_get_npt": ([eng, d, d, d, C.c_int], C.c_int),
        "cr_engine_get_launch": ([eng, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
        "cr_engine_autotune": ([eng, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)],
                               C.c_int),
        "cr_batch_create": ([C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
        "cr_batch_run": ([v, C.c_int], C.c_int),
        "cr_batch_info": ([v, C.POINTER(C.c_longlong), i, C.POINTER(C.c_float)], C.c_int),
        "cr_batch_timeline": ([v, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
        "cr_batch_destroy": ([v], C.c_int),
        "cr_water_create": ([C.POINTER(CrWaterDef), C.POINTER(C.c_void_p)], C.c_int),
        "cr_water_destroy": ([v], C.c_int),
        "cr_water_natoms": ([v], C.c_int),
        "cr_water_egrad": ([v, d, C.c_int, d, d, C.c_int], C.c_int),
        "cr_engine_create_water": ([C.POINTER(CrConfig), v, C.POINTER(C.c_void_p)], C.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


def lib(build: bool = True):
    """Load (building first if stale) the CUDA engine library."""
    global _lib
    if _lib is None:
        path = _build.build() if build else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"caracal_gb300 native library missing: {path}")
        _lib = C.CDLL(path)
        _sig(_lib)
    return _lib


def check(code, where):
    if code != CR_OK:
        raise CaracalError(code, where)


def dptr(a):
    return a.ctypes.data_as(c_double_p)


def iptr(a):
    return a.ctypes.data_as(c_int_p)
