"""ctypes mirror of the C ABI in include/molsim_gb300.h.

The structure layouts and function signatures here must match the header
exactly; tests/test_abi.py checks that every declared symbol is exported.
"""
import ctypes as C
import os

import numpy as np

MG_ABI_VERSION = 2

MG_OK = 0
STATUS = {
    0: "MG_OK", -1: "MG_ERR_ARG", -2: "MG_ERR_CUDA", -3: "MG_ERR_TABLE_UNDERRUN",
    -4: "MG_ERR_NEIGH_OVERFLOW", -5: "MG_ERR_NAN", -6: "MG_ERR_TIMEOUT", -7: "MG_ERR_IBUF",
    -8: "MG_ERR_TABLE", -9: "MG_ERR_STATE", -10: "MG_ERR_ALLOC", -11: "MG_ERR_UNSUPPORTED",
    -12: "MG_ERR_CELL",
}
MG_EWALD_NONE, MG_EWALD_STD, MG_EWALD_SPM = 0, 1, 2
MG_VLIST, MG_CELLLIST = 0, 1
MG_MD, MG_MC, MG_BD = 0, 1, 2
MG_FP64, MG_MIXED = 0, 1

PI32 = C.POINTER(C.c_int32)
PF64 = C.POINTER(C.c_double)


class MgParams(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("np", C.c_int32), ("npt", C.c_int32), ("nptpt", C.c_int32),
        ("iptpn", PI32), ("iptpt", PI32), ("az", PF64),
        ("nbuf", C.c_int32), ("ubuf", PF64), ("iubuflow", PI32), ("r2umin", PF64), ("r2atat", PF64),
        ("boxlen", C.c_double * 3), ("rcut", C.c_double), ("drnlist", C.c_double),
        ("txintlist", C.c_int32), ("mode", C.c_int32), ("form", C.c_int32), ("maxnneigh", C.c_int32),
        ("ewald", C.c_int32), ("ualpha", C.c_double), ("ncut", C.c_int32),
        ("ncutregion_cube", C.c_int32), ("order", C.c_int32), ("nmesh", C.c_int32),
        ("lsurf", C.c_int32), ("epsi_four_pi", C.c_double), ("force_fac", C.c_double),
        ("nbond", C.c_int32), ("bond_ip", PI32), ("bond_jp", PI32), ("bond_k", PF64),
        ("bond_eq", PF64), ("bond_p", PI32),
        ("nangle", C.c_int32), ("angle_jm", PI32), ("angle_ip", PI32), ("angle_jp", PI32),
        ("angle_k", PF64), ("angle_eq", PF64), ("angle_p", PI32),
    ]


class MgPotParams(C.Structure):
    _fields_ = [
        ("npt", C.c_int32), ("iptpt", PI32), ("zat", PF64), ("sigat", PF64), ("epsat", PF64),
        ("rcut", C.c_double), ("ualpha", C.c_double), ("epsi_four_pi", C.c_double),
        ("lcharge_ewald", C.c_int32), ("lljcut", C.c_int32), ("ljrcut", C.c_double),
        ("ljushift", C.c_double), ("r2uminin", C.c_double), ("utoltab", C.c_double),
        ("ftoltab", C.c_double), ("umaxtab", C.c_double), ("fmaxtab", C.c_double),
    ]


class MgPolyParams(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("np", C.c_int32), ("npt", C.c_int32), ("nptpt", C.c_int32),
        ("iptpn", PI32), ("iptpt", PI32), ("napt", PI32), ("na", C.c_int32), ("ianpn", PI32),
        ("iatan", PI32), ("nat", C.c_int32), ("natat", C.c_int32), ("iatat", PI32),
        ("nbuf", C.c_int32), ("ubuf", PF64), ("iubuflow", PI32), ("r2umin", PF64), ("r2atat", PF64),
        ("boxlen", C.c_double * 3), ("rcut", C.c_double), ("lmc", C.c_int32),
        ("aza", PF64), ("ualpha", C.c_double), ("epsi_four_pi", C.c_double),
    ]


# (name without prefix, restype, argtypes) shared by the library (mg_) and the
# oracle (orc_), whose entry points take the same arguments.
H = C.c_void_p
SIGNATURES = [
    ("create", C.c_int, [C.POINTER(MgParams), C.POINTER(C.c_void_p)]),
    ("set_positions", C.c_int, [H, PF64]),
    ("get_positions", C.c_int, [H, PF64]),
    ("nlist_set", C.c_int, [H]),
    ("nlist_update", C.c_int, [H, PF64, PI32]),
    ("nlist_get", C.c_int, [H, PI32, PI32, C.c_int32]),
    ("celllist_get", C.c_int, [H, PI32, PI32]),
    ("utotal", C.c_int, [H, PF64, PF64, PF64]),
    ("energy_terms", C.c_int, [H, PF64]),
    ("dutotal", C.c_int, [H, C.c_int32, PI32, PF64, PF64, PF64, PF64, PI32]),
    ("accept", C.c_int, [H]),
    ("md_setup", C.c_int, [H, C.c_double, PF64, PF64, PF64]),
    ("md_run", C.c_int, [H, C.c_int32, PF64, PF64, PF64, PF64]),
    ("bd_setup", C.c_int, [H, PF64, PF64, C.c_int32]),
    ("bd_run", C.c_int, [H, C.c_int32, PF64, PF64]),
    ("bd_get_seed", C.c_int, [H, PI32]),
    ("pot_twobody_tab", C.c_int, [C.POINTER(MgPotParams), PF64, C.c_int32, PI32, PI32, PF64, PI32]),
    ("rcut_to_alpha", C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, PF64]),
]

LIB_ONLY = [
    ("abi_version", C.c_int, []),
    ("status_string", C.c_char_p, [C.c_int]),
    ("last_error", C.c_int, [H, C.c_char_p, C.c_size_t]),
    ("destroy", C.c_int, [H]),
    ("dutotal_batch", C.c_int, [H, C.c_int32, PI32, PF64, PF64, PI32]),
    ("nlist_calls", C.c_int, [H, PI32]),
    ("fft_check", C.c_int, [H, PF64, PF64, PF64, PF64, PF64]),
    ("dipole_ewald", C.c_int, [H, PF64, PF64, PF64, PF64, PF64]),
    ("bd_step_host", C.c_int, [H, PF64, PF64, PF64]),
    ("phase_times", C.c_int, [H, PF64, C.c_int32, PI32, C.c_char_p, C.c_size_t]),
    ("phase_reset", C.c_int, [H, C.c_int32]),
    ("bench_steps", C.c_int, [H, C.c_int32, C.c_int32, C.c_int64, PF64]),
    ("step_kernels", C.c_int, [H, C.c_int32, PI32]),
    ("grad", C.c_int, [H, C.POINTER(MgPotParams), PF64, PF64, PF64, PF64]),
    ("virial_tensor", C.c_int, [H, PF64]),
    ("force_jvp", C.c_int, [H, PF64, PF64]),
    ("force_pvjp", C.c_int, [H, C.POINTER(MgPotParams), PF64, PF64, PF64, PF64]),
    ("ensemble_create", C.c_int, [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    ("ensemble_run", C.c_int, [H, C.c_int32, C.c_int32, PF64]),
    ("ensemble_kernels", C.c_int, [H, C.c_int32, PI32]),
    ("ensemble_last_error", C.c_int, [H, C.c_char_p, C.c_size_t]),
    ("ensemble_destroy", C.c_int, [H]),
    ("poly_create", C.c_int, [C.POINTER(MgPolyParams), C.c_int32, C.POINTER(C.c_void_p)]),
    ("poly_utwobody", C.c_int, [H, PF64, PF64, PI32, PI32, PF64, PF64, PF64]),
    ("poly_ewald_intra", C.c_int, [H, PF64, PF64, PF64]),
    ("poly_utwobody_list", C.c_int, [H, H, PF64, PF64, PF64, PF64]),
    ("poly_epilogue", C.c_int, [H, PF64, PF64, PF64, PF64, C.c_double, PF64, PF64, PF64]),
    ("poly_udipole_real", C.c_int, [H, PF64, PF64, PF64, PI32, PI32, PF64, PF64, PF64, PF64, PF64]),
    ("poly_udipole_self", C.c_int, [H, PF64, PF64, C.c_int32, PF64, PF64, PF64, PF64]),
    ("poly_udipole_finish", C.c_int, [H, PF64, PF64, PF64, PF64, PF64, PF64, PF64]),
    ("poly_dutwobody_batch", C.c_int, [H, PF64, PF64, PI32, PI32, C.c_int32, PI32, PF64, PF64, PF64, PI32]),
    ("poly_dutwobody_multi", C.c_int, [H, PF64, PF64, PI32, PI32, C.c_int32, PI32, PF64, PF64, PF64, PI32]),
    ("poly_rigid_setup", C.c_int, [H, C.c_double, C.c_double, C.c_int32, PF64, PF64, PF64, PF64, PF64, PF64,
                                   PF64, PF64]),
    ("poly_rigid_move", C.c_int, [H, PF64, PF64, PF64]),
    ("poly_rigid_kick", C.c_int, [H, PF64, PF64, PF64, PF64]),
    ("poly_rigid_prime", C.c_int, [H, PF64, PF64]),
    ("poly_rigid_get", C.c_int, [H, PF64, PF64]),
    ("poly_md_run", C.c_int, [H, H, H, PF64, C.c_int32, PF64, PF64, PF64, PF64, PF64]),
    ("poly_last_error", C.c_int, [H, C.c_char_p, C.c_size_t]),
    ("poly_destroy", C.c_int, [H]),
    ("ewald_rec_std_noalloc", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, PF64, C.c_double, C.c_int32,
                                        C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_char_p, C.c_size_t]),
]

# every function the header declares (checked against the .so in tests)
HEADER_FUNCTIONS = sorted(["mg_" + s[0] for s in SIGNATURES + LIB_ONLY])

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmolsim_gb300.so")


def declare(lib, prefix, sigs):
    for name, res, args in sigs:
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = None


def load_library(path=None):
    """Load the GB300 library.  There is no fallback: a missing library is an
    error (build it with __graft_entry__.build() or molsim_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"molsim_gb300: native library {p} is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    declare(lib, "mg_", SIGNATURES + LIB_ONLY)
    if lib.mg_abi_version() != MG_ABI_VERSION:
        raise RuntimeError("molsim_gb300: ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def ptr(a, ctype):
    """Pointer to a contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


def f64(a):
    return ptr(a, C.c_double)


def i32(a):
    return ptr(a, C.c_int32)


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def as_i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)
