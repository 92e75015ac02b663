"""TEST INFRASTRUCTURE ONLY: load the CPU oracle through ctypes.

The oracle exports orc_* entry points with the same arguments as the
library's mg_* entry points, so molsim_gb300.Engine(system, lib=oracle(),
prefix="orc_") runs the reference's algorithm on the CPU.
"""
import ctypes as C

from molsim_gb300 import abi

from .build_oracle import build

_lib = None


def oracle():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        abi.declare(lib, "orc_", abi.SIGNATURES)
        lib.orc_erf2.restype = C.c_double
        lib.orc_erf2.argtypes = [C.c_double]
        lib.orc_random.restype = C.c_double
        lib.orc_random.argtypes = [C.POINTER(C.c_int32)]
        lib.orc_gau_random.restype = C.c_double
        lib.orc_gau_random.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        lib.orc_fft_r2c_3d.restype = C.c_int
        lib.orc_fft_r2c_3d.argtypes = [C.c_int, abi.PF64, abi.PF64]
        lib.orc_fft_c2r_3d.restype = C.c_int
        lib.orc_fft_c2r_3d.argtypes = [C.c_int, abi.PF64, abi.PF64]
        lib.orc_cardinal_bspline.restype = C.c_int
        lib.orc_cardinal_bspline.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_int), abi.PF64, abi.PF64]
        lib.orc_celllist_test.restype = C.c_int
        lib.orc_celllist_test.argtypes = [C.c_void_p]
        lib.orc_get_qmesh.restype = C.c_int
        lib.orc_get_qmesh.argtypes = [C.c_void_p, abi.PF64]
        lib.orc_set_threads.restype = C.c_int
        lib.orc_set_threads.argtypes = [C.c_int]
        lib.orc_poly_dutwobody.restype = C.c_int
        lib.orc_poly_dutwobody.argtypes = [C.POINTER(abi.MgPolyParams), C.c_int32, abi.PF64, abi.PF64, abi.PI32,
                                           abi.PI32, C.c_int32, abi.PF64, abi.PF64, abi.PF64, abi.PI32]
        lib.orc_poly_dutwobody_multi.restype = C.c_int
        lib.orc_poly_dutwobody_multi.argtypes = [C.POINTER(abi.MgPolyParams), C.c_int32, abi.PF64, abi.PF64,
                                                 abi.PI32, abi.PI32, C.c_int32, abi.PI32, abi.PF64, abi.PF64,
                                                 abi.PF64, abi.PI32]
        lib.orc_poly_epilogue.restype = C.c_int
        lib.orc_poly_epilogue.argtypes = [C.POINTER(abi.MgPolyParams), abi.PF64, abi.PF64, abi.PF64, abi.PF64,
                                          C.c_double,
                                          abi.PF64, abi.PF64, abi.PF64]
        lib.orc_poly_ewald_intra.restype = C.c_int
        lib.orc_poly_ewald_intra.argtypes = [C.POINTER(abi.MgPolyParams), abi.PF64, abi.PF64, abi.PF64]
        lib.orc_poly_utwobody.restype = C.c_int
        lib.orc_poly_utwobody.argtypes = [C.POINTER(abi.MgPolyParams), C.c_int32, abi.PF64, abi.PF64, abi.PI32,
                                          abi.PI32, abi.PF64, abi.PF64, abi.PF64]
        lib.orc_angvel_to_quavel.restype = C.c_int
        lib.orc_angvel_to_quavel.argtypes = [C.c_int32, abi.PF64, abi.PF64, abi.PF64]
        lib.orc_rigid_move.restype = C.c_int
        lib.orc_rigid_move.argtypes = [C.c_int32, C.c_double, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64,
                                       abi.PF64, abi.PF64, abi.PF64, abi.PF64]
        lib.orc_rigid_kick.restype = C.c_int
        lib.orc_rigid_kick.argtypes = [C.c_int32, C.c_double, C.c_double, C.c_int32, abi.PF64, abi.PF64, abi.PF64,
                                       abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64]
        P = C.POINTER(abi.MgPolyParams)
        lib.orc_poly_udipole_real.restype = C.c_int
        lib.orc_poly_udipole_real.argtypes = [P, C.c_int32, abi.PF64, abi.PF64, abi.PF64, abi.PI32, abi.PI32,
                                              abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64]
        lib.orc_poly_udipole_self.restype = C.c_int
        lib.orc_poly_udipole_self.argtypes = [P, abi.PF64, abi.PF64, C.c_int32, abi.PF64, abi.PF64, abi.PF64,
                                              abi.PF64]
        lib.orc_poly_udipole_finish.restype = C.c_int
        lib.orc_poly_udipole_finish.argtypes = [P, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64,
                                                abi.PF64]
        lib.orc_dipole_ewald.restype = C.c_int
        lib.orc_dipole_ewald.argtypes = [C.c_void_p, abi.PF64, abi.PF64, abi.PF64, abi.PF64, abi.PF64]
        _lib = lib
    return _lib
