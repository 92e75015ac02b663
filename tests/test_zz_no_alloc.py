"""The allocation-free standard Ewald entry point, mg_ewald_rec_std_noalloc.

It exists for callers that cannot allocate device memory (a host code whose
device memory all belongs to its own pool, or one that must not let
cudaMalloc/cudaFree synchronise the device in the middle of its step).  It
takes caller-owned device buffers and keeps its working memory in a fixed
array inside the library.  These tests check it against the reciprocal part
of mg_utotal -- the same system with the Ewald sum on minus the same system
with it off -- on two calls in a row, so that a second call that saw the
first call's leftovers in the shared array would show up.

This file sorts last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import TOL_FP64, force_err
from molsim_gb300 import Engine, abi, configs, units

pytestmark = pytest.mark.gpu

MG_ERR_ARG = {name: code for code, name in abi.STATUS.items()}["MG_ERR_ARG"]
MAX_NCUT = 24   # MG_NOALLOC_MAX_NCUT


class _EwaldOff:
    """The same system (same table, lists and positions) with the Ewald sum
    switched off in the parameters handed to mg_create."""

    def __init__(self, system):
        self._s = system

    def params(self, form=abi.MG_FP64):
        p, keep = self._s.params(form)
        p.ewald = abi.MG_EWALD_NONE
        p.lsurf = 0
        return p, keep

    def __getattr__(self, name):
        return getattr(self._s, name)


def _system(ncut=6, cube=0):
    s = configs.small_system(seed=16, ewald=abi.MG_EWALD_STD, ncut=ncut)
    s.ncutregion_cube = cube
    s.build_table()
    return s


def _utotal(system):
    e = Engine(system)
    e.SetPositions(system.ro_flat())
    e.NList("write")
    r = e.UTotal()
    e.close()
    return r


def _call(lib, s, d_ro, d_az, d_force, d_uout, ncut=None):
    torch = pytest.importorskip("torch")
    box = (C.c_double * 3)(*[float(x) for x in s.boxlen])
    err = C.create_string_buffer(256)
    st = lib.mg_ewald_rec_std_noalloc(
        s.np_, C.c_void_p(d_ro.data_ptr()), C.c_void_p(d_az.data_ptr()),
        C.cast(box, abi.PF64), s.ualpha, s.ncut if ncut is None else ncut, s.ncutregion_cube,
        s.epsi_four_pi, C.c_void_p(d_force.data_ptr()), C.c_void_p(d_uout.data_ptr()), None,
        err, len(err))
    torch.cuda.synchronize()
    return st, err.value.decode()


# (ncut, ncutregion_cube): the spherical region; the largest ncut, which
# uses every slot of the fixed array; the cube region (|n|^2 <= 3 ncut^2)
@pytest.mark.parametrize("ncut,cube", [(6, 0), (MAX_NCUT, 0), (4, 1)], ids=["sphere6", "sphere_max", "cube4"])
def test_noalloc_matches_utotal_twice(ncut, cube, gpu_lib):
    torch = pytest.importorskip("torch")
    s = _system(ncut, cube)
    on = _utotal(s)
    off = _utotal(_EwaldOff(s))
    f_rec = (on["forceo"] - off["forceo"]).reshape(-1) / units.FORCE_FAC
    vir_rec = on["virial"] - off["virial"]
    assert off["u_rec"] == 0.0

    dev = torch.device("cuda", 0)
    d_ro = torch.from_numpy(s.ro_flat()).to(dev)
    d_az = torch.from_numpy(np.ascontiguousarray(s.az)).to(dev)
    d_force = torch.empty(3 * s.np_, dtype=torch.float64, device=dev)
    d_uout = torch.empty(2, dtype=torch.float64, device=dev)
    results = []
    for _ in range(2):
        d_force.zero_()
        d_uout.fill_(float("nan"))
        st, msg = _call(gpu_lib, s, d_ro, d_az, d_force, d_uout)
        assert st == abi.MG_OK, msg
        f = d_force.cpu().numpy()
        u = d_uout.cpu().numpy()
        assert abs(u[0] - on["u_rec"]) / max(abs(on["u_rec"]), 1.0) < TOL_FP64
        assert abs(u[1] - vir_rec) / max(abs(vir_rec), 1.0) < TOL_FP64
        assert force_err(f, f_rec) < TOL_FP64
        results.append((f, u))
    # the second call starts from the first call's leftovers and must not see them
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])


def test_noalloc_rejects_ncut_beyond_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    s = _system()
    dev = torch.device("cuda", 0)
    d_ro = torch.from_numpy(s.ro_flat()).to(dev)
    d_az = torch.from_numpy(np.ascontiguousarray(s.az)).to(dev)
    d_force = torch.zeros(3 * s.np_, dtype=torch.float64, device=dev)
    d_uout = torch.zeros(2, dtype=torch.float64, device=dev)
    st, msg = _call(gpu_lib, s, d_ro, d_az, d_force, d_uout, ncut=MAX_NCUT + 1)
    assert st == MG_ERR_ARG
    assert f"ncut = {MAX_NCUT + 1}" in msg and "scratch" in msg
    assert not d_force.any().item()
