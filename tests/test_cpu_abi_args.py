"""The C ABI refuses malformed systems before it touches the GPU: an empty or
one-particle system, inconsistent type-pair counts, missing arrays, unknown
options, a degenerate box; and malformed polyatomic descriptions (no GPU
needed: these checks run on the host)."""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import abi, configs
from molsim_gb300.system import iptpt_matrix

CODE = {name: code for code, name in abi.STATUS.items()}


@pytest.fixture(scope="module")
def lib():
    import molsim_gb300
    molsim_gb300.build()
    return abi.load_library()


@pytest.fixture(scope="module")
def good(orc):
    s = configs.small_system(seed=3)
    s.build_table(orc.orc_pot_twobody_tab)
    return s


def _create(lib, p):
    h = C.c_void_p()
    st = lib.mg_create(C.byref(p), C.byref(h))
    if st == 0:
        lib.mg_destroy(h)
    return st


@pytest.mark.parametrize("field,value,code", [
    ("np", 0, "MG_ERR_ARG"),                 # empty system
    ("np", 1, "MG_ERR_ARG"),                 # a single particle has no pairs
    ("npt", 0, "MG_ERR_ARG"),
    ("nptpt", 5, "MG_ERR_UNSUPPORTED"),      # not npt(npt+1)/2
    ("abi_version", 1, "MG_ERR_ARG"),
    ("form", 7, "MG_ERR_ARG"),
    ("mode", 9, "MG_ERR_ARG"),
    ("txintlist", 4, "MG_ERR_ARG"),
    ("rcut", 0.0, "MG_ERR_ARG"),
    ("drnlist", -1.0, "MG_ERR_ARG"),
    ("nbuf", 3, "MG_ERR_ARG"),               # shorter than one table record
])
def test_create_refuses_bad_parameters(field, value, code, good, lib):
    p, keep = good.params()
    setattr(p, field, value)
    assert _create(lib, p) == CODE[code]


def test_create_refuses_missing_arrays_and_flat_boxes(good, lib):
    for f in ("iptpn", "az", "ubuf", "r2umin"):
        p, keep = good.params()
        setattr(p, f, None)
        assert _create(lib, p) == CODE["MG_ERR_ARG"], f
    p, keep = good.params()
    p.boxlen[2] = 0.0
    assert _create(lib, p) == CODE["MG_ERR_ARG"]


def test_poly_create_refuses_bad_descriptions(orc, lib):
    s = configs.water_ions(seed=9, nwater=20, nsalt=2, L=14.0)
    s.build_table(orc.orc_pot_twobody_tab)

    def create(p, maxn=50):
        h = C.c_void_p()
        st = lib.mg_poly_create(C.byref(p), maxn, C.byref(h))
        assert not h.value or st != 0   # nothing is returned on a refusal
        return st

    p = s.params()
    assert create(p, maxn=0) == CODE["MG_ERR_ARG"]          # no list room
    bad = s.params()
    bad.na = 3                                                # fewer atoms than the particles hold
    assert create(bad) == CODE["MG_ERR_ARG"]
    bad = s.params()
    k = np.array(s.keep["iatan"]).copy()
    k[0] = 9                                                  # an atom type past nat
    bad.iatan = abi.i32(abi.as_i32(k))
    bad._k2 = k
    assert create(bad) == CODE["MG_ERR_ARG"]
    bad = s.params()
    bad.nptpt = 4                                             # not npt(npt+1)/2
    assert create(bad) == CODE["MG_ERR_ARG"]
