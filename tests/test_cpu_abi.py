"""The C ABI without a GPU: the header, the ctypes mirror and the built
library agree, and the host-only entry points (table build, alpha) match the
oracle bit for bit.  No call here touches a device."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from molsim_gb300 import abi, configs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "molsim_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import molsim_gb300
    molsim_gb300.build()
    return abi.load_library()


def test_header_and_ctypes_mirror_list_the_same_functions():
    assert header_functions() == abi.HEADER_FUNCTIONS


def test_library_exports_every_header_function(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    for f in header_functions():
        assert getattr(lib, f) is not None


def test_abi_version_and_status_strings(lib):
    assert lib.mg_abi_version() == abi.MG_ABI_VERSION
    for code, name in abi.STATUS.items():
        s = lib.mg_status_string(code)
        assert s is not None and len(s) > 0, name
    buf = C.create_string_buffer(64)
    assert lib.mg_last_error(None, buf, len(buf)) == 0


_LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "molsim_gb300.h"
#define F(T, m) printf("%s %s %zu\n", #T, #m, offsetof(T, m));
int main(void) {
@FIELDS@
    printf("mg_params sizeof %zu\n", sizeof(mg_params));
    printf("mg_pot_params sizeof %zu\n", sizeof(mg_pot_params));
    printf("mg_poly_params sizeof %zu\n", sizeof(mg_poly_params));
    return 0;
}
"""


def test_struct_layouts_match_the_header(tmp_path):
    lines = []
    for T, cls in (("mg_params", abi.MgParams), ("mg_pot_params", abi.MgPotParams),
                   ("mg_poly_params", abi.MgPolyParams)):
        for name, _ in cls._fields_:
            lines.append(f"    F({T}, {name})")
    src = tmp_path / "layout.c"
    src.write_text(_LAYOUT_C.replace("@FIELDS@", "\n".join(lines)))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            T, m, v = line.split()
            got[(T, m)] = int(v)
    for T, cls in (("mg_params", abi.MgParams), ("mg_pot_params", abi.MgPotParams),
                   ("mg_poly_params", abi.MgPolyParams)):
        for name, _ in cls._fields_:
            assert getattr(cls, name).offset == got[(T, name)], (T, name)
        assert C.sizeof(cls) == got[(T, "sizeof")], T


@pytest.mark.parametrize("factory", [
    lambda: configs.small_system(seed=3),
    lambda: configs.small_system(seed=4, ewald=abi.MG_EWALD_STD, ncut=5, lljcut=1),
    lambda: configs.electrolyte_spme(seed=2, n=200, L=60.0, nmesh=16),
])
def test_library_table_is_bit_identical_to_the_oracle(lib, orc, factory):
    s1, s2 = factory(), factory()
    s1.build_table(lib.mg_pot_twobody_tab)
    s2.build_table(orc.orc_pot_twobody_tab)
    assert np.array_equal(s1.iubuflow, s2.iubuflow)
    assert np.array_equal(s1.r2umin, s2.r2umin)
    assert s1.ubuf.shape == s2.ubuf.shape
    assert np.array_equal(s1.ubuf, s2.ubuf)


def test_library_rcut_to_alpha_matches_the_oracle(lib, orc):
    for tol, rc, q2, L in ((1e-5, 12.0, 65600.0, 700.0), (1e-4, 9.0, 400.0, 40.0), (1e-6, 30.0, 1000.0, 100.0)):
        a1, a2 = np.zeros(1), np.zeros(1)
        eps = 1389.35 / 78.5
        assert lib.mg_rcut_to_alpha(tol, rc, q2, L, eps, abi.f64(a1)) == 0
        assert orc.orc_rcut_to_alpha(tol, rc, q2, L, eps, abi.f64(a2)) == 0
        assert a1[0] == a2[0] and a1[0] > 0
