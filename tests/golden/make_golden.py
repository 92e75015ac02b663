"""Generate tests/golden/oracle_small.npz from the CPU oracle.

    python tests/golden/make_golden.py

The fixture freezes the oracle's outputs on small seeded systems: UTotal
(energies, virial, forces) for several list/Ewald combinations, a Verlet
list, five BD steps (positions and the GauRandom state) and five
velocity-Verlet steps, plus Erf2 and GauRandom samples.  The systems are
regenerated from their seeds by molsim_gb300.configs; the stored positions
guard against a generator change.  tests/test_cpu_golden.py checks that the
oracle still reproduces the fixture and tests/test_gpu_golden.py checks the
GPU against it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from molsim_gb300 import Engine, abi, configs  # noqa: E402

OUT = os.path.join(HERE, "oracle_small.npz")

# name -> keyword arguments of configs.small_system
CASES = {
    "spme_vlist_md": dict(seed=101),
    "spme_cell_bonds": dict(seed=102, txintlist=abi.MG_CELLLIST, chains=3, nseg=10),
    "std_vlist_surf": dict(seed=103, ewald=abi.MG_EWALD_STD, ncut=5, lsurf=1),
    "spme_order8_mc": dict(seed=104, nmesh=32, order=8, mode=abi.MG_MC),
    "wca_no_ewald": dict(seed=105, ewald=abi.MG_EWALD_NONE, lljcut=1),
}
BD_CASE = dict(seed=106, mode=abi.MG_BD, chains=2, nseg=8)
BD_SEED, BD_DT, BD_STEPS = 4711, 0.01, 5
MD_CASE = dict(seed=107)
MD_DT, MD_STEPS = 0.002, 5


def system(kw, orc):
    s = configs.small_system(**kw)
    s.build_table(orc.orc_pot_twobody_tab)
    return s


def make(orc):
    out = {}
    for name, kw in CASES.items():
        s = system(kw, orc)
        e = Engine(s, lib=orc, prefix="orc_")
        e.SetPositions(s.ro_flat())
        e.NList("write")
        r = e.UTotal()
        out[f"{name}/ro"] = s.ro_flat()
        out[f"{name}/u_twob"] = r["u_twob"]
        out[f"{name}/scalars"] = np.array([r["u_tot"], r["u_rec"], r["u_bond"], r["virial"]])
        out[f"{name}/forceo"] = r["forceo"].reshape(-1)
        if name == "spme_vlist_md":
            nn, lists = e.VList()
            pairs = sorted((min(i + 1, int(j)), max(i + 1, int(j))) for i, js in enumerate(lists) for j in js)
            out[f"{name}/nneighpn"] = nn
            out[f"{name}/pairs"] = np.array(pairs, dtype=np.int32)
        e.close()

    s = system(BD_CASE, orc)
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    e.BDSetup(BD_DT, BD_SEED)
    r = e.BDRun(BD_STEPS)
    out["bd/ro0"] = s.ro_flat()
    out["bd/ro"] = e.GetPositions().reshape(-1)
    out["bd/forceo"] = r["forceo"].reshape(-1)
    out["bd/seed"] = np.array([e.BDSeed()], dtype=np.int64)
    e.close()

    s = system(MD_CASE, orc)
    rod = s.maxwell_velocities(seed=MD_CASE["seed"])
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    e.MDSetup(MD_DT, rod)
    r = e.VelVer(MD_STEPS)
    out["md/ro0"] = s.ro_flat()
    out["md/rod0"] = np.asarray(rod, dtype=np.float64).reshape(-1)
    out["md/ro"] = e.GetPositions().reshape(-1)
    out["md/rod"] = r["rod"].reshape(-1)
    out["md/scalars"] = np.array([r["u_tot"], r["u_rec"], r["u_bond"], r["virial"]])
    e.close()

    xs = np.linspace(-6.5, 6.5, 53)
    out["erf2/x"] = xs
    out["erf2/y"] = np.array([orc.orc_erf2(float(x)) for x in xs])
    seed, flag, save = C.c_int32(12345), C.c_int32(1), C.c_double(0.0)
    out["gau/y"] = np.array([orc.orc_gau_random(C.byref(seed), C.byref(flag), C.byref(save))
                             for _ in range(21)])
    out["gau/seed"] = np.array([seed.value], dtype=np.int64)
    return out


if __name__ == "__main__":
    from oracle.loader import oracle
    data = make(oracle())
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays, {os.path.getsize(OUT)} bytes")
