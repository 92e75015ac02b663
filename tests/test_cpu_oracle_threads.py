"""The oracle's threads (the reference's MPI replicated-data ranks restated
with threads) against its serial path.

Thread t of nt takes the t-th contiguous particle range, accumulates private
force arrays, energy sums and (SPME) a private charge mesh, and the partials
are summed in thread order, as molsim_par's allreduce does.  The results
differ from the serial sums only by the order of the additions: energies and
forces agree to 1e-12 relative, the FFT agrees bit for bit (its lines are
independent), and a thread count gives the same bits on every run.
"""
import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs


@pytest.fixture
def orc_threads(orc):
    yield orc
    orc.orc_set_threads(1)


def _utotal(orc, s):
    e = Engine(s, lib=orc, prefix="orc_")
    e.SetPositions(s.ro_flat())
    e.NList("write")
    r = e.UTotal()
    e.close()
    return r


@pytest.mark.parametrize("kw", [
    dict(ewald=abi.MG_EWALD_SPM, chains=3, nseg=8),
    dict(ewald=abi.MG_EWALD_SPM, txintlist=abi.MG_CELLLIST, lsurf=1),
    dict(ewald=abi.MG_EWALD_STD, ncut=5),
], ids=["spme_vlist_bonds", "spme_cell_surf", "std_vlist"])
def test_threaded_utotal_matches_serial(orc_threads, kw):
    orc = orc_threads
    s = configs.small_system(seed=31, nmesh=32, **kw)
    s.build_table(orc.orc_pot_twobody_tab)
    assert orc.orc_set_threads(1) == 0
    r1 = _utotal(orc, s)
    assert orc.orc_set_threads(5) == 0
    r5 = _utotal(orc, s)
    r5b = _utotal(orc, s)
    for k in ("u_tot", "u_rec", "u_bond", "virial"):
        assert abs(r5[k] - r1[k]) <= 1e-12 * max(abs(r1[k]), 1.0), k
        assert r5[k] == r5b[k]                           # same thread count, same bits
    f1, f5 = r1["forceo"], r5["forceo"]
    assert np.abs(f5 - f1).max() <= 1e-12 * np.abs(f1).max()
    assert np.array_equal(f5, r5b["forceo"])


def test_threaded_fft_is_bitwise_serial(orc_threads):
    orc = orc_threads
    n = 32
    q = np.random.default_rng(4).standard_normal(n ** 3)
    out = []
    for nt in (1, 7):
        assert orc.orc_set_threads(nt) == 0
        fq = np.zeros(2 * (n // 2 + 1) * n * n)
        back = np.zeros(n ** 3)
        assert orc.orc_fft_r2c_3d(n, abi.f64(q), abi.f64(fq)) == 0
        assert orc.orc_fft_c2r_3d(n, abi.f64(fq), abi.f64(back)) == 0
        out.append((fq, back))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_thread_count_bounds(orc_threads):
    assert orc_threads.orc_set_threads(0) != 0
    assert orc_threads.orc_set_threads(65) != 0
