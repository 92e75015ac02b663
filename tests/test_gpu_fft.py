"""The device 3D FFT against cuFFT (torch.fft on the GPU).

The library's FFT replaces FFTW's r2c/c2r pair in SPMFFTRec
(energy.F90:6525-6587) around the influence-function multiply of
UEwaldRecSPM (energy.F90:1243-1254).  mg_fft_check runs the form's
transforms as UTotal does (FP64: line passes; mixed: plane/slab passes for
32..128 points, FP32 line passes otherwise) with a random multiplier in
place of meshfac, so that the output c2r(mult * r2c(q)) pins both the
forward and the inverse transform, and returns sum ew |r2c(q)|^2.  The same
quantities from torch.fft.rfftn/irfftn (cuFFT) must agree: FP64 within
1e-12, the mixed (FP32) form within 1e-5, relative to the largest value.

The device FFT supports the even meshes 2^a 3^b 5^c from 8 to 512 points
per edge (Stockham passes of radices 4, 2, 3 and 5; powers of two also
through the mixed form's plane passes); other sizes are refused.
"""
import ctypes as C

import numpy as np
import pytest

from molsim_gb300 import Engine, abi, configs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _fold(n):
    k = np.arange(n)
    return np.minimum(k, n - k)


def _handle(n, form):
    s = configs.small_system(seed=61, n=120, L=40.0, nmesh=n, order=4)
    s.build_table()
    return Engine(s, form=form)


def _cufft(q, mult, ew):
    n = q.shape[0]
    f = _fold(n)
    m_full = mult[f[:, None], f[None, :], :]          # [kz][ky][kx]
    e_full = ew[f[:, None], f[None, :], :]
    qt = torch.from_numpy(q).cuda()
    F = torch.fft.rfftn(qt)                            # axes z, y, x; x halved
    phi = torch.fft.irfftn(F * torch.from_numpy(m_full).cuda(), s=(n, n, n)) * n ** 3
    esum = float((torch.from_numpy(e_full).cuda() * F.abs() ** 2).sum())
    return phi.cpu().numpy(), esum


@pytest.mark.parametrize("n", [16, 24, 32, 40, 48, 60, 64, 96, 120, 128, 150, 256])
@pytest.mark.parametrize("form,tol", [(abi.MG_FP64, 1e-12), (abi.MG_MIXED, 1e-5)], ids=["fp64", "mixed"])
def test_fft_matches_cufft(n, form, tol, gpu_lib):
    rng = np.random.default_rng(1000 + n)
    nh = n // 2 + 1
    q = rng.uniform(-1.0, 1.0, (n, n, n))
    mult = rng.uniform(0.5, 1.5, (nh, nh, nh))
    ew = rng.uniform(0.0, 1.0, (nh, nh, nh))
    g = _handle(n, form)
    phi = np.zeros(n ** 3)
    esum = np.zeros(1)
    st = gpu_lib.mg_fft_check(g.h, abi.f64(np.ascontiguousarray(q.reshape(-1))),
                              abi.f64(np.ascontiguousarray(mult.reshape(-1))),
                              abi.f64(np.ascontiguousarray(ew.reshape(-1))), abi.f64(phi), abi.f64(esum))
    assert st == 0
    phi_ref, e_ref = _cufft(q, mult, ew)
    err = np.abs(phi.reshape(n, n, n) - phi_ref).max() / np.abs(phi_ref).max()
    assert err <= tol, err
    assert abs(esum[0] - e_ref) <= tol * abs(e_ref), (esum[0], e_ref)
    g.close()


def test_unsupported_meshes_are_refused(gpu_lib):
    """Odd meshes and meshes with a prime factor above 5 are refused at
    creation with MG_ERR_UNSUPPORTED."""
    from molsim_gb300.engine import MolsimError
    for n in (42, 45, 14):
        s = configs.small_system(seed=61, n=120, L=40.0, nmesh=n, order=4)
        s.build_table()
        with pytest.raises(MolsimError) as ex:
            Engine(s)
        assert abi.STATUS[ex.value.status] == "MG_ERR_UNSUPPORTED"


def test_fft_check_then_utotal_unchanged(gpu_lib):
    """mg_fft_check leaves no trace: UTotal afterwards gives the same bits
    as before it."""
    s = configs.small_system(seed=62, n=200, L=36.0, nmesh=32, order=6)
    s.build_table()
    g = Engine(s)
    g.SetPositions(s.ro_flat())
    g.NList("write")
    before = g.UTotal()
    n, nh = 32, 17
    phi = np.zeros(n ** 3)
    esum = np.zeros(1)
    assert gpu_lib.mg_fft_check(g.h, abi.f64(np.ones(n ** 3)), abi.f64(np.ones(nh ** 3)),
                                abi.f64(np.ones(nh ** 3)), abi.f64(phi), abi.f64(esum)) == 0
    # a constant mesh has only the k = 0 component: phi = n^3 q, esum = (n^3)^2
    assert np.allclose(phi, n ** 3) and abs(esum[0] - float(n ** 6)) <= 1e-9 * n ** 6
    after = g.UTotal()
    assert np.array_equal(before["forceo"], after["forceo"]) and before["u_tot"] == after["u_tot"]
    g.close()
