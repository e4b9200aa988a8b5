"""imsrg_gpu_commutator_host: the commutator on host operands (copies in,
commutator, copy out in one call) equals the device-operand commutator bit for
bit, from page-locked and from ordinary host buffers, call after call."""
import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu


def _pinned(a):
    import torch
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    out = t.numpy()
    out[:] = a
    return out, t


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_commutator_equals_device_commutator(gpu_lib, precision, pinned):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(4)
    B = gpu_lib.Basis.from_dict(bas)
    keep = []
    for seed in (5, 6):
        Hh, Oh = synth_hamiltonian(lay, seed), synth_omega(lay, seed)
        O, H, R = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(O, H, R, precision=precision)
        ref = R.download()
        if pinned:
            (ho, to), (hh, th), (hr, tr) = _pinned(Oh), _pinned(Hh), _pinned(np.zeros(lay.nfull))
            keep += [to, th, tr]
        else:
            ho, hh, hr = Oh.copy(), Hh.copy(), np.zeros(lay.nfull)
        for _ in range(3):  # first call builds, later calls replay
            hr[:] = np.nan
            gpu_lib.commutator_host(B, ho, -1, hh, 1, hr, precision=precision)
            assert np.array_equal(hr, ref)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_host_commutator_emax6_every_element_returned(gpu_lib, precision):
    """At emax=6 the result comes back in several address ranges beside the
    assembly; every element (the host buffer starts as NaN) must equal the
    device-operand commutator, with the operands' Hermiticity either way."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(6)
    B = gpu_lib.Basis.from_dict(bas)
    Hh, Oh = synth_hamiltonian(lay, 3), synth_omega(lay, 3)
    (ho, to), (hh, th), (hr, tr) = _pinned(Oh), _pinned(Hh), _pinned(np.zeros(lay.nfull))
    omega, ham = (-1, Oh, ho), (1, Hh, hh)
    for (hL, XL, pL), (hR, XR, pR) in ((omega, ham), (ham, omega)):
        L, R, RES = gpu_lib.Operator(B, hL, XL), gpu_lib.Operator(B, hR, XR), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(L, R, RES, precision=precision)
        ref = RES.download()
        for _ in range(2):
            hr[:] = np.nan
            gpu_lib.commutator_host(B, pL, hL, pR, hR, hr, precision=precision)
            assert np.array_equal(hr, ref)


def test_host_commutator_rejects_aliased_result(gpu_lib):
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    a, r = np.zeros(lay.nfull), np.zeros(lay.nfull)
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.commutator_host(B, a, -1, r, 1, r)
    # wrong length, dtype or a strided view are refused before the call
    for bad in (a[:-1], a.astype(np.float32), np.zeros(2 * lay.nfull)[::2]):
        with pytest.raises(ValueError):
            gpu_lib.commutator_host(B, bad, -1, a, 1, np.zeros(lay.nfull))


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("emax", [4, 6])
def test_packed_host_commutator_equals_device_commutator(gpu_lib, precision, pinned, emax):
    """imsrg_gpu_commutator_host_packed (operands in the vectorize layout of
    basic_IMSRG.f90:3794-3918): its result is the packed form of the
    device-operand commutator bit for bit, call after call, interleaved with
    the flat host call on the same basis."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    B.set_split_digits(5)
    keep = []
    for seed in (5, 6):
        Hh, Oh = synth_hamiltonian(lay, seed), synth_omega(lay, seed)
        O, H, R = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(O, H, R, precision=precision)
        ref = R.download_packed()
        Op, Hp = O.download_packed(), H.download_packed()
        if pinned:
            (ho, to), (hh, th), (hr, tr) = _pinned(Op), _pinned(Hp), _pinned(np.zeros(B.neq))
            (fo, t1), (fh, t2), (fr, t3) = _pinned(Oh), _pinned(Hh), _pinned(np.zeros(lay.nfull))
            keep += [to, th, tr, t1, t2, t3]
        else:
            ho, hh, hr = Op.copy(), Hp.copy(), np.zeros(B.neq)
            fo, fh, fr = Oh.copy(), Hh.copy(), np.zeros(lay.nfull)
        for _ in range(3):  # first call builds, later calls replay
            hr[:] = np.nan
            gpu_lib.commutator_host_packed(B, ho, -1, hh, 1, hr, precision=precision)
            assert np.array_equal(hr, ref)
            gpu_lib.commutator_host(B, fo, -1, fh, 1, fr, precision=precision)
            assert np.array_equal(fr, R.download())
    with pytest.raises(ValueError):
        gpu_lib.commutator_host_packed(B, np.zeros(lay.nfull), -1, hh, 1, hr)
