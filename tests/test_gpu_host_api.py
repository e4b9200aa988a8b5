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


def test_host_commutator_rejects_aliased_result(gpu_lib):
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    a, r = np.zeros(lay.nfull), np.zeros(lay.nfull)
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.commutator_host(B, a, -1, r, 1, r)
