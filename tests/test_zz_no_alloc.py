"""The allocation-free commutator entry point (collected last on purpose).

imsrg_gpu_commutator_noalloc serves callers that may not allocate device
memory while they run (memory owned or capped by another allocator, or code
where a cudaMalloc/cudaFree, which can synchronise the device, is not
allowed).  Its intermediates live in one fixed library array, so these tests
check it, through the C ABI, against the regular imsrg_gpu_commutator on
calls in a row with different inputs and every Hermiticity pair (the
(+1, +1) and (-1, -1) pairs take the branch without the 220 energy terms),
without E0, on a caller-created stream, and check the size and overlap
rules."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10  # the FP64 path's bar, max-norm relative


@pytest.mark.parametrize("emax", [2, 4])
def test_noalloc_matches_commutator_in_a_row(gpu_lib, emax):
    from imsrg_gpu.synth import random_operator, synth_hamiltonian, synth_omega
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    cases = [(synth_omega(lay, 21), -1, synth_hamiltonian(lay, 21), 1),
             (random_operator(lay, 1, 22, 1), 1, random_operator(lay, -1, 23, 2), -1),
             (random_operator(lay, 1, 24, 1), 1, random_operator(lay, 1, 25, 2), 1),
             (random_operator(lay, -1, 26, 1), -1, random_operator(lay, -1, 27, 2), -1)]
    for Lh, hL, Rh, hR in cases:  # calls in a row, different inputs
        L, R = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh)
        ref, out = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(L, R, ref, precision="fp64")
        gpu_lib.commutator_noalloc(B, L.device_ptr(), hL, R.device_ptr(), hR, out.device_ptr())
        B.synchronize()
        want = ref.download()
        got = out.download()
        assert rel_err(got, want) <= TOL, (hL, hR)
        assert abs(got[0] - want[0]) <= TOL * max(1.0, abs(want[0])), (hL, hR)


def test_noalloc_without_e0_on_caller_stream(gpu_lib):
    """with_e0 = 0 leaves E0 of the output as it was; the work runs on a
    stream the caller created."""
    import torch
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(4)
    B = gpu_lib.Basis.from_dict(bas)
    L, R = gpu_lib.Operator(B, -1, synth_omega(lay, 31)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 31))
    init = np.zeros(lay.nfull)
    init[0] = 7.5
    ref, out = gpu_lib.Operator(B, 1, init), gpu_lib.Operator(B, 1, init)
    gpu_lib.commutator(L, R, ref, precision="fp64", with_e0=False)
    s = torch.cuda.Stream()
    B.synchronize()
    for _ in range(2):
        gpu_lib.commutator_noalloc(B, L.device_ptr(), -1, R.device_ptr(), 1, out.device_ptr(), with_e0=False,
                                   stream=s.cuda_stream)
    s.synchronize()
    got, want = out.download(), ref.download()
    assert got[0] == 7.5
    assert rel_err(got, want) <= TOL


def test_noalloc_rejects_basis_beyond_limit(gpu_lib):
    bas, lay = make_case(6)
    B = gpu_lib.Basis.from_dict(bas)
    L, R, out = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.commutator_noalloc(B, L.device_ptr(), -1, R.device_ptr(), 1, out.device_ptr())
    assert e.value.status == 9


def test_noalloc_rejects_overlapping_output(gpu_lib):
    """An output that shares elements with an input, even offset from it, is
    rejected before any work is queued."""
    import torch
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    buf = torch.zeros(3 * lay.nfull, dtype=torch.float64, device="cuda")
    base = buf.data_ptr()
    d_L, d_R = base, base + lay.nfull * 8
    for d_RES in (base + 8 * (lay.nfull // 2), d_R + 8, d_L):
        with pytest.raises(gpu_lib.ImsrgError) as e:
            gpu_lib.commutator_noalloc(B, d_L, -1, d_R, 1, d_RES)
        assert e.value.status == 1
