"""The allocation-free commutator entry point (collected last on purpose).

imsrg_gpu_commutator_noalloc serves callers that may not allocate device
memory while they run (memory owned or capped by another allocator, or code
where a cudaMalloc/cudaFree, which can synchronise the device, is not
allowed).  Its intermediates live in one fixed library array, so these tests
check it, through the C ABI, against the regular imsrg_gpu_commutator on two
calls in a row with different inputs, and check the size limit."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10  # the FP64 path's bar, max-norm relative


@pytest.mark.parametrize("emax", [2, 4])
def test_noalloc_matches_commutator_twice(gpu_lib, emax):
    from imsrg_gpu.synth import random_operator, synth_hamiltonian, synth_omega
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    cases = [(synth_omega(lay, 21), -1, synth_hamiltonian(lay, 21), 1),
             (random_operator(lay, 1, 22, 1), 1, random_operator(lay, -1, 23, 2), -1)]
    for Lh, hL, Rh, hR in cases:  # two calls in a row, different inputs
        L, R = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh)
        ref, out = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(L, R, ref, precision="fp64")
        gpu_lib.commutator_noalloc(B, L.device_ptr(), hL, R.device_ptr(), hR, out.device_ptr())
        B.synchronize()
        want = ref.download()
        got = out.download()
        assert rel_err(got, want) <= TOL
        assert abs(got[0] - want[0]) <= TOL * max(1.0, abs(want[0]))


def test_noalloc_rejects_basis_beyond_limit(gpu_lib):
    bas, lay = make_case(6)
    B = gpu_lib.Basis.from_dict(bas)
    L, R, out = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.commutator_noalloc(B, L.device_ptr(), -1, R.device_ptr(), 1, out.device_ptr())
    assert e.value.status == 9
