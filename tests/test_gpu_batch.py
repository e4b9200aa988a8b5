"""Batches of independent commutators (imsrg_gpu_batch_*): the products of all
bases in one persistent launch give, for every basis, exactly the commutator
its own call gives (bit for bit, both precisions, graph replays included), for
bases of different sizes and Hamiltonians of different scales."""
import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu


def _instances(gpu_lib, emaxes, digits=None):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    out = []
    for k, emax in enumerate(emaxes):
        bas, lay = make_case(emax)
        B = gpu_lib.Basis.from_dict(bas)
        if digits:
            B.set_split_digits(digits)
        Hh = synth_hamiltonian(lay, 40 + k, hw=12.0 + 3.0 * k, sigma2=0.5 + 0.3 * k)
        Oh = synth_omega(lay, 40 + k)
        out.append((B, lay, Hh, Oh))
    return out


@pytest.mark.parametrize("precision,digits", [("ozaki", None), ("fp64", None), ("ozaki", 8)])
def test_batch_equals_single_commutators(gpu_lib, precision, digits):
    """digits = 8: the FP64-class split engine (chunked FP64 sums at emax = 6)."""
    inst = _instances(gpu_lib, [2, 4, 6, 4, 2, 6], digits)
    refs = []
    for B, lay, Hh, Oh in inst:
        O, H, R = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
        gpu_lib.commutator(O, H, R, precision=precision)
        refs.append(R.download())
    batch = gpu_lib.Batch([i[0] for i in inst])
    L = [gpu_lib.Operator(B, -1, Oh) for B, lay, Hh, Oh in inst]
    Rr = [gpu_lib.Operator(B, 1, Hh) for B, lay, Hh, Oh in inst]
    RES = [gpu_lib.Operator(B, 1) for B, lay, Hh, Oh in inst]
    for _ in range(3):  # capture, then graph replays
        for r in RES:
            r.upload(np.full(r.basis.nfull, np.nan))
        batch.commutator(L, Rr, RES, precision=precision)
        for r, ref in zip(RES, refs):
            assert np.array_equal(r.download(), ref)
    batch.close()


def test_batch_rejects_bad_arguments(gpu_lib):
    inst = _instances(gpu_lib, [2, 2])
    B0, B1 = inst[0][0], inst[1][0]
    with pytest.raises(gpu_lib.ImsrgError):  # a basis twice
        gpu_lib.Batch([B0, B0])
    batch = gpu_lib.Batch([B0, B1])
    L = [gpu_lib.Operator(B0, -1), gpu_lib.Operator(B1, -1)]
    R = [gpu_lib.Operator(B0, 1), gpu_lib.Operator(B1, 1)]
    RES = [gpu_lib.Operator(B0, 1), gpu_lib.Operator(B1, 1)]
    with pytest.raises(gpu_lib.ImsrgError):  # operators of the wrong basis
        batch.commutator([L[1], L[0]], R, RES)
    with pytest.raises(gpu_lib.ImsrgError):  # one pair of Hermiticities per batch
        batch.commutator([L[0], gpu_lib.Operator(B1, 1)], R, RES)
    with pytest.raises(gpu_lib.ImsrgError):  # result aliasing an operand
        batch.commutator(L, R, [R[0], RES[1]])
    batch.commutator(L, R, RES)  # still usable
    batch.close()
