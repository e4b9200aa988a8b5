"""Split-precision contractions longer than the FP32 accumulators' exact
range run in chunks whose exact int64 level sums the epilogue adds before
one conversion.  Forcing short chunks (2 or 5 K steps of 16, every ladder
and WCC product of emax = 4 and 6 then spans several) must stay within the
split path's error bound of the FP64 path (1e-7 relative at five digits,
max-norm) and be deterministic."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("emax,steps,digits", [(4, 2, 5), (6, 5, 5), (4, 2, 8), (6, 3, 7)])
def test_forced_chunks_match_fp64(gpu_lib, emax, steps, digits):
    """At seven and eight digits the chunks add in FP64 instead (every
    level exact within a chunk): the same bound holds, far inside it."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    B.set_split_digits(digits)
    B.set_split_chunk(steps)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 8)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 8))
    R64, Roz, Roz2 = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    gpu_lib.commutator(O, H, Roz2, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert rel_err(a, b) <= (1e-7 if digits < 7 else 1e-12)
    assert abs(a[0] - b[0]) <= 1e-6
    assert np.array_equal(a, Roz2.download())


def test_chunk_setting_rules(gpu_lib):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    with pytest.raises(gpu_lib.ImsrgError):
        B.set_split_chunk(-1)
    B.set_split_chunk(3)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 3)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 3))
    gpu_lib.commutator(O, H, gpu_lib.Operator(B, 1), precision="ozaki")
    B.set_split_chunk(3)  # the setting in use is accepted
    with pytest.raises(gpu_lib.ImsrgError):
        B.set_split_chunk(0)  # the plan exists


def test_emax8_split_commutator_runs_in_chunks(gpu_lib):
    """emax = 8 (90 j-orbits, 6.7 M doubles per operator): its pppp blocks hold
    up to 606 pairs, so the two-term pphh ladder products contract over
    2 x 606 = 1212 > 816 elements and run in chunks; the commutator matches
    the FP64 path at the five-digit bound."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(8)
    assert max(b.npp for b in lay.blocks) == 606
    B = gpu_lib.Basis.from_dict(bas)
    B.set_split_digits(5)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 8)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 8))
    R64, Roz = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert rel_err(a, b) <= 1e-7
    assert abs(a[0] - b[0]) <= 1e-6
