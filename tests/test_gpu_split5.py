"""Five- and four-digit split precision (15 and 10 BF16 products per term
instead of 21) against the FP64 path and the oracle.  Each digit fewer
multiplies the truncation bound (2^-42 K max|A| max|B| with six) by 128, so
the commutator is checked at 1e-7 (five) and 2e-5 (four) relative
(max-norm); the flow still has to meet |dE0| < 1e-6 MeV."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu
TOL = {5: 1e-7, 4: 2e-5}


def _basis(gpu_lib, emax, digits=5):
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    B.set_split_digits(digits)
    return bas, lay, B


@pytest.mark.parametrize("digits", [5, 4])
@pytest.mark.parametrize("emax", [2, 4, 6])
def test_split5_matches_fp64_path(gpu_lib, emax, digits):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B = _basis(gpu_lib, emax, digits)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 5)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 5))
    R64, Roz = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert rel_err(a, b) <= TOL[digits]
    assert abs(a[0] - b[0]) <= 1e-6


@pytest.mark.parametrize("digits", [5, 4])
@pytest.mark.parametrize("hL,hR", [(-1, 1), (-1, -1), (1, 1)])
def test_split5_matches_oracle_random_ops(gpu_lib, oracle_mod, hL, hR, digits):
    from imsrg_gpu.synth import random_operator
    bas, lay, B = _basis(gpu_lib, 4, digits)
    Lh, Rh = random_operator(lay, hL, 61, 1), random_operator(lay, hR, 62, 2)
    ref = oracle_mod.Oracle(**bas).commutator(Lh, hL, Rh, hR)
    L, R, RES = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(L, R, RES, precision="ozaki")
    assert rel_err(RES.download(), ref) <= TOL[digits]


@pytest.mark.parametrize("digits", [5, 8])
@pytest.mark.parametrize("scale", [2.0 ** -40, 2.0 ** 200])
def test_split5_any_magnitude_matches_fp64(gpu_lib, scale, digits):
    """Any magnitude, also at eight digits, whose digit extraction shifts the
    significand left for the block's largest elements."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B = _basis(gpu_lib, 4, digits)
    O = gpu_lib.Operator(B, -1, synth_omega(lay, 5))
    H = gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 5) * scale)
    R64, Roz = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert np.all(np.isfinite(a))
    assert rel_err(a, b) <= (1e-7 if digits == 5 else 1e-13)


@pytest.mark.parametrize("digits", [5, 4])
def test_split5_magnus_flow_emax6(gpu_lib, oracle_mod, digits):
    """emax = 6 Magnus flow to s = 50: E0 within 1e-6 MeV of the FP64 flow."""
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay, B = _basis(gpu_lib, 6, digits)
    Hh = oracle_mod.Oracle(**bas).normal_order(synth_hamiltonian(lay, 13))
    flows = {}
    for prec in ("fp64", "ozaki"):
        HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
        flows[prec] = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5, precision=prec)
    t64, toz = flows["fp64"]["trace"], flows["ozaki"]["trace"]
    assert flows["fp64"]["steps"] == flows["ozaki"]["steps"] > 2
    assert np.max(np.abs(toz[:, 2] - t64[:, 2])) < 1e-6


def test_split_digits_rules(gpu_lib):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    for bad in (3, 9):
        with pytest.raises(gpu_lib.ImsrgError):
            B.set_split_digits(bad)
    B.set_split_digits(5)
    B.set_split_digits(6)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 3)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 3))
    gpu_lib.commutator(O, H, gpu_lib.Operator(B, 1), precision="ozaki")
    B.set_split_digits(6)  # the count in use is accepted
    with pytest.raises(gpu_lib.ImsrgError):
        B.set_split_digits(5)  # the plan exists
