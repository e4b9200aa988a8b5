"""Split-precision (Ozaki, tcgen05) commutator against the FP64 path and the
oracle.  The bar for this path is |dE0| < 1e-6 MeV in the flow; element-wise
the products carry about 2^-42 K max|A| max|B| of truncation, so the
commutator is checked at 1e-9 relative (max-norm) and E0 at 1e-8 MeV."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def _pair(gpu_lib, emax, seed=5):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    Hh, Oh = synth_hamiltonian(lay, seed), synth_omega(lay, seed)
    return bas, lay, B, Hh, Oh


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_ozaki_matches_fp64_path(gpu_lib, emax):
    bas, lay, B, Hh, Oh = _pair(gpu_lib, emax)
    O, H = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh)
    R64, Roz = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert rel_err(a, b) <= 1e-9
    assert abs(a[0] - b[0]) <= 1e-8


@pytest.mark.parametrize("hL,hR", [(-1, 1), (-1, -1), (1, 1)])
def test_ozaki_matches_oracle_random_ops(gpu_lib, oracle_mod, hL, hR):
    from imsrg_gpu.synth import random_operator
    bas, lay = make_case(4)
    B = gpu_lib.Basis.from_dict(bas)
    Lh, Rh = random_operator(lay, hL, 61, 1), random_operator(lay, hR, 62, 2)
    ref = oracle_mod.Oracle(**bas).commutator(Lh, hL, Rh, hR)
    L, R, RES = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(L, R, RES, precision="ozaki")
    assert rel_err(RES.download(), ref) <= 1e-9


def test_ozaki_is_deterministic(gpu_lib):
    bas, lay, B, Hh, Oh = _pair(gpu_lib, 6, seed=9)
    O, H = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh)
    R1, R2 = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R1, precision="ozaki")
    gpu_lib.commutator(O, H, R2, precision="ozaki")
    assert np.array_equal(R1.download(), R2.download())


def test_ozaki_magnus_flow_emax2(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    orc = oracle_mod.Oracle(**bas)
    Hh = orc.normal_order(synth_hamiltonian(lay, 11))
    ref = orc.magnus_decouple(Hh, s_max=50.0, ds=0.5)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5, precision="ozaki")
    assert abs(out["trace"][-1, 2] - ref["trace"][-1, 2]) < 1e-6


def test_ozaki_magnus_flow_emax6(gpu_lib, oracle_mod):
    """emax = 6 Magnus flow to s = 50 with every two-body contraction in split
    precision: E0 within 1e-6 MeV of the FP64 GPU flow, which itself follows
    the FP64 oracle (checked here over the first steps, s <= 1)."""
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(6)
    B = gpu_lib.Basis.from_dict(bas)
    orc = oracle_mod.Oracle(**bas)
    Hh = orc.normal_order(synth_hamiltonian(lay, 13))
    flows = {}
    for prec in ("fp64", "ozaki"):
        HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
        flows[prec] = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5, precision=prec)
    t64, toz = flows["fp64"]["trace"], flows["ozaki"]["trace"]
    assert flows["fp64"]["steps"] == flows["ozaki"]["steps"] > 2
    assert abs(toz[-1, 2] - t64[-1, 2]) < 1e-6
    assert np.max(np.abs(toz[:, 2] - t64[:, 2])) < 1e-6
    ref = orc.magnus_decouple(Hh, s_max=1.0, ds=0.5)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    short = gpu_lib.magnus_decouple(HS, G, s_max=1.0, ds=0.5, precision="fp64")
    assert short["steps"] == ref["steps"]
    assert np.max(np.abs(short["trace"][:, 2] - ref["trace"][:, 2])) < 1e-8


def test_split_schedule_is_autotuned(gpu_lib):
    bas, lay, B, Hh, Oh = _pair(gpu_lib, 4)
    with pytest.raises(gpu_lib.ImsrgError):
        B.split_schedule()
    O, H, R = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R, precision="ozaki")
    choice, us = B.split_schedule()
    assert len(us) >= 2 and all(t > 0 for t in us)
    assert us[choice] == min(us)


def test_pinned_split_schedule_gives_identical_results(gpu_lib):
    """Each CTA schedule computes every tile the same way, so a commutator is
    bit-identical whichever candidate schedule is pinned."""
    bas, lay, B, Hh, Oh = _pair(gpu_lib, 4)
    O, H = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh)
    R = gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R, precision="ozaki")
    ref = R.download()
    _, us = B.split_schedule()
    for model in range(len(us)):
        B.set_split_schedule(model)
        assert B.split_schedule()[0] == model
        gpu_lib.commutator(O, H, R, precision="ozaki")
        assert np.array_equal(R.download(), ref), model
    with pytest.raises(gpu_lib.ImsrgError):
        B.set_split_schedule(len(us))


@pytest.mark.parametrize("scale", [2.0 ** -40, 2.0 ** 70, 2.0 ** 200])
def test_ozaki_any_magnitude_matches_fp64(gpu_lib, scale):
    """Operands far from MeV magnitudes: the digit scales follow each block's
    exponent, so the split path matches the FP64 path at any magnitude (a
    diverging BCH series must end as in FP64)."""
    bas, lay, B, Hh, Oh = _pair(gpu_lib, 4)
    O, H = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh * scale)
    R64, Roz = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R64, precision="fp64")
    gpu_lib.commutator(O, H, Roz, precision="ozaki")
    a, b = Roz.download(), R64.download()
    assert np.all(np.isfinite(a))
    assert rel_err(a, b) <= 1e-9
