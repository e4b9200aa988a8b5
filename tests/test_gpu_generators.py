"""atan and w2 generators (generators.f90:109-376) and flows driven by them,
against the oracle."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def _setup(gpu_lib, oracle_mod, emax, seed):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(**bas)
    H = orc.normal_order(synth_hamiltonian(lay, seed))
    return bas, orc, H


@pytest.mark.parametrize("emax", [2, 4])
def test_atan_generator_matches_oracle(gpu_lib, oracle_mod, emax):
    bas, orc, Hh = _setup(gpu_lib, oracle_mod, emax, 31)
    B = gpu_lib.Basis.from_dict(bas)
    H, ETA = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1, np.zeros_like(Hh))
    gpu_lib.build_gs_atan(H, ETA)
    assert rel_err(ETA.download(), orc.atan_gen(Hh)) <= 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("ozaki", 1e-9)])
def test_w2_generator_matches_oracle(gpu_lib, oracle_mod, precision, tol):
    bas, orc, Hh = _setup(gpu_lib, oracle_mod, 4, 32)
    B = gpu_lib.Basis.from_dict(bas)
    H, ETA = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1, np.zeros_like(Hh))
    gpu_lib.build_gs_w2(H, ETA, precision=precision)
    assert rel_err(ETA.download(), orc.w2_gen(Hh)) <= tol


@pytest.mark.parametrize("generator", ["atan", "w2"])
def test_flow_with_generator_matches_oracle(gpu_lib, oracle_mod, generator):
    bas, orc, Hh = _setup(gpu_lib, oracle_mod, 2, 33)
    ref = orc.magnus_decouple_gen(Hh, generator, s_max=50.0, ds=0.5)
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple_gen(HS, G, generator, s_max=50.0, ds=0.5)
    assert out["steps"] == ref["steps"]
    assert np.max(np.abs(out["trace"][:, 2] - ref["trace"][:, 2])) < 1e-8


def test_white_generator_flow_is_the_default(gpu_lib, oracle_mod):
    bas, orc, Hh = _setup(gpu_lib, oracle_mod, 2, 34)
    B = gpu_lib.Basis.from_dict(bas)
    a = gpu_lib.magnus_decouple_gen(gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1), "white", s_max=5.0)
    b = gpu_lib.magnus_decouple(gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1), s_max=5.0)
    assert np.array_equal(a["trace"], b["trace"])
