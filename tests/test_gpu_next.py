"""Callers and formats beside the commutator path: checkpoint files (the
vectorize stream), normal ordering on the device, dHds for an external ODE
solver, and the observable BCH transformation, each against the oracle."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def _case(gpu_lib, oracle_mod, emax, seed):
    from imsrg_gpu.synth import synth_hamiltonian, random_operator
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(**bas)
    return bas, lay, orc, synth_hamiltonian(lay, seed)


@pytest.mark.parametrize("herm", [1, -1])
def test_checkpoint_file_is_the_vectorize_stream(gpu_lib, oracle_mod, tmp_path, herm):
    from imsrg_gpu.synth import random_operator
    bas, lay = make_case(4)
    orc = oracle_mod.Oracle(**bas)
    X = random_operator(lay, herm, 41, 1)
    B = gpu_lib.Basis.from_dict(bas)
    op = gpu_lib.Operator(B, herm, X)
    path = tmp_path / "O16_hw20_s2.5000.bin"
    op.save(path)
    raw = path.read_bytes()
    assert raw == orc.vectorize(X).astype("<f8").tobytes()
    back = gpu_lib.Operator(B, herm)
    back.load(path)
    assert np.array_equal(back.download(), X)


def test_checkpoint_load_rejects_wrong_length(gpu_lib, tmp_path):
    bas, lay = make_case(2)
    B = gpu_lib.Basis.from_dict(bas)
    op = gpu_lib.Operator(B, 1)
    bad = tmp_path / "short.bin"
    bad.write_bytes(np.zeros(10).tobytes())
    with pytest.raises(gpu_lib.ImsrgError):
        op.load(bad)
    with pytest.raises(gpu_lib.ImsrgError):
        op.load(tmp_path / "missing.bin")


@pytest.mark.parametrize("emax", [2, 4])
def test_normal_order_matches_oracle(gpu_lib, oracle_mod, emax):
    bas, lay, orc, Hh = _case(gpu_lib, oracle_mod, emax, 51)
    B = gpu_lib.Basis.from_dict(bas)
    H = gpu_lib.Operator(B, 1, Hh)
    gpu_lib.normal_order(H)
    assert rel_err(H.download(), orc.normal_order(Hh)) <= 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("ozaki", 1e-9)])
def test_dhds_matches_oracle(gpu_lib, oracle_mod, precision, tol):
    bas, lay, orc, Hh = _case(gpu_lib, oracle_mod, 4, 52)
    Hh = orc.normal_order(Hh)
    B = gpu_lib.Basis.from_dict(bas)
    HS, DH = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.dhds(HS, DH, "white", precision)
    ref = orc.commutator(orc.white(Hh), -1, Hh, 1)
    assert rel_err(DH.download(), ref) <= tol


def test_observable_bch_matches_oracle(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import random_operator, synth_omega
    bas, lay = make_case(4)
    orc = oracle_mod.Oracle(**bas)
    Oh = random_operator(lay, 1, 53, 1)
    Gh = synth_omega(lay, 54)
    refHS, _ = orc.bch_expand(Gh, Oh)
    B = gpu_lib.Basis.from_dict(bas)
    Op, G = gpu_lib.Operator(B, 1, Oh), gpu_lib.Operator(B, -1, Gh)
    gpu_lib.transform_bch(Op, G)
    assert rel_err(Op.download(), refHS) <= 1e-10
