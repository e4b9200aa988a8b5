"""The setup steps on the GPU library against the oracle's restatement: the
ASCII interaction file with its centre-of-mass / Lawson terms
(read_interaction), the HO one-body part (calculate_h0_harm_osc) and
Hartree-Fock (calc_HF), then the full pipeline file -> h0 -> HF -> Magnus
flow as main_IMSRG.f90 runs it."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def _both(gpu_lib, oracle_mod, emax):
    from oracle.hf import Setup
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(bas["nn"], bas["ll"], bas["jj"], bas["itzp"], bas["con"])
    S = Setup(orc, bas["nn"], bas["ll"], bas["jj"], bas["itzp"], bas["con"])
    return S, orc, lay, gpu_lib.Basis.from_dict(bas)


def _file(lay, path, seed=5, sigma2=0.5):
    from imsrg_gpu.synth import synth_hamiltonian, write_vrenorm
    V = synth_hamiltonian(lay, seed, sigma2=sigma2)
    V[:lay.off_fpp + lay.P * lay.P] = 0.0
    write_vrenorm(lay, V, path, seed=seed)
    return V


@pytest.mark.parametrize("htype,beta", [(1, 0.0), (1, 0.4), (2, 0.0), (3, 0.0)])
def test_read_interaction_matches_oracle(gpu_lib, oracle_mod, tmp_path, htype, beta):
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 4)
    path = str(tmp_path / "v.int")
    _file(lay, path)
    ref = S.read_interaction(path, htype=htype, hw=20.0, com_hw=18.0, lawson_beta=beta, mass=16)
    H = gpu_lib.Operator(B, 1, np.full(lay.nfull, 7.0))  # the reader clears it first
    gpu_lib.read_interaction(H, path, htype=htype, hw=20.0, com_hw=18.0, lawson_beta=beta, mass=16)
    got = H.download()
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    if htype == 3 or (htype == 2 and beta == 0.0):  # no centre-of-mass terms: the file's values exactly
        assert np.count_nonzero(got) == np.count_nonzero(ref)


def test_read_interaction_errors(gpu_lib, oracle_mod, tmp_path):
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 2)
    H = gpu_lib.Operator(B, 1)
    with pytest.raises(gpu_lib.ImsrgError):  # no such file
        gpu_lib.read_interaction(H, str(tmp_path / "missing.int"))
    bad = tmp_path / "bad.int"
    bad.write_text("\n" * 8 + "0 0 0 1 2 x 4 1.0\n")
    with pytest.raises(gpu_lib.ImsrgError):  # malformed line
        gpu_lib.read_interaction(H, str(bad))
    wrong = tmp_path / "wrong.int"
    wrong.write_text("\n" * 8 + "0 1 0 1 2 1 2 1.0\n")  # orbits 1, 2 (0s p, 0s n) have parity 0
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.read_interaction(H, str(wrong))
    with pytest.raises(gpu_lib.ImsrgError):  # anti-Hermitian target
        gpu_lib.read_interaction(gpu_lib.Operator(B, -1), str(bad))


@pytest.mark.parametrize("htype,beta", [(1, 0.0), (1, 0.3), (2, 0.0), (3, 0.0), (4, 0.0), (5, 0.0)])
def test_h0_matches_oracle(gpu_lib, oracle_mod, htype, beta):
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 4)
    rng = np.random.default_rng(1)
    start = rng.normal(size=lay.nfull)
    ref = S.h0_harm_osc(start, htype=htype, hw=20.0, com_hw=17.0, lawson_beta=beta, mass=16)
    H = gpu_lib.Operator(B, 1, start)
    gpu_lib.h0_harm_osc(H, htype=htype, hw=20.0, com_hw=17.0, lawson_beta=beta, mass=16)
    # the host compiler may contract a*b + c*d into a fused multiply-add
    np.testing.assert_allclose(H.download(), ref, rtol=1e-14, atol=0)


@pytest.mark.parametrize("emax", [2, 4])
def test_hartree_fock_matches_oracle(gpu_lib, oracle_mod, tmp_path, emax):
    S, orc, lay, B = _both(gpu_lib, oracle_mod, emax)
    path = str(tmp_path / "v.int")
    _file(lay, path)
    H0 = S.h0_harm_osc(S.read_interaction(path, htype=1, hw=20.0, mass=16), htype=1, hw=20.0, mass=16)
    ref, ehf, D, it = S.hartree_fock(H0, tol=1e-6)
    H = gpu_lib.Operator(B, 1)
    gpu_lib.read_interaction(H, path, htype=1, hw=20.0, mass=16)
    gpu_lib.h0_harm_osc(H, htype=1, hw=20.0, mass=16)
    assert rel_err(H.download(), H0) <= 1e-12
    out = gpu_lib.hartree_fock(H, tol=1e-6)
    assert out["iterations"] == it
    assert out["e_hf"] == pytest.approx(ehf, abs=1e-9)
    assert np.max(np.abs(out["coefs"] - D)) <= 1e-9
    assert rel_err(H.download(), ref) <= 1e-10


def test_hartree_fock_then_flow(gpu_lib, oracle_mod, tmp_path):
    """main_IMSRG.f90's pipeline: file -> h0 -> HF -> Magnus flow (White
    generator) to s = 50, E0 within 1e-6 MeV of the oracle's pipeline."""
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 2)
    path = str(tmp_path / "v.int")
    _file(lay, path, sigma2=1.0)
    H0 = S.h0_harm_osc(S.read_interaction(path, htype=1, hw=20.0, mass=4), htype=1, hw=20.0, mass=4)
    hf_ref, ehf, _, _ = S.hartree_fock(H0)
    ref = orc.magnus_decouple(hf_ref, s_max=50.0, ds=0.5)
    HS, G = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, -1)
    gpu_lib.read_interaction(HS, path, htype=1, hw=20.0, mass=4)
    gpu_lib.h0_harm_osc(HS, htype=1, hw=20.0, mass=4)
    res = gpu_lib.hartree_fock(HS)
    assert res["e_hf"] == pytest.approx(ehf, abs=1e-9)
    out = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5)
    assert out["steps"] == ref["steps"]
    assert abs(out["trace"][-1, 2] - ref["trace"][-1, 2]) < 1e-6


def test_hartree_fock_not_converged(gpu_lib, oracle_mod, tmp_path):
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 2)
    path = str(tmp_path / "v.int")
    _file(lay, path)
    H = gpu_lib.Operator(B, 1)
    gpu_lib.read_interaction(H, path, mass=4)
    gpu_lib.h0_harm_osc(H, mass=4)
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.hartree_fock(H, tol=1e-6, max_iter=1)
    assert e.value.status == 4  # IMSRG_ERR_NOT_CONVERGED


def test_transform_to_hf_matches_oracle_and_hf(gpu_lib, oracle_mod, tmp_path):
    """observable_to_HF: a second Hermitian operator in the HF basis equals the
    oracle's; the bare Hamiltonian transformed with the HF coefficients gives
    back what hartree_fock left (two-body part bit for bit, E0 and the Fock
    matrix to the convergence of the iteration)."""
    from imsrg_gpu.synth import synth_hamiltonian
    S, orc, lay, B = _both(gpu_lib, oracle_mod, 4)
    path = str(tmp_path / "v.int")
    _file(lay, path)
    H = gpu_lib.Operator(B, 1)
    gpu_lib.read_interaction(H, path, htype=1, hw=20.0, mass=16)
    gpu_lib.h0_harm_osc(H, htype=1, hw=20.0, mass=16)
    bare = H.download()
    res = gpu_lib.hartree_fock(H, tol=1e-11)
    hf = H.download()
    X = gpu_lib.Operator(B, 1, bare)
    gpu_lib.transform_to_hf(X, res["coefs"])
    got = X.download()
    two = lay.off_fpp + lay.P * lay.P
    assert np.array_equal(got[two:], hf[two:])
    assert got[0] == pytest.approx(hf[0], abs=1e-8)
    assert np.max(np.abs(got[1:two] - hf[1:two])) <= 1e-8 * np.max(np.abs(hf))
    obs = synth_hamiltonian(lay, 77, hw=0.0, sigma1=0.3, sigma2=0.2)  # some other Hermitian scalar operator
    Y = gpu_lib.Operator(B, 1, obs)
    gpu_lib.transform_to_hf(Y, res["coefs"])
    ref = S.transform_to_hf(obs, res["coefs"])
    assert rel_err(Y.download(), ref) <= 1e-11
