"""White generator, norms, mbpt2, Magnus/BCH series and the full Magnus
flow on the GPU against the oracle."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def _setup(gpu_lib, oracle_mod, emax):
    bas, lay = make_case(emax)
    return bas, lay, gpu_lib.Basis.from_dict(bas), oracle_mod.Oracle(**bas)


@pytest.mark.parametrize("emax", [2, 4])
def test_norm_add_mbpt2(gpu_lib, oracle_mod, emax):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, emax)
    Hh, Oh = synth_hamiltonian(lay, 3), synth_omega(lay, 3)
    H, O, C = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1)
    assert gpu_lib.mat_frob_norm(H) == pytest.approx(orc.norm(Hh), rel=1e-13)
    assert gpu_lib.mbpt2(H) == pytest.approx(orc.mbpt2(Hh), rel=1e-12)
    gpu_lib.add_sq_op(H, 0.5, O, -2.0, C)
    assert rel_err(C.download(), orc.add(Hh, 0.5, Oh, -2.0)) <= 1e-15
    gpu_lib.copy_sq_op(O, C)
    assert C.herm == -1 and np.array_equal(C.download(), Oh)
    gpu_lib.clear_sq_op(C)
    assert not C.download().any()


@pytest.mark.parametrize("emax", [2, 4])
def test_white_generator(gpu_lib, oracle_mod, emax):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, emax)
    Hh = orc.normal_order(synth_hamiltonian(lay, 4))
    H, ETA = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.build_gs_white(H, ETA)
    assert ETA.herm == -1
    assert rel_err(ETA.download(), orc.white(Hh)) <= 1e-12


def test_magnus_and_bch_series(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 4)
    Hh = orc.normal_order(synth_hamiltonian(lay, 6))
    Gh = synth_omega(lay, 6)
    eta = orc.white(Hh)
    dg_ref, n_ref = orc.magnus_expand(eta, Gh)
    G, DG = gpu_lib.Operator(B, -1, Gh), gpu_lib.Operator(B, -1, eta)
    n = gpu_lib.magnus_expand(DG, G)
    assert n == n_ref
    assert rel_err(DG.download(), dg_ref) <= 1e-10
    hs_ref, nb_ref = orc.bch_expand(Gh, Hh)
    H, HS = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    nb = gpu_lib.bch_expand(HS, G, H)
    assert nb == nb_ref
    assert rel_err(HS.download(), hs_ref) <= 1e-10
    s = gpu_lib.euler_step(G, DG, 1.0, 0.5)
    assert s == 1.5
    assert rel_err(G.download(), orc.add(Gh, 1.0, dg_ref, 0.5)) <= 1e-10


def test_magnus_flow_emax2(gpu_lib, oracle_mod):
    """Magnus flow with the White generator to s = 50 (4He, emax = 2)."""
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 2)
    Hh = orc.normal_order(synth_hamiltonian(lay, 11))
    ref = orc.magnus_decouple(Hh, s_max=50.0, ds=0.5)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5)
    assert out["steps"] == ref["steps"]
    assert abs(out["trace"][-1, 2] - ref["trace"][-1, 2]) < 1e-6  # E0 in MeV
    np.testing.assert_allclose(out["trace"][:, 2], ref["trace"][:, 2], rtol=0, atol=1e-6)
    assert rel_err(HS.download(), ref["H"]) <= 1e-8
