"""The ODE flow (decouple_hamiltonian with the Shampine-Gordon solver,
IMSRG_ODE.f90:9-178, adams_ode.f90) on the device against the oracle's
restatement of the same solver."""
import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu


def _case(oracle_mod, emax, seed):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(**bas)
    return bas, orc, orc.normal_order(synth_hamiltonian(lay, seed))


def test_ode_flow_to_convergence_matches_oracle(gpu_lib, oracle_mod):
    from oracle.sg_ode import decouple_hamiltonian
    bas, orc, Hh = _case(oracle_mod, 2, 21)
    ref = decouple_hamiltonian(orc, Hh)
    B = gpu_lib.Basis.from_dict(bas)
    HS = gpu_lib.Operator(B, 1, Hh)
    out = gpu_lib.ode_decouple(HS)
    assert out["steps"] == ref["steps"]
    assert out["nfev"] == ref["nfev"]
    assert out["trace"][-1, 4] < 1e-6
    # same step sequence: E0 along the flow to solver round-off
    assert np.max(np.abs(out["trace"][:, 2] - ref["trace"][:, 2])) < 1e-9
    assert np.max(np.abs(HS.download() - ref["H"])) < 1e-9


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("ozaki", 1e-7)])
def test_ode_flow_emax4_matches_oracle(gpu_lib, oracle_mod, precision, tol):
    from oracle.sg_ode import decouple_hamiltonian
    bas, orc, Hh = _case(oracle_mod, 4, 22)
    ref = decouple_hamiltonian(orc, Hh, s_max=0.5)
    B = gpu_lib.Basis.from_dict(bas)
    HS = gpu_lib.Operator(B, 1, Hh)
    out = gpu_lib.ode_decouple(HS, precision=precision, s_max=0.5)
    assert out["steps"] == ref["steps"] == 5
    assert np.max(np.abs(out["trace"][:, 2] - ref["trace"][:, 2])) < tol


def test_ode_flow_agrees_with_magnus_flow(gpu_lib, oracle_mod):
    """Both flows decouple the same Hamiltonian: their converged E0 differ
    only by the truncation the Magnus expansion adds (a small fraction of the
    correlation energy)."""
    bas, orc, Hh = _case(oracle_mod, 2, 23)
    B = gpu_lib.Basis.from_dict(bas)
    a = gpu_lib.ode_decouple(gpu_lib.Operator(B, 1, Hh))
    m = gpu_lib.magnus_decouple(gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1), s_max=50.0)
    e_ode, e_mag, e_ref = a["trace"][-1, 2], m["trace"][-1, 2], Hh[0]
    assert abs(e_ode - e_mag) < 0.05 * abs(e_ref - e_ode) + 1e-3


def test_ode_rejects_bad_input(gpu_lib, oracle_mod):
    bas, orc, Hh = _case(oracle_mod, 2, 24)
    B = gpu_lib.Basis.from_dict(bas)
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.ode_decouple(gpu_lib.Operator(B, -1, Hh))
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.ode_decouple(gpu_lib.Operator(B, 1, Hh), ds=0.0)
