"""Reverse-mode derivatives, through the C ABI.

* The adjoint of the commutator is the transpose of [X, .]: for consistent
  operators X, Y and any Cbar, <Cbar, [X, Y]> = <adjoint(X, Cbar), Y>, and
  by antisymmetry <Cbar, [X, Y]> = -<adjoint(Y, Cbar), X> (every Hermiticity
  pair, with and without the E0 terms).  Both sides are sums of the same
  products in different orders, so they agree to 1e-12 of the sum of the
  products' magnitudes.
* The White generator's adjoint against central differences of the generator.
* dE0/dc_k of the Magnus flow for H(c) = T + sum_k c_k V_k (four seeded
  N(0,1) MeV two-body terms, emax = 4, c = (1,1,1,1)) from ONE backward sweep,
  against central finite differences (h = 1e-4) of the oracle's FP64 flow to
  convergence (|E_mbpt2| < 1e-6, the reference's stop) and against the
  tangent-linear flow, in FP64 and split precision."""
import os

import numpy as np
import pytest

from conftest import ROOT, make_case

pytestmark = pytest.mark.gpu


def _rand_flat(lay, seed):
    return np.random.default_rng(seed).standard_normal(lay.nfull)


@pytest.mark.parametrize("emax", [2, 4])
@pytest.mark.parametrize("hX,hY", [(-1, 1), (1, 1), (-1, -1), (1, -1)])
@pytest.mark.parametrize("with_e0", [True, False])
def test_commutator_adjoint_is_the_transpose(gpu_lib, emax, hX, hY, with_e0):
    from imsrg_gpu.synth import random_operator
    bas, lay = make_case(emax)
    B = gpu_lib.Basis.from_dict(bas)
    Xh, Yh = random_operator(lay, hX, 71 + emax, 1), random_operator(lay, hY, 72 + emax, 2)
    Cb = _rand_flat(lay, 73 + emax)
    X, Y = gpu_lib.Operator(B, hX, Xh), gpu_lib.Operator(B, hY, Yh)
    RES = gpu_lib.Operator(B, 1)
    gpu_lib.commutator(X, Y, RES, precision="fp64", with_e0=with_e0)
    F = RES.download()
    CbO = gpu_lib.Operator(B, 1, Cb)
    Yb, Xb = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator_adjoint(X, CbO, hY, Yb, with_e0=with_e0)
    gpu_lib.commutator_adjoint(Y, CbO, hX, Xb, with_e0=with_e0)
    lhs = float(np.dot(Cb, F))
    rY = float(np.dot(Yb.download(), Yh))
    rX = -float(np.dot(Xb.download(), Xh))
    scale = float(np.dot(np.abs(Cb), np.abs(F))) + abs(lhs) + 1.0
    assert abs(lhs - rY) <= 1e-12 * scale, (lhs, rY)
    assert abs(lhs - rX) <= 1e-12 * scale, (lhs, rX)


def test_white_adjoint_against_central_differences(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(4)
    B = gpu_lib.Basis.from_dict(bas)
    orc = oracle_mod.Oracle(**bas)
    Hh = orc.normal_order(synth_hamiltonian(lay, 81))
    Vh = orc.normal_order(synth_hamiltonian(lay, 82, hw=0.0))
    Eb = _rand_flat(lay, 83)
    H, EbO, Hb = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1, Eb), gpu_lib.Operator(B, 1)
    gpu_lib.white_adjoint(H, EbO, Hb)
    got = float(np.dot(Hb.download(), Vh))
    h = 1e-6
    eta = []
    for sgn in (1, -1):
        ETA = gpu_lib.Operator(B, -1)
        gpu_lib.build_gs_white(gpu_lib.Operator(B, 1, Hh + sgn * h * Vh), ETA)
        eta.append(ETA.download())
    fd = float(np.dot(Eb, (eta[0] - eta[1]) / (2 * h)))
    assert abs(got - fd) <= 1e-7 * max(1.0, abs(fd)), (got, fd)


@pytest.fixture(scope="module")
def fd_case(oracle_mod):
    """The oracle's central differences of E0(s) at convergence."""
    bas, lay = make_case(4)
    orc = oracle_mod.Oracle(**bas)
    from imsrg_gpu.synth import adjoint_terms
    T, V = adjoint_terms(lay)
    c = np.ones(4)

    def H_of(cv):
        return orc.normal_order(T + sum(ck * vk for ck, vk in zip(cv, V)))

    h = 1e-4
    base = orc.magnus_decouple(H_of(c), s_max=50.0, ds=0.5)
    fd = []
    for k in range(4):
        ep = orc.magnus_decouple(H_of(c + h * np.eye(4)[k]), s_max=50.0, ds=0.5)
        em = orc.magnus_decouple(H_of(c - h * np.eye(4)[k]), s_max=50.0, ds=0.5)
        assert ep["steps"] == em["steps"] == base["steps"]
        fd.append((ep["trace"][-1, 2] - em["trace"][-1, 2]) / (2 * h))
    dirs = [orc.normal_order(v) for v in V]
    return bas, lay, H_of(c), dirs, np.array(fd), base


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_flow_adjoint_matches_oracle_finite_differences(gpu_lib, fd_case, precision):
    bas, lay, H0, dirs, fd, base = fd_case
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, -1)
    D = [gpu_lib.Operator(B, 1, d) for d in dirs]
    out = gpu_lib.magnus_decouple_adjoint(HS, G, D, s_max=50.0, ds=0.5, precision=precision)
    assert out["steps"] == base["steps"] > 10
    tol = 1e-6 if precision == "fp64" else 1e-5
    np.testing.assert_allclose(out["grad"], fd, rtol=tol, atol=tol)
    # the flow part is the plain flow
    B2 = gpu_lib.Basis.from_dict(bas)
    HSp, Gp = gpu_lib.Operator(B2, 1, H0), gpu_lib.Operator(B2, -1)
    plain = gpu_lib.magnus_decouple(HSp, Gp, s_max=50.0, ds=0.5, precision=precision)
    assert np.array_equal(out["trace"], plain["trace"])
    assert np.array_equal(HS.download(), HSp.download())


def test_flow_adjoint_equals_tangent_flow(gpu_lib, fd_case):
    """Reverse and forward mode differentiate the same discrete flow: one
    backward sweep gives every dE0/dc_k that four tangent runs give."""
    bas, lay, H0, dirs, fd, base = fd_case
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, -1)
    Hbar = gpu_lib.Operator(B, 1)
    D = [gpu_lib.Operator(B, 1, d) for d in dirs]
    adj = gpu_lib.magnus_decouple_adjoint(HS, G, D, Hbar=Hbar, s_max=50.0, ds=0.5)
    tan = []
    for d in dirs:
        HS, dHS = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, 1, d)
        G, dG = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, -1)
        tan.append(gpu_lib.magnus_decouple_tangent(HS, dHS, G, dG, s_max=50.0, ds=0.5)["dtrace"][-1, 2])
    np.testing.assert_allclose(adj["grad"], tan, rtol=1e-9, atol=1e-9)
    # the whole gradient: its dot product with each direction is grad
    hb = Hbar.download()
    np.testing.assert_allclose([np.dot(hb, d) for d in dirs], adj["grad"], rtol=1e-12, atol=1e-12)


def test_committed_fd_fixture_is_the_oracles(fd_case):
    """The oracle gradients bench.py reports the adjoint against
    (tests/golden/adjoint_fd_emax4.npz) are the oracle's central differences."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "adjoint_fd_emax4.npz"))
    np.testing.assert_allclose(g["fd"], fd_case[4], rtol=1e-9, atol=0)
    assert int(g["steps"]) == fd_case[5]["steps"]
