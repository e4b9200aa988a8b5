"""Parity at the benchmark's own configuration, element by element, against
the oracle (the C restatement of commutators.f90:10-925,
cross_coupled.f90:1190-1300 and IMSRG_MAGNUS.f90:15-234).

Element-wise bar: every element satisfies
    |gpu_i - oracle_i| <= tol * |oracle_i| + floor * max|oracle|
with tol = 1e-10 (the plain path's 1e-10 relative on matrix elements) and
floor = 1e-14 for FP64; a floor absorbs elements that are sums of much larger
terms of opposite sign, whose rounding depends on the summation order.  The
split path truncates every product at about 2^-(7S) K max|A| max|B| (S digits
per operand, K the contraction length), so its floor is that bound over the
result's scale: 2e-11 (six digits) and 1e-9 (five digits); at the FP64-class
seven and eight digits (every level exact) 2e-13 and FP64's own 1e-14.

The flow checks follow the reference's own acceptance: E0 within 1e-6 MeV of
the FP64 oracle at every Magnus step, and the Magnus operator Omega(s) close
to the oracle's (its norm, as mat_frob_norm, basic_IMSRG.f90:3921-3952, to
1e-8 relative in FP64 and 1e-6 split)."""
import os

import numpy as np
import pytest

from conftest import ROOT, elem_err, make_case

pytestmark = pytest.mark.gpu

FP64_TOL, FP64_FLOOR = 1e-10, 1e-14
SPLIT_FLOOR = {8: 1e-14, 7: 2e-13, 6: 2e-11, 5: 1e-9}


@pytest.fixture(scope="module")
def emax6(gpu_lib, oracle_mod):
    """The benchmark's step: [Omega, H] at emax = 6 (16O, 56 j-orbits) on the
    seed-1 synthetic operators, with the oracle's result."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    oracle_mod.set_threads(os.cpu_count())
    bas, lay = make_case(6)
    Hh, Oh = synth_hamiltonian(lay, 1), synth_omega(lay, 1)
    ref = oracle_mod.Oracle(**bas).commutator(Oh, -1, Hh, 1)
    return bas, lay, Hh, Oh, ref


def test_emax6_fp64_elementwise(gpu_lib, emax6):
    bas, lay, Hh, Oh, ref = emax6
    B = gpu_lib.Basis.from_dict(bas)
    O, H, RES = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, RES, precision="fp64")
    got = RES.download()
    ratio, worst = elem_err(got, ref, FP64_TOL, FP64_FLOOR)
    print(f"emax6 fp64: bound ratio {ratio:.3e}, worst element rel err {worst:.3e}, "
          f"|dE0| {abs(got[0] - ref[0]):.3e} MeV")
    assert ratio <= 1.0
    assert abs(got[0] - ref[0]) <= FP64_TOL * abs(ref[0])


@pytest.mark.parametrize("digits", [8, 7, 6, 5])
def test_emax6_split_elementwise(gpu_lib, emax6, digits):
    bas, lay, Hh, Oh, ref = emax6
    B = gpu_lib.Basis.from_dict(bas)
    B.set_split_digits(digits)
    O, H, RES = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, RES, precision="ozaki")
    got = RES.download()
    ratio, worst = elem_err(got, ref, FP64_TOL, SPLIT_FLOOR[digits])
    print(f"emax6 split S={digits}: bound ratio {ratio:.3e}, worst element rel err {worst:.3e}, "
          f"|dE0| {abs(got[0] - ref[0]):.3e} MeV")
    assert ratio <= 1.0
    assert abs(got[0] - ref[0]) < 1e-6


@pytest.mark.parametrize("hL,hR", [(-1, 1), (1, 1), (-1, -1), (1, -1)])
def test_emax4_fp64_elementwise(gpu_lib, oracle_mod, hL, hR):
    """emax = 4 (60 orbits in the 2j-degenerate count, 30 j-orbits, 16O):
    the single-commutator configuration with the element-wise 1e-10 check,
    for the benchmark distributions and every Hermiticity pair."""
    from imsrg_gpu.synth import random_operator, synth_hamiltonian, synth_omega
    bas, lay = make_case(4)
    B = gpu_lib.Basis.from_dict(bas)
    orc = oracle_mod.Oracle(**bas)
    if (hL, hR) == (-1, 1):
        Lh, Rh = synth_omega(lay, 4), synth_hamiltonian(lay, 4)
    else:
        Lh, Rh = random_operator(lay, hL, 51, 1), random_operator(lay, hR, 52, 2)
    ref = orc.commutator(Lh, hL, Rh, hR)
    L, R, RES = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(L, R, RES, precision="fp64")
    ratio, worst = elem_err(RES.download(), ref, FP64_TOL, FP64_FLOOR)
    print(f"emax4 fp64 ({hL},{hR}): bound ratio {ratio:.3e}, worst element rel err {worst:.3e}")
    assert ratio <= 1.0


@pytest.fixture(scope="module")
def flow6(gpu_lib, oracle_mod):
    """The emax = 6 Magnus flow to s = 50 (ds = 0.5, White generator) of the
    normal-ordered seed-13 Hamiltonian, run by the oracle once."""
    from imsrg_gpu.synth import synth_hamiltonian
    oracle_mod.set_threads(os.cpu_count())
    bas, lay = make_case(6)
    orc = oracle_mod.Oracle(**bas)
    Hh = orc.normal_order(synth_hamiltonian(lay, 13))
    ref = orc.magnus_decouple(Hh, s_max=50.0, ds=0.5)
    ref["omega_norm"] = orc.norm(ref["Omega"])
    return bas, lay, Hh, ref


def test_oracle_flow_matches_committed_trace(flow6):
    """The committed emax = 6 flow fixture (the benchmark compares its GPU
    flows with it) is the oracle's flow."""
    bas, lay, Hh, ref = flow6
    g = np.load(os.path.join(ROOT, "tests", "golden", "emax6_flow.npz"))
    assert int(g["steps"]) == ref["steps"]
    np.testing.assert_allclose(g["trace"], ref["trace"], rtol=0, atol=1e-9)
    assert abs(float(g["omega_norm"]) - ref["omega_norm"]) <= 1e-10 * ref["omega_norm"]


@pytest.mark.parametrize("precision,digits", [("fp64", None), ("ozaki", 5), ("ozaki", 6), ("ozaki", 8)])
def test_emax6_flow_against_oracle(gpu_lib, flow6, precision, digits):
    bas, lay, Hh, ref = flow6
    B = gpu_lib.Basis.from_dict(bas)
    if digits:
        B.set_split_digits(digits)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple(HS, G, s_max=50.0, ds=0.5, precision=precision)
    assert out["steps"] == ref["steps"] > 20
    assert out["ncomm"] == ref["ncomm"]
    de0 = np.abs(out["trace"][:, 2] - ref["trace"][:, 2])
    dnorm = abs(gpu_lib.mat_frob_norm(G) - ref["omega_norm"]) / ref["omega_norm"]
    ratio, worst = elem_err(G.download(), ref["Omega"], 1e-6, 1e-8)
    print(f"emax6 flow {precision} S={digits}: max |dE0| {de0.max():.3e} MeV over {out['steps']} steps, "
          f"|Omega| rel err {dnorm:.3e}, Omega element bound ratio {ratio:.3e}, worst rel {worst:.3e}")
    assert de0.max() < 1e-6
    assert dnorm < (1e-8 if precision == "fp64" or digits == 8 else 1e-6)
    assert ratio <= 1.0


def test_emax6_graph_flow_equals_host_flow(gpu_lib, flow6):
    """The graph-captured flow (the benchmark's flow) at emax = 6 is the
    host-driven flow bit for bit, in both precisions."""
    bas, lay, Hh, ref = flow6
    for precision in ("fp64", "ozaki"):
        outs = []
        for fn in (gpu_lib.magnus_decouple, gpu_lib.magnus_decouple_graph):
            B = gpu_lib.Basis.from_dict(bas)
            B.set_split_digits(5)
            HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
            o = fn(HS, G, s_max=50.0, ds=0.5, precision=precision)
            o["H"], o["Omega"] = HS.download(), G.download()
            outs.append(o)
        host, graph = outs
        assert graph["steps"] == host["steps"] == ref["steps"]
        assert graph["ncomm"] == host["ncomm"]
        assert np.array_equal(graph["trace"], host["trace"]), precision
        assert np.array_equal(graph["H"], host["H"]), precision
        assert np.array_equal(graph["Omega"], host["Omega"]), precision
