"""Committed golden fixtures (tests/golden/make_golden.py, from the oracle):
the oracle must keep reproducing them (CPU), and the GPU path must match them
(GPU, through the C ABI)."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_err

G = np.load(os.path.join(ROOT, "tests", "golden", "emax2_golden.npz"))
BAS = {k: G[k] for k in ("nn", "ll", "jj", "itzp", "con")}


def test_oracle_reproduces_golden(oracle_mod):
    orc = oracle_mod.Oracle(**BAS)
    assert rel_err(orc.commutator(G["Omega"], -1, G["H"], 1), G["comm"]) <= 1e-13
    assert rel_err(orc.commutator(G["A"], -1, G["B"], 1), G["commAB"]) <= 1e-13
    assert rel_err(orc.white(G["H"]), G["eta"]) <= 1e-13
    hs, n = orc.bch_expand(G["Omega"], G["H"])
    assert n == int(G["nbch"]) and rel_err(hs, G["bch"]) <= 1e-12
    flow = orc.magnus_decouple(G["H"], s_max=50.0, ds=0.5)
    np.testing.assert_allclose(flow["trace"], G["flow_trace"], rtol=0, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_gpu_matches_golden(gpu_lib, precision):
    tol = 1e-10 if precision == "fp64" else 1e-9
    B = gpu_lib.Basis.from_dict(BAS)
    O, H, R = gpu_lib.Operator(B, -1, G["Omega"]), gpu_lib.Operator(B, 1, G["H"]), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R, precision=precision)
    assert rel_err(R.download(), G["comm"]) <= tol
    A, Bo = gpu_lib.Operator(B, -1, G["A"]), gpu_lib.Operator(B, 1, G["B"])
    gpu_lib.commutator(A, Bo, R, precision=precision)
    assert rel_err(R.download(), G["commAB"]) <= tol
    ETA = gpu_lib.Operator(B, -1)
    gpu_lib.build_gs_white(H, ETA)
    assert rel_err(ETA.download(), G["eta"]) <= 1e-12
    HS, Gm = gpu_lib.Operator(B, 1, G["H"]), gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple(HS, Gm, s_max=50.0, ds=0.5, precision=precision)
    np.testing.assert_allclose(out["trace"][:, 2], G["flow_trace"][:, 2], rtol=0, atol=1e-6)
