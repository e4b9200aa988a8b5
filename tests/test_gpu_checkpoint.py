"""Omega checkpoints inside the Magnus flow (IMSRG_MAGNUS.f90:56-110,
basic_IMSRG.f90:3132-3312): a flow stopped on the host after some steps and
started again from its newest checkpoint file takes the uninterrupted flow's
steps and reproduces its trace, H(s) and Omega(s), in both precisions and on
both the host-driven and the graph-captured step; the write period, the
removal of the checkpoint 12 units of s back and the 'testcase' prefix follow
the reference.

H(s) and Omega(s) agree to rounding, not bit for bit: the checkpoint format
(vectorize) keeps the upper triangle of each square array, and repackage
(basic_IMSRG.f90:3906-3911) writes its diagonal as herm x the stored value.
The flow leaves rounding residue (about 1e-25 here) on the diagonals of the
anti-Hermitian Omega, which is mathematically zero there, so it comes back
from the file with the opposite sign, as in the reference."""
import os

import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu
PREFIX = "O16_e4_hw20_chk"


def _hamiltonian(oracle_mod, emax=4, seed=13):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(emax)
    return bas, lay, oracle_mod.Oracle(**bas).normal_order(synth_hamiltonian(lay, seed))


def _name(gpu_lib, d, s):
    return gpu_lib.checkpoint_name(d, PREFIX, s)


@pytest.mark.parametrize("precision,graph", [("fp64", False), ("fp64", True), ("ozaki", False), ("ozaki", True)])
def test_restart_continues_the_flow(gpu_lib, oracle_mod, tmp_path, precision, graph):
    bas, lay, Hh = _hamiltonian(oracle_mod)
    d = str(tmp_path) + os.sep
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    full = (gpu_lib.magnus_decouple_graph if graph else gpu_lib.magnus_decouple)(HS, G, s_max=50.0, ds=0.5,
                                                                                   precision=precision)
    H_full, G_full = HS.download(), G.download()
    assert full["steps"] > 12

    # the same flow with checkpoints every 4 steps, stopped after 10 steps
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    a = gpu_lib.magnus_decouple_checkpoint(HS, G, d, PREFIX, chk=4, max_steps=10, precision=precision,
                                           graph=graph)
    assert a["steps"] == 10 and a["s_restart"] == -1.0
    assert np.array_equal(a["trace"], full["trace"][:11])
    # Omega was written before the Magnus steps 4 and 8, at s = 1.5 and 3.5
    assert sorted(os.listdir(tmp_path)) == sorted(os.path.basename(_name(gpu_lib, d, s)) for s in (1.5, 3.5))

    # a new run from the unevolved H restarts from the newest file
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    b = gpu_lib.magnus_decouple_checkpoint(HS, G, d, PREFIX, chk=4, precision=precision, graph=graph)
    assert b["s_restart"] == 3.5
    assert b["steps"] == full["steps"]
    np.testing.assert_allclose(b["trace"][8:], full["trace"][8:], rtol=0, atol=1e-10)
    for got, want in ((HS.download(), H_full), (G.download(), G_full)):
        assert np.max(np.abs(got - want)) <= 1e-13 * np.max(np.abs(want))


def test_old_checkpoints_removed_and_testcase_prefix(gpu_lib, oracle_mod, tmp_path):
    bas, lay, Hh = _hamiltonian(oracle_mod)
    d = str(tmp_path) + os.sep
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    gpu_lib.magnus_decouple(HS, G, s_max=2.0, ds=0.5)
    # a checkpoint at s = 20 (restart: step counter 40) and an older one at
    # s = 11.5, which the write at s = 23.5 (step 48) removes
    G.save(_name(gpu_lib, d, 20.0))
    G.save(_name(gpu_lib, d, 11.5))
    HS = gpu_lib.Operator(B, 1, Hh)
    G2 = gpu_lib.Operator(B, -1)
    out = gpu_lib.magnus_decouple_checkpoint(HS, G2, d, PREFIX, chk=4, max_steps=48)
    assert out["s_restart"] == 20.0 and out["steps"] == 48
    # step 44 was the first write due after the restart (skipped), step 48 wrote s = 23.5
    assert sorted(os.listdir(tmp_path)) == sorted(os.path.basename(_name(gpu_lib, d, s)) for s in (20.0, 23.5))
    # 'testcase' runs neither read nor write checkpoints
    HS, G3 = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    t = gpu_lib.magnus_decouple_checkpoint(HS, G3, d, "testcase_hw20", chk=1, max_steps=3)
    assert t["s_restart"] == -1.0 and t["steps"] == 3
    assert len(os.listdir(tmp_path)) == 2


def test_reference_rules(gpu_lib_cpu):
    """ds and chk of magnus_decouple (IMSRG_MAGNUS.f90:45-62); host only."""
    from imsrg_gpu.layout import ho_basis
    B = gpu_lib_cpu.Basis.from_dict(ho_basis(4))
    assert gpu_lib_cpu.magnus_rules(B, 0.0) == (0.5, 24)
    assert gpu_lib_cpu.magnus_rules(B, 5.9) == (0.5, 24)
    assert gpu_lib_cpu.magnus_rules(B, 6.0) == (0.1, 24)
