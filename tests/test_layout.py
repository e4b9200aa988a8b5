"""Host layout (numpy restatement) against the oracle's layout, and the
vectorize/repackage format of basic_IMSRG.f90:3794-3918."""
import numpy as np
import pytest

from conftest import make_case


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_layout_matches_oracle(oracle_mod, emax):
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(**bas)
    assert orc.nfull == lay.nfull and orc.neq == lay.neq and orc.nblocks == lay.nblocks
    assert (orc.block_dims() == lay.block_dims()).all()
    for q in range(1, lay.nblocks + 1):
        for c in (1, 2, 3):
            assert (orc.block_qn(q, c) == lay.blocks[q - 1].qn[c - 1]).all()


def test_reference_sizes():
    """Orbit counts and block sizes of the 4He/16O bases (reference counting)."""
    for emax, norb, nh, nblocks, neq in ((2, 12, 2, 36, 1149), (4, 30, 6, 60, 37183), (6, 56, 6, 84, 485221)):
        bas, lay = make_case(emax)
        assert (lay.norb, lay.A, lay.nblocks, lay.neq) == (norb, nh, nblocks, neq)
    bas, lay = make_case(6)
    d = lay.block_dims()
    assert (d[:, 3].max(), d[:, 4].max(), d[:, 5].max()) == (232, 42, 5)


@pytest.mark.parametrize("herm", [1, -1])
def test_vectorize_roundtrip(oracle_mod, herm):
    from imsrg_gpu.synth import random_operator
    bas, lay = make_case(4)
    orc = oracle_mod.Oracle(**bas)
    op = random_operator(lay, herm, 9)
    v = lay.vectorize(op)
    np.testing.assert_array_equal(v, orc.vectorize(op))
    np.testing.assert_array_equal(lay.repackage(v, herm), orc.repackage(v, herm))
    np.testing.assert_array_equal(lay.repackage(v, herm), op)
