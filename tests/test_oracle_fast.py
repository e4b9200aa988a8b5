"""The timed CPU-baseline build of the oracle (contraction allowed, optional
external OpenBLAS dgemm) computes the same commutator as the parity build,
to rounding."""
import numpy as np

from conftest import make_case, rel_err


def test_fast_build_matches_parity_build(oracle_mod):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay = make_case(4)
    Hh, Oh = synth_hamiltonian(lay, 3), synth_omega(lay, 3)
    ref = oracle_mod.Oracle(**bas).commutator(Oh, -1, Hh, 1)
    fast = oracle_mod.Oracle(**bas, variant="fast")
    try:
        assert rel_err(fast.commutator(Oh, -1, Hh, 1), ref) <= 1e-13
        if oracle_mod.use_blas(2) is not None:
            assert rel_err(fast.commutator(Oh, -1, Hh, 1), ref) <= 1e-13
    finally:
        oracle_mod.lib("fast").orc_set_dgemm(None)
