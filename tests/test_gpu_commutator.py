"""GPU commutator against the oracle, through the C ABI (FP64 path).

Tolerance: max |gpu - oracle| <= 1e-10 * max |oracle| over each operator
(the plain-path bar of 1e-10 relative on matrix elements)."""
import numpy as np
import pytest

from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _setup(gpu_lib, oracle_mod, emax):
    bas, lay = make_case(emax)
    return bas, lay, gpu_lib.Basis.from_dict(bas), oracle_mod.Oracle(**bas)


@pytest.mark.parametrize("emax", [2, 4])
@pytest.mark.parametrize("hL,hR", [(-1, 1), (-1, -1), (1, 1), (1, -1)])
def test_commutator_random_ops(gpu_lib, oracle_mod, emax, hL, hR):
    from imsrg_gpu.synth import random_operator
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, emax)
    Lh = random_operator(lay, hL, 31 + emax, 1)
    Rh = random_operator(lay, hR, 41 + emax, 2)
    ref = orc.commutator(Lh, hL, Rh, hR)
    L, R, RES = gpu_lib.Operator(B, hL, Lh), gpu_lib.Operator(B, hR, Rh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(L, R, RES)
    got = RES.download()
    assert RES.herm == -hL * hR
    assert rel_err(got, ref) <= TOL
    assert abs(got[0] - ref[0]) <= TOL * max(1.0, abs(ref[0]))


@pytest.mark.parametrize("emax", [2, 4])
def test_commutator_omega_h(gpu_lib, oracle_mod, emax):
    """[Omega, H] on the synthetic benchmark inputs."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, emax)
    Hh, Oh = synth_hamiltonian(lay, 5), synth_omega(lay, 5)
    ref = orc.commutator(Oh, -1, Hh, 1)
    O, H, RES = gpu_lib.Operator(B, -1, Oh), gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, RES)
    got = RES.download()
    assert rel_err(got, ref) <= TOL
    # the one-body and E0 parts separately
    o = lay.off_fpp + lay.P * lay.P
    assert rel_err(got[1:o], ref[1:o]) <= TOL
    assert abs(got[0] - ref[0]) <= TOL * abs(ref[0])


def test_commutator_without_e0_keeps_e0(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import random_operator
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 2)
    L = gpu_lib.Operator(B, -1, random_operator(lay, -1, 1))
    R = gpu_lib.Operator(B, -1, random_operator(lay, -1, 2))
    init = np.zeros(lay.nfull)
    init[0] = 3.25
    RES = gpu_lib.Operator(B, 1, init)
    gpu_lib.commutator(L, R, RES, with_e0=False)
    assert RES.download()[0] == 3.25


def test_commutator_is_deterministic(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 4)
    O, H = gpu_lib.Operator(B, -1, synth_omega(lay, 2)), gpu_lib.Operator(B, 1, synth_hamiltonian(lay, 2))
    R1, R2 = gpu_lib.Operator(B, 1), gpu_lib.Operator(B, 1)
    gpu_lib.commutator(O, H, R1)
    gpu_lib.commutator(O, H, R2)
    assert np.array_equal(R1.download(), R2.download())


def test_fortran_style_upload_download(gpu_lib, oracle_mod):
    from imsrg_gpu.synth import random_operator
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 4)
    flat = random_operator(lay, 1, 77)
    gams = [lay.gam(flat, q, g).copy(order="F") for q in range(1, lay.nblocks + 1) for g in range(1, 7)]
    op = gpu_lib.Operator(B, 1)
    op.upload_arrays(flat[0], lay.fhh(flat), lay.fph(flat), lay.fpp(flat), gams)
    assert np.array_equal(op.download(), flat)
    shapes = ((lay.A, lay.A), (lay.P, lay.A), (lay.P, lay.P), [g.shape for g in gams])
    e0, fhh, fph, fpp, gk = op.download_arrays(shapes)
    assert e0 == flat[0] and np.array_equal(fph, lay.fph(flat))
    assert all(np.array_equal(a, b) for a, b in zip(gk, gams))


@pytest.mark.parametrize("herm", [1, -1])
def test_packed_layout(gpu_lib, oracle_mod, herm):
    from imsrg_gpu.synth import random_operator
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 4)
    flat = random_operator(lay, herm, 78)
    op = gpu_lib.Operator(B, herm, flat)
    vec = op.download_packed()
    assert np.array_equal(vec, orc.vectorize(flat))
    op2 = gpu_lib.Operator(B, herm)
    op2.upload_packed(vec)
    assert np.array_equal(op2.download(), orc.repackage(vec, herm))


def test_error_codes(gpu_lib, oracle_mod):
    bas, lay, B, orc = _setup(gpu_lib, oracle_mod, 2)
    bas4, lay4 = make_case(4)
    B4 = gpu_lib.Basis.from_dict(bas4)
    L, R = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, 1)
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.commutator(L, R, L)
    assert e.value.status == 1
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.commutator(L, R, gpu_lib.Operator(B4, 1))
    assert e.value.status == 7
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.Operator(B, 3)
    assert e.value.status == 1
    with pytest.raises(gpu_lib.ImsrgError) as e:
        gpu_lib.Basis(bas["nn"], bas["ll"], bas["jj"] + 1, bas["itzp"], bas["con"])  # even 2j
    assert e.value.status == 1
