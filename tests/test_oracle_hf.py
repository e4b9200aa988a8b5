"""The oracle's restatement of the setup steps (interaction file, HO one-body
part, Hartree-Fock) checked against identities that do not use it: file round
trips, symmetries of the r1.r2 / p1.p2 elements, the non-interacting limit,
self-consistency and the normal-ordering identity (E_HF and the HF Fock matrix
equal what the oracle's independent normal_order gives for the bare
Hamiltonian transformed to the HF basis)."""
import numpy as np
import pytest

from conftest import make_case


def _setup(oracle_mod, emax):
    from oracle.hf import Setup
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(bas["nn"], bas["ll"], bas["jj"], bas["itzp"], bas["con"])
    return Setup(orc, bas["nn"], bas["ll"], bas["jj"], bas["itzp"], bas["con"]), orc, lay


def _two_body(lay, H):
    out = H.copy()
    out[:lay.off_fpp + lay.P * lay.P] = 0.0
    return out


@pytest.mark.parametrize("emax", [2, 4])
def test_interaction_file_round_trip(oracle_mod, tmp_path, emax):
    from imsrg_gpu.synth import synth_hamiltonian, write_vrenorm
    S, orc, lay = _setup(oracle_mod, emax)
    V = _two_body(lay, synth_hamiltonian(lay, 11))
    path = str(tmp_path / "v.int")
    n = write_vrenorm(lay, V, path, seed=3)  # random pair / bra-ket orders with their phases
    assert n > 0
    got = S.read_interaction(path, htype=3, hw=20.0, lawson_beta=0.0, mass=16)
    assert np.array_equal(got, V)


def test_com_elements_symmetries(oracle_mod):
    """r1.r2 and p1.p2 between normalised antisymmetric kets are Hermitian and
    change by the pair phase -(-1)^((ja+jb-J)/2) when a pair is reversed."""
    S, orc, lay = _setup(oracle_mod, 2)
    nz = 0
    for b in lay.blocks:
        pairs = np.concatenate([b.qn[0], b.qn[1], b.qn[2]]).reshape(-1, 2)
        for (a, bb) in pairs:
            for (c, d) in pairs:
                for p in (False, True):
                    v = S.r1_r2_p1_p2(a, bb, c, d, b.J2, p)
                    nz += abs(v) > 1e-12
                    assert v == pytest.approx(S.r1_r2_p1_p2(c, d, a, bb, b.J2, p), abs=1e-12)
                    if a != bb:
                        ph = -(-1) ** ((lay.jj[a - 1] + lay.jj[bb - 1] - b.J2) // 2)
                        assert S.r1_r2_p1_p2(bb, a, c, d, b.J2, p) == pytest.approx(ph * v, abs=1e-12)
    assert nz > 0


def test_h0_is_the_ho_kinetic_matrix(oracle_mod):
    """htype 3: diagonal hw/2 (2n + l + 3/2); the single-precision off-diagonals
    agree with the exact ones to float rounding."""
    S, orc, lay = _setup(oracle_mod, 4)
    H = S.h0_harm_osc(np.zeros(lay.nfull), htype=3, hw=20.0)
    for a in range(1, lay.norb + 1):
        n, l = lay.nn[a - 1], lay.ll[a - 1]
        assert orc.f_elem(a, a, H, 1) == 10.0 * (2 * n + l + 1.5)
        for c in range(1, lay.norb + 1):
            if lay.same_ljt(a, c) and lay.nn[c - 1] == n + 1:
                exact = 10.0 * np.sqrt((n + 1) * (n + l + 1.5))
                assert orc.f_elem(a, c, H, 1) == pytest.approx(exact, rel=1e-7)


def _bare(oracle_mod, tmp_path, emax, seed=5, sigma2=0.5):
    from imsrg_gpu.synth import synth_hamiltonian, write_vrenorm
    S, orc, lay = _setup(oracle_mod, emax)
    V = _two_body(lay, synth_hamiltonian(lay, seed, sigma2=sigma2))
    path = str(tmp_path / "v.int")
    write_vrenorm(lay, V, path, seed=seed)
    H = S.read_interaction(path, htype=1, hw=20.0, lawson_beta=0.0, mass=16)
    return S, orc, lay, S.h0_harm_osc(H, htype=1, hw=20.0, mass=16)


def test_hf_without_interaction_diagonalises_t(oracle_mod):
    S, orc, lay = _setup(oracle_mod, 4)
    T = S.h0_harm_osc(np.zeros(lay.nfull), htype=1, hw=20.0, mass=16)
    _, ehf, D, it = S.hartree_fock(T, tol=1e-12)
    want = 0.0
    for j, st in S.sp_blocks():
        if not st:
            continue
        M = np.array([[orc.f_elem(a, c, T, 1) for c in st] for a in st])
        nh = sum(lay.con[s - 1] for s in st)
        want += np.sum(np.linalg.eigvalsh(M)[:nh]) * (j + 1)
    assert ehf == pytest.approx(want, rel=1e-13)
    assert np.allclose(D.T @ D, np.eye(lay.norb), atol=1e-13)


def test_hf_normal_order_identity(oracle_mod, tmp_path):
    """Transforming the bare H to the HF basis and normal ordering it (the
    oracle's normal_order) reproduces E_HF and the HF Fock matrix; the Fock
    matrix is diagonal within each (l, j, tz) block at convergence."""
    S, orc, lay, H0 = _bare(oracle_mod, tmp_path, 4)
    Hhf, ehf, D, it = S.hartree_fock(H0, tol=1e-11)
    assert it > 3
    # the bare operator in the HF basis, not normal ordered
    Hb = H0.copy()
    Dsm = np.zeros((lay.norb + 1, lay.norb + 1))
    Dsm[1:, 1:] = D
    S._transform_2b(Hb, Dsm)
    for j, st in S.sp_blocks():
        if not st:
            continue
        idx = np.array(st) - 1
        Tq = np.array([[orc.f_elem(a, c, H0, 1) for c in st] for a in st])
        T1 = D[np.ix_(idx, idx)].T @ Tq @ D[np.ix_(idx, idx)]
        for a in range(len(st)):
            for c in range(len(st)):
                k = S.f_index(st[a], st[c])
                Hb[k] = T1[a, c] if lay.con[st[a] - 1] + lay.con[st[c] - 1] != 1 or \
                    lay.con[st[c] - 1] > lay.con[st[a] - 1] else T1[c, a]
    Hb[0] = 0.0
    no = orc.normal_order(Hb, 1)
    scale = np.max(np.abs(Hhf))
    assert no[0] == pytest.approx(ehf, abs=1e-8)
    assert np.max(np.abs(no[1:lay.off_fpp + lay.P * lay.P] - Hhf[1:lay.off_fpp + lay.P * lay.P])) < 1e-8 * scale
    assert np.array_equal(no[lay.off_fpp + lay.P * lay.P:], Hhf[lay.off_fpp + lay.P * lay.P:])
    # Brillouin: no particle-hole Fock elements
    assert np.max(np.abs(lay.fph(Hhf))) < 1e-8 * scale
