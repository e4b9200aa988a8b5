"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py
Writes emax2_golden.npz: the 4He emax=2 basis, seeded synthetic Omega and H
(H normal-ordered), the oracle's [Omega,H], White generator of H, one BCH
transform, and the Magnus-flow trace (step, s, E0, E0+mbpt2, |mbpt2|) to s=50;
plus a uniform-[-5,5] operator pair (brute_force_testing.f90 style) and its
commutator.
Writes emax6_flow.npz: the oracle's Magnus flow (White generator, ds = 0.5,
s_max = 50) of the normal-ordered seed-13 synthetic Hamiltonian in the 16O
emax=6 basis: the trace rows (step, s, E0, E0+mbpt2, |mbpt2|), the step and
commutator counts and mat_frob_norm of the final Omega.  bench.py reports its
emax=6 flows against this trace.  Only the emax=6 fixture:
python tests/golden/make_golden.py emax6
Writes adjoint_fd_emax4.npz: dE0/dc_k of the oracle's Magnus flow (White
generator, ds = 0.5, to |E_mbpt2| < 1e-6) for H(c) = T + sum_k c_k V_k in the
16O emax=4 basis (T the seed-300 one-body part, V_k the seed-301..304
two-body parts, c = 1) by central differences with h = 1e-4; bench.py
reports its adjoint gradients against them.  Only this fixture:
python tests/golden/make_golden.py adjoint
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "eom-imsrg_full_gb300"))

from imsrg_gpu.layout import Layout, ho_basis  # noqa: E402
from imsrg_gpu.synth import adjoint_terms, random_operator, synth_hamiltonian, synth_omega  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402


def emax6_flow():
    import os as _os
    from oracle.oracle import set_threads
    set_threads(_os.cpu_count())
    bas = ho_basis(6)
    lay = Layout(**bas)
    orc = Oracle(**bas)
    H = orc.normal_order(synth_hamiltonian(lay, 13))
    flow = orc.magnus_decouple(H, s_max=50.0, ds=0.5)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "emax6_flow.npz")
    np.savez_compressed(out, trace=flow["trace"], steps=flow["steps"], ncomm=flow["ncomm"],
                        omega_norm=orc.norm(flow["Omega"]), seed=13, s_max=50.0, ds=0.5)
    print("wrote", out, "flow steps", flow["steps"], "E0", flow["trace"][-1, 2])


def adjoint_fd():
    import os as _os
    from oracle.oracle import set_threads
    set_threads(_os.cpu_count())
    bas = ho_basis(4)
    lay = Layout(**bas)
    orc = Oracle(**bas)
    T, V = adjoint_terms(lay)
    c = np.ones(4)
    h = 1e-4

    def e0(cv):
        f = orc.magnus_decouple(orc.normal_order(T + sum(ck * vk for ck, vk in zip(cv, V))), s_max=50.0, ds=0.5)
        return f["trace"][-1, 2], f["steps"]

    base, steps = e0(c)
    fd = []
    for k in range(4):
        (ep, sp), (em, sm) = e0(c + h * np.eye(4)[k]), e0(c - h * np.eye(4)[k])
        assert sp == sm == steps
        fd.append((ep - em) / (2 * h))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "adjoint_fd_emax4.npz")
    np.savez_compressed(out, fd=np.array(fd), e0=base, steps=steps, h=h, c=c)
    print("wrote", out, "dE0/dc", fd)


def main():
    bas = ho_basis(2)
    lay = Layout(**bas)
    orc = Oracle(**bas)
    H = orc.normal_order(synth_hamiltonian(lay, 1))
    O = synth_omega(lay, 1)
    comm = orc.commutator(O, -1, H, 1)
    eta = orc.white(H)
    hs, nbch = orc.bch_expand(O, H)
    flow = orc.magnus_decouple(H, s_max=50.0, ds=0.5)
    A = random_operator(lay, -1, 1001, 1)
    Bm = random_operator(lay, 1, 1002, 2)
    commAB = orc.commutator(A, -1, Bm, 1)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "emax2_golden.npz")
    np.savez_compressed(out, nn=bas["nn"], ll=bas["ll"], jj=bas["jj"], itzp=bas["itzp"], con=bas["con"],
                        H=H, Omega=O, comm=comm, eta=eta, bch=hs, nbch=nbch, flow_trace=flow["trace"],
                        flow_H=flow["H"], A=A, B=Bm, commAB=commAB)
    print("wrote", out, "flow steps", flow["steps"], "E0", flow["trace"][-1, 2])


if __name__ == "__main__":
    if sys.argv[1:] == ["emax6"]:
        emax6_flow()
    elif sys.argv[1:] == ["adjoint"]:
        adjoint_fd()
    else:
        main()
        emax6_flow()
        adjoint_fd()
