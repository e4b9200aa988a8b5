"""Graph-captured Magnus steps (one CUDA graph per step, device-side series
loops) and batched flows: bit-for-bit equal to the host-driven flow and to
the unbatched flow."""
import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu


def _hamiltonian(gpu_lib, oracle_mod, emax, seed, hw=20.0, sigma2=1.0):
    from imsrg_gpu.synth import synth_hamiltonian
    bas, lay = make_case(emax)
    orc = oracle_mod.Oracle(**bas)
    return bas, orc.normal_order(synth_hamiltonian(lay, seed, hw=hw, sigma2=sigma2))


def _flow(gpu_lib, bas, Hh, fn, **kw):
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    out = fn(HS, G, **kw)
    out["H"], out["Omega"] = HS.download(), G.download()
    return out


@pytest.mark.parametrize("emax,precision", [(2, "fp64"), (4, "fp64"), (4, "ozaki")])
def test_graph_flow_equals_host_flow(gpu_lib, oracle_mod, emax, precision):
    bas, Hh = _hamiltonian(gpu_lib, oracle_mod, emax, 21)
    kw = dict(s_max=10.0, ds=0.5, precision=precision)
    host = _flow(gpu_lib, bas, Hh, gpu_lib.magnus_decouple, **kw)
    graph = _flow(gpu_lib, bas, Hh, gpu_lib.magnus_decouple_graph, **kw)
    assert graph["steps"] == host["steps"] > 2
    assert graph["ncomm"] == host["ncomm"]
    assert np.array_equal(graph["trace"], host["trace"])
    assert np.array_equal(graph["H"], host["H"])
    assert np.array_equal(graph["Omega"], host["Omega"])


def test_graph_is_reused_across_calls(gpu_lib, oracle_mod):
    bas, Hh = _hamiltonian(gpu_lib, oracle_mod, 2, 22)
    B = gpu_lib.Basis.from_dict(bas)
    HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
    a = gpu_lib.magnus_decouple_graph(HS, G, s_max=5.0, ds=0.5)
    HS.upload(Hh)
    b = gpu_lib.magnus_decouple_graph(HS, G, s_max=5.0, ds=0.5)
    assert np.array_equal(a["trace"], b["trace"])


def test_batched_flows_equal_unbatched(gpu_lib, oracle_mod):
    """Instances with their own hbar*omega (U[12, 28] MeV), two-body scale
    (U[0.5, 2] MeV) and emax, advanced together: each equals its own flow bit
    for bit, including an instance whose BCH series fails to converge (it
    stops with IMSRG_ERR_NOT_CONVERGED, as the reference STOPs, while the
    others carry on)."""
    rng = np.random.default_rng(7)
    cases = []
    for k, emax in enumerate([2, 4, 2, 4, 6, 2]):
        hw, sig = float(rng.uniform(12.0, 28.0)), float(rng.uniform(0.5, 2.0))
        cases.append((emax,) + _hamiltonian(gpu_lib, oracle_mod, emax, 100 + k, hw=hw, sigma2=sig))
    kw = dict(s_max=3.0, ds=0.5)
    for precision in ("fp64", "ozaki"):
        single = []
        for _, bas, Hh in cases:
            B = gpu_lib.Basis.from_dict(bas)
            HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
            one = gpu_lib.magnus_decouple_batch([HS], [G], precision=precision, **kw)[0]
            one["H"], one["Omega"] = HS.download(), G.download()
            single.append(one)
        Bs = [gpu_lib.Basis.from_dict(bas) for _, bas, _ in cases]
        HS = [gpu_lib.Operator(B, 1, Hh) for B, (_, _, Hh) in zip(Bs, cases)]
        G = [gpu_lib.Operator(B, -1) for B in Bs]
        batch = gpu_lib.magnus_decouple_batch(HS, G, precision=precision, **kw)
        assert sum(o["status"] == 0 for o in single) >= 4
        for i, (one, many) in enumerate(zip(single, batch)):
            assert many["status"] == one["status"], i
            assert many["steps"] == one["steps"] and many["ncomm"] == one["ncomm"], i
            assert np.array_equal(many["trace"], one["trace"]), i
            assert np.array_equal(HS[i].download(), one["H"]), i
            assert np.array_equal(G[i].download(), one["Omega"]), i


def test_batch_rejects_shared_basis(gpu_lib, oracle_mod):
    bas, Hh = _hamiltonian(gpu_lib, oracle_mod, 2, 23)
    B = gpu_lib.Basis.from_dict(bas)
    HS = [gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, 1, Hh)]
    G = [gpu_lib.Operator(B, -1), gpu_lib.Operator(B, -1)]
    with pytest.raises(gpu_lib.ImsrgError):
        gpu_lib.magnus_decouple_batch(HS, G, s_max=1.0)


@pytest.mark.parametrize("precision", ["ozaki", "fp64"])
def test_lockstep_batch_flows_equal_unbatched(gpu_lib, oracle_mod, precision):
    """imsrg_gpu_batch_magnus_decouple: instances of mixed emax, hbar*omega
    and two-body scale in lockstep (one graph per step for all, one merged
    product launch per series term, stopped series and flows skipped on the
    device) equal their unbatched graph-captured flows bit for bit, including
    an instance whose BCH series does not converge; the step graph is reused
    by a second call."""
    rng = np.random.default_rng(7)
    cases = []
    for k, emax in enumerate([2, 4, 2, 4, 6, 2]):
        hw, sig = float(rng.uniform(12.0, 28.0)), float(rng.uniform(0.5, 2.0))
        cases.append((emax,) + _hamiltonian(gpu_lib, oracle_mod, emax, 100 + k, hw=hw, sigma2=sig))
    kw = dict(s_max=3.0, ds=0.5)
    single = []
    for _, bas, Hh in cases:
        B = gpu_lib.Basis.from_dict(bas)
        B.set_split_digits(5)
        HS, G = gpu_lib.Operator(B, 1, Hh), gpu_lib.Operator(B, -1)
        one = gpu_lib.magnus_decouple_batch([HS], [G], precision=precision, **kw)[0]
        one["H"], one["Omega"] = HS.download(), G.download()
        single.append(one)
    assert sum(o["status"] == 0 for o in single) >= 4
    Bs = []
    for _, bas, _ in cases:
        B = gpu_lib.Basis.from_dict(bas)
        B.set_split_digits(5)
        Bs.append(B)
    batch = gpu_lib.Batch(Bs)
    HS = [gpu_lib.Operator(B, 1, Hh) for B, (_, _, Hh) in zip(Bs, cases)]
    G = [gpu_lib.Operator(B, -1) for B in Bs]
    for rep in range(2):
        for i, (_, _, Hh) in enumerate(cases):
            HS[i].upload(Hh)
        many = batch.magnus_decouple(HS, G, precision=precision, **kw)
        for i, (one, m) in enumerate(zip(single, many)):
            assert m["status"] == one["status"], (rep, i)
            assert m["steps"] == one["steps"] and m["ncomm"] == one["ncomm"], (rep, i)
            assert np.array_equal(m["trace"], one["trace"]), (rep, i)
            assert np.array_equal(HS[i].download(), one["H"]), (rep, i)
            assert np.array_equal(G[i].download(), one["Omega"]), (rep, i)
    batch.close()
