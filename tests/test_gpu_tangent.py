"""dE0/dc_k of the Magnus flow for H(c) = T + sum_k c_k V_k (four seeded
N(0,1) MeV two-body terms, emax = 4, c = (1,1,1,1)) from the library's
tangent-linear flow, against central finite differences (h = 1e-4) of the
oracle's FP64 CPU flow."""
import numpy as np
import pytest

from conftest import make_case

pytestmark = pytest.mark.gpu

S_MAX = 2.0  # the flow stops on s in every run, so each run takes the same steps


def _terms(lay, oracle_mod, bas):
    from imsrg_gpu.synth import synth_hamiltonian
    one = lay.off_fpp + lay.P * lay.P  # E0 + one-body part of the flat layout
    T = synth_hamiltonian(lay, 300)
    T[one:] = 0.0
    V = []
    for k in range(4):
        v = synth_hamiltonian(lay, 301 + k)
        v[:one] = 0.0
        V.append(v)
    return T, V


def test_tangent_flow_matches_oracle_finite_differences(gpu_lib, oracle_mod):
    bas, lay = make_case(4)
    orc = oracle_mod.Oracle(**bas)
    T, V = _terms(lay, oracle_mod, bas)
    c = np.ones(4)

    def H_of(cv):
        return orc.normal_order(T + sum(ck * vk for ck, vk in zip(cv, V)))

    B = gpu_lib.Basis.from_dict(bas)
    H0 = H_of(c)
    # the undifferentiated part of the tangent flow is the plain flow
    HSp, Gp = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, -1)
    plain = gpu_lib.magnus_decouple(HSp, Gp, s_max=S_MAX, ds=0.5)
    h = 1e-4
    for k in range(4):
        HS, dHS = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, 1, orc.normal_order(V[k]))
        G, dG = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, -1)
        out = gpu_lib.magnus_decouple_tangent(HS, dHS, G, dG, s_max=S_MAX, ds=0.5)
        assert out["steps"] == plain["steps"]
        assert np.array_equal(out["trace"], plain["trace"])
        grad = out["dtrace"][-1, 2]
        ep = orc.magnus_decouple(H_of(c + h * np.eye(4)[k]), s_max=S_MAX, ds=0.5)
        em = orc.magnus_decouple(H_of(c - h * np.eye(4)[k]), s_max=S_MAX, ds=0.5)
        assert ep["steps"] == em["steps"] == out["steps"]
        fd = (ep["trace"][-1, 2] - em["trace"][-1, 2]) / (2 * h)
        assert abs(grad - fd) < 1e-6 * max(1.0, abs(fd)), (k, grad, fd)


def test_tangent_is_linear_in_the_direction(gpu_lib, oracle_mod):
    """d(E0) along V_0 + 2 V_1 equals d(E0)/dc_0 + 2 d(E0)/dc_1 (to rounding)."""
    bas, lay = make_case(2)
    orc = oracle_mod.Oracle(**bas)
    T, V = _terms(lay, oracle_mod, bas)
    H0 = orc.normal_order(T + sum(V))
    B = gpu_lib.Basis.from_dict(bas)
    res = []
    for d in (V[0], V[1], V[0] + 2 * V[1]):
        HS, dHS = gpu_lib.Operator(B, 1, H0), gpu_lib.Operator(B, 1, orc.normal_order(d))
        G, dG = gpu_lib.Operator(B, -1), gpu_lib.Operator(B, -1)
        res.append(gpu_lib.magnus_decouple_tangent(HS, dHS, G, dG, s_max=S_MAX, ds=0.5)["dtrace"][-1, 2])
    assert abs(res[2] - (res[0] + 2 * res[1])) < 1e-9 * max(1.0, abs(res[2]))
