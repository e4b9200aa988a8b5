"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liborc.so`` (built by ``oracle/Makefile``) and exposes
the restated reference routines on numpy arrays in the flat operator layout.
Only the tests, the smoke check and the CPU-baseline leg of the benchmark use
this module; the GPU library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# parity: the checker (-ffp-contract=off); fast: the timed CPU baseline
LIB_PATHS = {"parity": os.path.join(HERE, "_build", platform.machine(), "liborc.so"),
             "fast": os.path.join(HERE, "_build", platform.machine(), "liborc_fast.so")}
LIB_PATH = LIB_PATHS["parity"]

_libs = {}


def build(force: bool = False):
    src = os.path.join(HERE, "imsrg_oracle.c")
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < os.path.getmtime(src) for p in LIB_PATHS.values()):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib(variant: str = "parity"):
    if variant not in _libs:
        build()
        L = C.CDLL(LIB_PATHS[variant])
        vp, dp, ip, lp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_long)
        i, d = C.c_int, C.c_double
        sig = {
            "orc_basis_new": (vp, [i, ip, ip, ip, ip, ip]),
            "orc_basis_free": (None, [vp]),
            "orc_basis_info": (None, [vp, lp]),
            "orc_block_dims": (None, [vp, ip]),
            "orc_block_qn": (None, [vp, i, i, ip]),
            "orc_cc_dims": (None, [vp, ip]),
            "orc_commutator": (None, [vp, dp, i, dp, i, dp]),
            "orc_commutator_parts": (None, [vp, dp, i, dp, i, dp, dp, dp, dp, dp, dp]),
            "orc_comm110": (d, [vp, dp, i, dp, i]),
            "orc_comm220": (d, [vp, dp, i, dp, i]),
            "orc_cross_coupled": (None, [vp, dp, i, dp]),
            "orc_white": (None, [vp, dp, i, dp]),
            "orc_atan": (None, [vp, dp, i, dp]),
            "orc_atanxx": (None, [vp, dp, i, dp, dp]),
            "orc_w2": (None, [vp, dp, i, dp]),
            "orc_magnus_decouple_gen": (i, [vp, i, dp, dp, d, d, i, dp, ip]),
            "orc_normal_order": (None, [vp, dp, i]),
            "orc_mbpt2": (d, [vp, dp, i]),
            "orc_norm": (d, [vp, dp]),
            "orc_add": (None, [vp, dp, d, dp, d, dp]),
            "orc_vectorize": (None, [vp, dp, dp]),
            "orc_repackage": (None, [vp, dp, i, dp]),
            "orc_magnus_expand": (i, [vp, dp, dp]),
            "orc_bch_expand": (i, [vp, dp, dp, dp]),
            "orc_magnus_decouple": (i, [vp, dp, dp, d, d, i, dp, ip]),
            "orc_bf_0body": (d, [vp, dp, i, dp, i]),
            "orc_bf_1body": (d, [vp, dp, i, dp, i, i, i]),
            "orc_bf_2body": (d, [vp, dp, i, dp, i, i, i, i, i, i]),
            "orc_v_elem": (d, [vp, i, i, i, i, i, dp, i]),
            "orc_f_elem": (d, [vp, i, i, dp, i]),
            "orc_sixj": (d, [vp, i, i, i, i, i, i]),
            "orc_d6ji": (d, [vp, i, i, i, i, i, i]),
            "orc_coef9": (d, [vp] + [i] * 9),
            "orc_set_threads": (None, [i]),
            "orc_get_threads": (i, []),
            "orc_set_dgemm": (None, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[variant] = L
    return _libs[variant]


def _dp(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


class Oracle:
    """One basis of the oracle; methods mirror the reference routines.
    variant "parity" (default) is the checker; "fast" is the timed CPU
    baseline build (see use_blas)."""

    def __init__(self, nn, ll, jj, itzp, con, variant: str = "parity"):
        self._L = L = lib(variant)
        self._keep = [_ip(x) for x in (nn, ll, jj, itzp, con)]
        self.h = L.orc_basis_new(len(jj), *[p for _, p in self._keep])
        info = np.zeros(11, np.int64)
        L.orc_basis_info(self.h, info.ctypes.data_as(C.POINTER(C.c_long)))
        (self.norb, self.A, self.P, self.nblocks, self.Jtotal_max, self.lmax, self.nfull, self.neq,
         self.ccblocks, self.cc_total, self.wcc_total) = [int(x) for x in info]

    def __del__(self):
        try:
            self._L.orc_basis_free(self.h)
        except Exception:
            pass

    # layout queries ---------------------------------------------------
    def block_dims(self):
        out = np.zeros(6 * self.nblocks, np.int32)
        self._L.orc_block_dims(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out.reshape(-1, 6)

    def block_qn(self, q, c):
        dims = self.block_dims()[q - 1]
        n = dims[2 + c]
        out = np.zeros(2 * n, np.int32)
        self._L.orc_block_qn(self.h, q, c, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out.reshape(-1, 2)

    def cc_dims(self):
        out = np.zeros(3 * self.ccblocks, np.int32)
        self._L.orc_cc_dims(self.h, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out.reshape(-1, 3)

    # operators --------------------------------------------------------
    def zeros(self):
        return np.zeros(self.nfull)

    def commutator(self, Lop, hL, Rop, hR):
        out = self.zeros()
        self._L.orc_commutator(self.h, _dp(Lop), hL, _dp(Rop), hR, _dp(out))
        return out

    def commutator_parts(self, Lop, hL, Rop, hR):
        res, w1, w2 = self.zeros(), self.zeros(), self.zeros()
        lcc, rcc = np.zeros(self.cc_total + 1), np.zeros(self.cc_total + 1)
        wcc = np.zeros(self.wcc_total + 1)
        self._L.orc_commutator_parts(self.h, _dp(Lop), hL, _dp(Rop), hR, _dp(res), _dp(w1), _dp(w2), _dp(lcc),
                                   _dp(rcc), _dp(wcc))
        return dict(res=res, w1=w1, w2=w2, lcc=lcc[:self.cc_total], rcc=rcc[:self.cc_total],
                    wcc=wcc[:self.wcc_total])

    def comm110(self, Lop, hL, Rop, hR):
        return self._L.orc_comm110(self.h, _dp(Lop), hL, _dp(Rop), hR)

    def comm220(self, Lop, hL, Rop, hR):
        return self._L.orc_comm220(self.h, _dp(Lop), hL, _dp(Rop), hR)

    def cross_coupled(self, op, herm):
        out = np.zeros(self.cc_total + 1)
        self._L.orc_cross_coupled(self.h, _dp(op), herm, _dp(out))
        return out[:self.cc_total]

    def white(self, H, herm=1):
        eta = self.zeros()
        self._L.orc_white(self.h, _dp(H), herm, _dp(eta))
        return eta

    def atan_gen(self, H, herm=1):
        """build_gs_atan (generators.f90:162-266)."""
        eta = self.zeros()
        self._L.orc_atan(self.h, _dp(H), herm, _dp(eta))
        return eta

    def atanxx_gen(self, Hold, H, herm=1):
        """build_gs_atanxx (generators.f90:271-376)."""
        eta = self.zeros()
        self._L.orc_atanxx(self.h, _dp(Hold), herm, _dp(H), _dp(eta))
        return eta

    def w2_gen(self, H, herm=1):
        """build_gs_w2 (generators.f90:109-159)."""
        eta = self.zeros()
        self._L.orc_w2(self.h, _dp(H), herm, _dp(eta))
        return eta

    def normal_order(self, H, herm=1):
        out = H.copy()
        self._L.orc_normal_order(self.h, _dp(out), herm)
        return out

    def mbpt2(self, H, herm=1):
        return self._L.orc_mbpt2(self.h, _dp(H), herm)

    def norm(self, op):
        return self._L.orc_norm(self.h, _dp(op))

    def add(self, A, ax, B, bx):
        out = self.zeros()
        self._L.orc_add(self.h, _dp(A), ax, _dp(B), bx, _dp(out))
        return out

    def vectorize(self, op):
        out = np.zeros(self.neq)
        self._L.orc_vectorize(self.h, _dp(op), _dp(out))
        return out

    def repackage(self, vec, herm):
        out = self.zeros()
        self._L.orc_repackage(self.h, _dp(np.ascontiguousarray(vec, np.float64)), herm, _dp(out))
        return out

    def magnus_expand(self, eta, G):
        dg = eta.copy()
        n = self._L.orc_magnus_expand(self.h, _dp(dg), _dp(G))
        return dg, n

    def bch_expand(self, G, H):
        hs = self.zeros()
        n = self._L.orc_bch_expand(self.h, _dp(hs), _dp(G), _dp(H))
        return hs, n

    def magnus_decouple(self, H, s_max=50.0, ds=0.5, max_steps=1000):
        hs = H.copy()
        G = self.zeros()
        trace = np.zeros(5 * (max_steps + 1))
        nc = C.c_int(0)
        steps = self._L.orc_magnus_decouple(self.h, _dp(hs), _dp(G), s_max, ds, max_steps, _dp(trace), C.byref(nc))
        nrow = max(steps, 0) + 1
        return dict(H=hs, Omega=G, steps=steps, trace=trace[:5 * nrow].reshape(nrow, 5), ncomm=nc.value)

    def magnus_decouple_gen(self, H, generator="white", s_max=50.0, ds=0.5, max_steps=1000):
        gen = {"white": 0, "atan": 1, "w2": 2}[generator]
        hs = H.copy()
        G = self.zeros()
        trace = np.zeros(5 * (max_steps + 1))
        nc = C.c_int(0)
        steps = self._L.orc_magnus_decouple_gen(self.h, gen, _dp(hs), _dp(G), s_max, ds, max_steps, _dp(trace),
                                              C.byref(nc))
        nrow = max(steps, 0) + 1
        return dict(H=hs, Omega=G, steps=steps, trace=trace[:5 * nrow].reshape(nrow, 5), ncomm=nc.value)

    # known-answer formulas -------------------------------------------------
    def bf_0body(self, A, hA, B, hB):
        return self._L.orc_bf_0body(self.h, _dp(A), hA, _dp(B), hB)

    def bf_1body(self, A, hA, B, hB, a, b):
        return self._L.orc_bf_1body(self.h, _dp(A), hA, _dp(B), hB, a, b)

    def bf_2body(self, A, hA, B, hB, a, b, c, d, J2):
        return self._L.orc_bf_2body(self.h, _dp(A), hA, _dp(B), hB, a, b, c, d, J2)

    def v_elem(self, a, b, c, d, J2, op, herm):
        return self._L.orc_v_elem(self.h, a, b, c, d, J2, _dp(op), herm)

    def f_elem(self, a, b, op, herm):
        return self._L.orc_f_elem(self.h, a, b, _dp(op), herm)

    def sixj(self, *j):
        return self._L.orc_sixj(self.h, *j)

    def d6ji(self, *j):
        return self._L.orc_d6ji(self.h, *j)

    def coef9(self, *j):
        return self._L.orc_coef9(self.h, *j)


def set_threads(n: int):
    lib().orc_set_threads(n)


def get_threads() -> int:
    return lib().orc_get_threads()


def use_blas(threads: int | None = None) -> str | None:
    """Route the fast build's dgemm to the OpenBLAS that numpy bundles (its
    Fortran ILP64 interface), on `threads` threads.  Returns a description of
    the BLAS, or None when none was found (the own GEMM stays)."""
    import glob
    import numpy
    libdir = os.path.join(os.path.dirname(numpy.__file__), "..", "numpy.libs")
    for path in sorted(glob.glob(os.path.join(libdir, "*openblas*.so*"))):
        try:
            ob = C.CDLL(path)
            fn = ob.scipy_dgemm_64_
        except (OSError, AttributeError):
            continue
        desc = os.path.basename(path)
        try:
            ob.scipy_openblas_get_config64_.restype = C.c_char_p
            desc = ob.scipy_openblas_get_config64_().decode().strip()
        except AttributeError:
            pass
        if threads:
            try:
                ob.scipy_openblas_set_num_threads64_.argtypes = [C.c_int]
                ob.scipy_openblas_set_num_threads64_(int(threads))
            except AttributeError:
                pass
        _libs.setdefault("_blas", ob)  # keep it loaded
        lib("fast").orc_set_dgemm(C.cast(fn, C.c_void_p))
        return desc
    return None
