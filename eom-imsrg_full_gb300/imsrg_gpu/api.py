"""Python mirror of the reference operator interface over libimsrg_gpu.so.

Names follow the Fortran routines they replace (n-parzuchowski/EOM-IMSRG_FULL,
im-SRG/): ``commutator`` is the 110..222_ph sequence of IMSRG_MAGNUS.f90:207-219,
``build_gs_white`` generators.f90:4, ``magnus_expand`` / ``bch_expand`` /
``euler_step`` / ``magnus_decouple`` IMSRG_MAGNUS.f90:622 / :149 / :756 / :15,
``add_sq_op`` / ``copy_sq_op`` / ``clear_sq_op`` / ``mat_frob_norm`` /
``mbpt2`` basic_IMSRG.f90:3450 / :2942 / :3537 / :3921 / :4030.

Every call goes through the C ABI of include/imsrg_gpu.h; a failing status
raises ImsrgError (the reference STOPs instead).  There is no CPU fallback:
a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libimsrg_gpu.so")

PREC = {"fp64": 0, "ozaki": 1}

SYMBOLS = (
    "imsrg_gpu_basis_create", "imsrg_gpu_basis_destroy", "imsrg_gpu_basis_info", "imsrg_gpu_block_dims",
    "imsrg_gpu_synchronize", "imsrg_gpu_op_create", "imsrg_gpu_op_destroy", "imsrg_gpu_op_set_herm",
    "imsrg_gpu_op_get_herm", "imsrg_gpu_op_upload", "imsrg_gpu_op_download", "imsrg_gpu_op_upload_flat",
    "imsrg_gpu_op_download_flat", "imsrg_gpu_op_upload_packed", "imsrg_gpu_op_download_packed",
    "imsrg_gpu_op_device_ptr", "imsrg_gpu_op_copy", "imsrg_gpu_op_clear", "imsrg_gpu_op_add",
    "imsrg_gpu_op_norm", "imsrg_gpu_op_mbpt2", "imsrg_gpu_op_get_e0", "imsrg_gpu_commutator",
    "imsrg_gpu_build_gs_white", "imsrg_gpu_magnus_expand", "imsrg_gpu_bch_expand", "imsrg_gpu_euler_step",
    "imsrg_gpu_magnus_decouple", "imsrg_gpu_strerror", "imsrg_gpu_launch_count",
    "imsrg_gpu_basis_get_stream", "imsrg_gpu_basis_set_stream", "imsrg_gpu_profile_enable",
    "imsrg_gpu_profile_read", "imsrg_gpu_profile_reset", "imsrg_gpu_commutator_noalloc",
    "imsrg_gpu_magnus_decouple_graph", "imsrg_gpu_magnus_decouple_batch", "imsrg_gpu_magnus_decouple_tangent",
    "imsrg_gpu_split_schedule", "imsrg_gpu_split_schedule_set", "imsrg_gpu_split_digits_set", "imsrg_gpu_build_gs_atan", "imsrg_gpu_build_gs_w2", "imsrg_gpu_magnus_decouple_gen",
    "imsrg_gpu_op_save", "imsrg_gpu_op_load", "imsrg_gpu_checkpoint_name", "imsrg_gpu_normal_order",
    "imsrg_gpu_dhds", "imsrg_gpu_transform_bch", "imsrg_gpu_ode_decouple", "imsrg_gpu_commutator_host",
    "imsrg_gpu_read_interaction", "imsrg_gpu_h0_harm_osc", "imsrg_gpu_hartree_fock", "imsrg_gpu_transform_to_hf",
    "imsrg_gpu_batch_create", "imsrg_gpu_batch_commutator", "imsrg_gpu_batch_destroy",
    "imsrg_gpu_magnus_rules", "imsrg_gpu_magnus_decouple_checkpoint",
    "imsrg_gpu_commutator_adjoint", "imsrg_gpu_white_adjoint", "imsrg_gpu_op_dot",
    "imsrg_gpu_magnus_decouple_adjoint", "imsrg_gpu_split_chunk_set", "imsrg_gpu_batch_magnus_decouple",
    "imsrg_gpu_commutator_host_packed",
)

KERNELS = ("cc_forward", "gemm_fp64", "assemble_2body", "assemble_1body", "ozaki_slice", "ozaki_mma",
           "ozaki_epilogue", "ops")


class ImsrgError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {strerror(status)} (status {status})")


class BasisInfo(C.Structure):
    _fields_ = [("norb", C.c_int), ("nholes", C.c_int), ("nparts", C.c_int), ("nblocks", C.c_int),
                ("jtotal_max", C.c_int), ("ccblocks", C.c_int), ("nfull", C.c_long), ("neq", C.c_long),
                ("cc_total", C.c_long), ("wcc_total", C.c_long)]


_lib = None


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip, i, d = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int, C.c_double
        sig = {
            "imsrg_gpu_basis_create": [i, ip, ip, ip, ip, ip, C.POINTER(vp)],
            "imsrg_gpu_basis_destroy": [vp],
            "imsrg_gpu_basis_info": [vp, C.POINTER(BasisInfo)],
            "imsrg_gpu_block_dims": [vp, i, ip, ip, ip],
            "imsrg_gpu_synchronize": [vp],
            "imsrg_gpu_op_create": [vp, i, C.POINTER(vp)],
            "imsrg_gpu_op_destroy": [vp],
            "imsrg_gpu_op_set_herm": [vp, i],
            "imsrg_gpu_op_get_herm": [vp, ip],
            "imsrg_gpu_op_upload": [vp, d, dp, dp, dp, C.POINTER(dp)],
            "imsrg_gpu_op_download": [vp, dp, dp, dp, dp, C.POINTER(dp)],
            "imsrg_gpu_op_upload_flat": [vp, dp],
            "imsrg_gpu_op_download_flat": [vp, dp],
            "imsrg_gpu_op_upload_packed": [vp, dp],
            "imsrg_gpu_op_download_packed": [vp, dp],
            "imsrg_gpu_op_device_ptr": [vp, C.POINTER(vp)],
            "imsrg_gpu_op_copy": [vp, vp],
            "imsrg_gpu_op_clear": [vp],
            "imsrg_gpu_op_add": [vp, d, vp, d, vp],
            "imsrg_gpu_op_norm": [vp, dp],
            "imsrg_gpu_op_mbpt2": [vp, dp],
            "imsrg_gpu_op_get_e0": [vp, dp],
            "imsrg_gpu_commutator": [vp, vp, vp, i, i],
            "imsrg_gpu_commutator_host": [vp, vp, i, vp, i, vp, i, i],
            "imsrg_gpu_commutator_host_packed": [vp, vp, i, vp, i, vp, i, i],
            "imsrg_gpu_build_gs_white": [vp, vp],
            "imsrg_gpu_magnus_expand": [vp, vp, i, ip],
            "imsrg_gpu_bch_expand": [vp, vp, vp, i, ip],
            "imsrg_gpu_euler_step": [vp, vp, dp, d],
            "imsrg_gpu_magnus_decouple": [vp, vp, d, d, i, i, dp, ip, ip],
            "imsrg_gpu_launch_count": [vp, C.POINTER(C.c_long)],
            "imsrg_gpu_basis_get_stream": [vp, C.POINTER(vp)],
            "imsrg_gpu_basis_set_stream": [vp, vp],
            "imsrg_gpu_profile_enable": [vp, i],
            "imsrg_gpu_profile_read": [vp, i, dp, C.POINTER(C.c_long)],
            "imsrg_gpu_profile_reset": [vp],
            "imsrg_gpu_commutator_noalloc": [vp, vp, i, vp, i, vp, i, vp],
            "imsrg_gpu_magnus_decouple_graph": [vp, vp, d, d, i, i, dp, ip, ip],
            "imsrg_gpu_magnus_decouple_batch": [i, C.POINTER(vp), C.POINTER(vp), d, d, i, i, C.POINTER(dp), ip, ip,
                                                ip],
            "imsrg_gpu_magnus_decouple_tangent": [vp, vp, vp, vp, d, d, i, i, dp, dp, ip, ip],
            "imsrg_gpu_split_schedule": [vp, ip, ip, dp, i],
            "imsrg_gpu_split_schedule_set": [vp, i],
            "imsrg_gpu_split_digits_set": [vp, i],
            "imsrg_gpu_split_chunk_set": [vp, i],
            "imsrg_gpu_build_gs_atan": [vp, vp],
            "imsrg_gpu_build_gs_w2": [vp, vp, i],
            "imsrg_gpu_magnus_decouple_gen": [vp, vp, i, d, d, i, i, dp, ip, ip],
            "imsrg_gpu_op_save": [vp, C.c_char_p],
            "imsrg_gpu_op_load": [vp, C.c_char_p],
            "imsrg_gpu_checkpoint_name": [C.c_char_p, C.c_char_p, d, C.c_char_p, i],
            "imsrg_gpu_normal_order": [vp],
            "imsrg_gpu_dhds": [vp, vp, i, i],
            "imsrg_gpu_ode_decouple": [vp, i, i, d, d, i, d, d, dp, ip, C.POINTER(C.c_long)],
            "imsrg_gpu_transform_bch": [vp, vp, i, ip],
            "imsrg_gpu_read_interaction": [vp, C.c_char_p, i, d, d, d, i],
            "imsrg_gpu_h0_harm_osc": [vp, i, d, d, d, i],
            "imsrg_gpu_hartree_fock": [vp, d, i, dp, ip, dp],
            "imsrg_gpu_transform_to_hf": [vp, dp],
            "imsrg_gpu_batch_create": [i, C.POINTER(vp), C.POINTER(vp)],
            "imsrg_gpu_batch_commutator": [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), i, i],
            "imsrg_gpu_batch_destroy": [vp],
            "imsrg_gpu_batch_magnus_decouple": [vp, C.POINTER(vp), C.POINTER(vp), d, d, i, i, C.POINTER(dp), ip, ip,
                                                ip],
            "imsrg_gpu_magnus_rules": [vp, d, dp, ip],
            "imsrg_gpu_commutator_adjoint": [vp, vp, i, i, vp],
            "imsrg_gpu_white_adjoint": [vp, vp, vp],
            "imsrg_gpu_op_dot": [vp, vp, dp],
            "imsrg_gpu_magnus_decouple_adjoint": [vp, vp, vp, d, d, i, i, i, C.POINTER(vp), dp, dp, ip, ip],
            "imsrg_gpu_magnus_decouple_checkpoint": [vp, vp, i, d, d, i, i, i, C.c_char_p, C.c_char_p, i, dp, ip,
                                                     ip, dp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.imsrg_gpu_strerror.argtypes = [C.c_int]
        L.imsrg_gpu_strerror.restype = C.c_char_p
        _lib = L
    return _lib


def strerror(status: int) -> str:
    return lib().imsrg_gpu_strerror(status).decode()


def _check(status: int, where: str):
    if status != 0:
        raise ImsrgError(status, where)


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


_F64 = np.dtype(np.float64)


def _addr(a: np.ndarray) -> int:
    """Address of an array's data for a void* argument (the cheapest route
    for writable arrays, whose buffer ctypes can wrap directly)."""
    return C.addressof(C.c_char.from_buffer(a)) if a.flags.writeable else a.ctypes.data


class Basis:
    """Device basis tables (imsrg_gpu_basis_create)."""

    def __init__(self, nn, ll, jj, itzp, con):
        arrs = [np.ascontiguousarray(x, np.int32) for x in (nn, ll, jj, itzp, con)]
        self._h = C.c_void_p()
        _check(lib().imsrg_gpu_basis_create(len(arrs[2]), *[a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs],
                                            C.byref(self._h)), "basis_create")
        info = BasisInfo()
        _check(lib().imsrg_gpu_basis_info(self._h, C.byref(info)), "basis_info")
        self.info = info
        self.nfull = info.nfull
        self.neq = info.neq
        self.norb = len(arrs[2])
        self.jj, self.con = arrs[2].copy(), arrs[4].copy()

    @classmethod
    def from_dict(cls, d):
        return cls(d["nn"], d["ll"], d["jj"], d["itzp"], d["con"])

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        _check(lib().imsrg_gpu_synchronize(self._h), "synchronize")

    def launch_count(self) -> int:
        n = C.c_long(0)
        _check(lib().imsrg_gpu_launch_count(self._h, C.byref(n)), "launch_count")
        return n.value

    def stream(self) -> int:
        """cudaStream_t (as an int) that all work of this basis runs on."""
        p = C.c_void_p()
        _check(lib().imsrg_gpu_basis_get_stream(self._h, C.byref(p)), "basis_get_stream")
        return p.value or 0

    def set_stream(self, stream: int | None):
        _check(lib().imsrg_gpu_basis_set_stream(self._h, C.c_void_p(stream or 0)), "basis_set_stream")

    def profile(self, on: bool = True):
        _check(lib().imsrg_gpu_profile_enable(self._h, int(on)), "profile_enable")

    def profile_reset(self):
        _check(lib().imsrg_gpu_profile_reset(self._h), "profile_reset")

    def profile_read(self) -> dict:
        """{kernel: (total_ms, launches)} since the last reset."""
        out = {}
        for k, name in enumerate(KERNELS):
            ms, n = C.c_double(), C.c_long()
            _check(lib().imsrg_gpu_profile_read(self._h, k, C.byref(ms), C.byref(n)), "profile_read")
            out[name] = (ms.value, n.value)
        return out

    def split_schedule(self):
        """(chosen model, [time in us of each candidate]) of the split engine's
        autotuned CTA schedule; available after the first split commutator."""
        ch, nc = C.c_int(), C.c_int()
        us = np.zeros(16)
        _check(lib().imsrg_gpu_split_schedule(self._h, C.byref(ch), C.byref(nc), _dp(us), 16), "split_schedule")
        return ch.value, us[:nc.value].tolist()

    def set_split_schedule(self, model: int):
        """Pin the split engine's CTA schedule to candidate `model` without
        timing (e.g. under a profiler whose serialised launches distort the
        autotuner's event timings); results do not depend on the schedule."""
        _check(lib().imsrg_gpu_split_schedule_set(self._h, int(model)), "split_schedule_set")

    def set_split_chunk(self, steps: int):
        """Cap the split engine's exact accumulator chunk at `steps` K steps
        (0: the default, the largest exact chunk); before the first split call."""
        _check(lib().imsrg_gpu_split_chunk_set(self.handle, int(steps)), "split_chunk_set")

    def set_split_digits(self, digits: int):
        """Digits per operand of the split engine on this basis: 6 (default,
        21 BF16 products), 5 (15 products), 4 (10 products), or the
        FP64-class 7 and 8 (28 and 36 products, every level exact); each
        digit fewer multiplies the truncation bound by 128.  Only before the
        basis' first split-precision call."""
        _check(lib().imsrg_gpu_split_digits_set(self._h, int(digits)), "split_digits_set")

    def block_dims(self, q):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(lib().imsrg_gpu_block_dims(self._h, q, C.byref(a), C.byref(b), C.byref(c)), "block_dims")
        return a.value, b.value, c.value

    def close(self):
        if self._h:
            lib().imsrg_gpu_basis_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Operator:
    """A scalar operator resident in HBM (sq_op)."""

    def __init__(self, basis: Basis, herm: int = 1, flat: np.ndarray | None = None):
        self.basis = basis
        self._h = C.c_void_p()
        _check(lib().imsrg_gpu_op_create(basis.handle, herm, C.byref(self._h)), "op_create")
        if flat is not None:
            self.upload(flat)

    @property
    def handle(self):
        return self._h

    @property
    def herm(self) -> int:
        h = C.c_int()
        _check(lib().imsrg_gpu_op_get_herm(self._h, C.byref(h)), "op_get_herm")
        return h.value

    @herm.setter
    def herm(self, v: int):
        _check(lib().imsrg_gpu_op_set_herm(self._h, int(v)), "op_set_herm")

    def upload(self, flat: np.ndarray):
        flat = np.ascontiguousarray(flat, np.float64)
        assert flat.size == self.basis.nfull
        _check(lib().imsrg_gpu_op_upload_flat(self._h, _dp(flat)), "op_upload_flat")

    def download(self, out: np.ndarray = None) -> np.ndarray:
        """The flat layout; into `out` (e.g. a pinned buffer) when given."""
        if out is None:
            out = np.empty(self.basis.nfull)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.basis.nfull
        _check(lib().imsrg_gpu_op_download_flat(self._h, _dp(out)), "op_download_flat")
        return out

    def save(self, path: str):
        """Checkpoint file: the packed (vectorize) vector as a raw stream."""
        _check(lib().imsrg_gpu_op_save(self._h, str(path).encode()), "op_save")

    def load(self, path: str):
        _check(lib().imsrg_gpu_op_load(self._h, str(path).encode()), "op_load")

    def upload_packed(self, vec: np.ndarray):
        vec = np.ascontiguousarray(vec, np.float64)
        assert vec.size == self.basis.neq
        _check(lib().imsrg_gpu_op_upload_packed(self._h, _dp(vec)), "op_upload_packed")

    def download_packed(self) -> np.ndarray:
        out = np.empty(self.basis.neq)
        _check(lib().imsrg_gpu_op_download_packed(self._h, _dp(out)), "op_download_packed")
        return out

    def upload_arrays(self, e0, fhh, fph, fpp, gams):
        """Fortran sq_op style: gams[(q-1)*6 + g-1] is gam(g) of block q (column-major)."""
        keep = [np.asfortranarray(x, np.float64) for x in (fhh, fph, fpp)]
        gk = [np.asfortranarray(g, np.float64) for g in gams]
        ptrs = (C.POINTER(C.c_double) * len(gk))(*[g.ctypes.data_as(C.POINTER(C.c_double)) for g in gk])
        _check(lib().imsrg_gpu_op_upload(self._h, float(e0), *[k.ctypes.data_as(C.POINTER(C.c_double)) for k in keep],
                                         ptrs), "op_upload")

    def download_arrays(self, shapes):
        """Inverse of upload_arrays; shapes = (fhh, fph, fpp, [gam shapes])."""
        fhh, fph, fpp = [np.zeros(s, order="F") for s in shapes[:3]]
        gk = [np.zeros(s, order="F") for s in shapes[3]]
        ptrs = (C.POINTER(C.c_double) * len(gk))(*[g.ctypes.data_as(C.POINTER(C.c_double)) for g in gk])
        e0 = C.c_double()
        _check(lib().imsrg_gpu_op_download(self._h, C.byref(e0), *[k.ctypes.data_as(C.POINTER(C.c_double))
                                                                  for k in (fhh, fph, fpp)], ptrs), "op_download")
        return e0.value, fhh, fph, fpp, gk

    def device_ptr(self) -> int:
        p = C.c_void_p()
        _check(lib().imsrg_gpu_op_device_ptr(self._h, C.byref(p)), "op_device_ptr")
        return p.value

    def e0(self) -> float:
        v = C.c_double()
        _check(lib().imsrg_gpu_op_get_e0(self._h, C.byref(v)), "op_get_e0")
        return v.value

    def close(self):
        if self._h:
            lib().imsrg_gpu_op_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --- reference-named operations -------------------------------------------
def copy_sq_op(src: Operator, dst: Operator):
    _check(lib().imsrg_gpu_op_copy(src.handle, dst.handle), "op_copy")


def clear_sq_op(op: Operator):
    _check(lib().imsrg_gpu_op_clear(op.handle), "op_clear")


def add_sq_op(A: Operator, ax: float, B: Operator, bx: float, C_: Operator):
    _check(lib().imsrg_gpu_op_add(A.handle, float(ax), B.handle, float(bx), C_.handle), "op_add")


def mat_frob_norm(op: Operator) -> float:
    v = C.c_double()
    _check(lib().imsrg_gpu_op_norm(op.handle, C.byref(v)), "op_norm")
    return v.value


def mbpt2(H: Operator) -> float:
    v = C.c_double()
    _check(lib().imsrg_gpu_op_mbpt2(H.handle, C.byref(v)), "op_mbpt2")
    return v.value


def commutator(L: Operator, R: Operator, RES: Operator, precision: str = "fp64", with_e0: bool = True):
    """[L, R] -> RES (RES herm = -herm(L) herm(R)); asynchronous on the basis stream."""
    _check(lib().imsrg_gpu_commutator(L.handle, R.handle, RES.handle, PREC[precision], int(with_e0)), "commutator")


def commutator_host(basis: Basis, L: np.ndarray, herm_L: int, R: np.ndarray, herm_R: int, RES: np.ndarray,
                    precision: str = "fp64", with_e0: bool = True):
    """[L, R] on host operands in the flat layout (RES written in place, herm
    -herm_L herm_R): copies in, commutator, copy out, one call.  Pinned
    (page-locked) buffers let the sequence replay as one CUDA graph."""
    n = basis.nfull
    for a in (L, R, RES):
        if a.dtype != _F64 or not a.flags.c_contiguous or a.size != n:
            raise ValueError(f"commutator_host: operands must be C-contiguous float64 arrays of {n} elements")
    _check(lib().imsrg_gpu_commutator_host(basis.handle, _addr(L), int(herm_L), _addr(R), int(herm_R), _addr(RES),
                                           PREC[precision], int(with_e0)), "commutator_host")


def commutator_host_packed(basis: Basis, L: np.ndarray, herm_L: int, R: np.ndarray, herm_R: int, RES: np.ndarray,
                           precision: str = "fp64", with_e0: bool = True):
    """[L, R] on host operands in the packed (vectorize) layout, neq doubles
    each.  Page-locked arrays the device can address (e.g. pinned torch
    tensors' numpy views) are read and written in place by the device's
    unpack and pack kernels; other arrays are copied in and out."""
    n = basis.neq
    for a in (L, R, RES):
        if a.dtype != _F64 or not a.flags.c_contiguous or a.size != n:
            raise ValueError(f"commutator_host_packed: operands must be C-contiguous float64 arrays of {n} elements")
    _check(lib().imsrg_gpu_commutator_host_packed(basis.handle, _addr(L), int(herm_L), _addr(R), int(herm_R),
                                                  _addr(RES), PREC[precision], int(with_e0)), "commutator_host_packed")


def commutator_noalloc(basis: Basis, d_L: int, herm_L: int, d_R: int, herm_R: int, d_RES: int,
                       with_e0: bool = True, stream: int | None = None):
    """FP64 [L, R] on caller-owned device buffers (flat layout) that allocates
    no device memory: for callers that may not allocate while they run.  The
    intermediates use one fixed 8 MiB library array (bases up to emax = 4);
    larger bases raise ImsrgError with status IMSRG_ERR_TOO_LARGE (9)."""
    _check(lib().imsrg_gpu_commutator_noalloc(basis.handle, C.c_void_p(d_L), int(herm_L), C.c_void_p(d_R),
                                              int(herm_R), C.c_void_p(d_RES), int(with_e0),
                                              C.c_void_p(stream or 0)), "commutator_noalloc")


def build_gs_white(H: Operator, ETA: Operator):
    _check(lib().imsrg_gpu_build_gs_white(H.handle, ETA.handle), "build_gs_white")


def magnus_expand(DG: Operator, G: Operator, precision: str = "fp64") -> int:
    n = C.c_int(0)
    _check(lib().imsrg_gpu_magnus_expand(DG.handle, G.handle, PREC[precision], C.byref(n)), "magnus_expand")
    return n.value


def bch_expand(HS: Operator, G: Operator, H: Operator, precision: str = "fp64") -> int:
    n = C.c_int(0)
    _check(lib().imsrg_gpu_bch_expand(HS.handle, G.handle, H.handle, PREC[precision], C.byref(n)), "bch_expand")
    return n.value


def euler_step(G: Operator, DG: Operator, s: float, ds: float) -> float:
    sv = C.c_double(s)
    _check(lib().imsrg_gpu_euler_step(G.handle, DG.handle, C.byref(sv), float(ds)), "euler_step")
    return sv.value


def magnus_decouple(HS: Operator, G: Operator, s_max: float = 50.0, ds: float = 0.5, max_steps: int = 1000,
                    precision: str = "fp64"):
    trace = np.zeros(5 * (max_steps + 1))
    steps, nc = C.c_int(0), C.c_int(0)
    _check(lib().imsrg_gpu_magnus_decouple(HS.handle, G.handle, float(s_max), float(ds), int(max_steps),
                                           PREC[precision], _dp(trace), C.byref(steps), C.byref(nc)),
           "magnus_decouple")
    n = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, trace=trace[:5 * n].reshape(n, 5))


def magnus_decouple_graph(HS: Operator, G: Operator, s_max: float = 50.0, ds: float = 0.5, max_steps: int = 1000,
                          precision: str = "fp64"):
    """magnus_decouple with one CUDA graph launch per Magnus step."""
    trace = np.zeros(5 * (max_steps + 1))
    steps, nc = C.c_int(0), C.c_int(0)
    _check(lib().imsrg_gpu_magnus_decouple_graph(HS.handle, G.handle, float(s_max), float(ds), int(max_steps),
                                                 PREC[precision], _dp(trace), C.byref(steps), C.byref(nc)),
           "magnus_decouple_graph")
    n = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, trace=trace[:5 * n].reshape(n, 5))


def magnus_rules(basis: Basis, lawson_beta: float = 0.0):
    """The reference's ds and checkpoint period of magnus_decouple
    (IMSRG_MAGNUS.f90:45-62) for this basis: (ds, chk)."""
    ds, chk = C.c_double(), C.c_int()
    _check(lib().imsrg_gpu_magnus_rules(basis.handle, float(lawson_beta), C.byref(ds), C.byref(chk)),
           "magnus_rules")
    return ds.value, chk.value


def magnus_decouple_checkpoint(HS: Operator, G: Operator, directory: str | None, prefix: str | None,
                               chk: int = 0, generator: str = "white", s_max: float = 50.0, ds: float = 0.5,
                               max_steps: int = 1000, precision: str = "fp64", graph: bool = False):
    """magnus_decouple writing Omega checkpoints every chk steps into
    directory (file names of checkpoint_name) and restarting from the newest
    one found there (IMSRG_MAGNUS.f90:56-110).  Returns steps (the final step
    counter), ncomm, s_restart (-1 without a restart) and the trace rows up to
    the final step (rows before a restart are left zero)."""
    gen = {"white": 0, "atan": 1, "w2": 2}[generator]
    trace = np.zeros(5 * (max_steps + 1))
    steps, nc, sx = C.c_int(0), C.c_int(0), C.c_double(0.0)
    _check(lib().imsrg_gpu_magnus_decouple_checkpoint(
        HS.handle, G.handle, gen, float(s_max), float(ds), int(max_steps), PREC[precision], int(bool(graph)),
        directory.encode() if directory is not None else None, prefix.encode() if prefix is not None else None,
        int(chk), _dp(trace), C.byref(steps), C.byref(nc), C.byref(sx)), "magnus_decouple_checkpoint")
    n = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, s_restart=sx.value, trace=trace[:5 * n].reshape(n, 5))


def commutator_adjoint(X: Operator, Cbar: Operator, herm_Y: int, Ybar: Operator, with_e0: bool = True):
    """Ybar = d<Cbar, [X, Y]>/dY for Y of hermiticity herm_Y (FP64)."""
    _check(lib().imsrg_gpu_commutator_adjoint(X.handle, Cbar.handle, int(herm_Y), int(bool(with_e0)),
                                              Ybar.handle), "commutator_adjoint")


def white_adjoint(H: Operator, ETAbar: Operator, Hbar: Operator):
    """Hbar = (d White(H) / dH)^T ETAbar."""
    _check(lib().imsrg_gpu_white_adjoint(H.handle, ETAbar.handle, Hbar.handle), "white_adjoint")


def op_dot(A: Operator, B: Operator) -> float:
    v = C.c_double()
    _check(lib().imsrg_gpu_op_dot(A.handle, B.handle, C.byref(v)), "op_dot")
    return v.value


def magnus_decouple_adjoint(HS: Operator, G: Operator, dirs: list, Hbar: Operator | None = None,
                            s_max: float = 50.0, ds: float = 0.5, max_steps: int = 1000, precision: str = "fp64"):
    """The Magnus flow (as magnus_decouple) and one backward sweep: grad[j] =
    dE0(s)/d(HS along dirs[j]); Hbar (optional) receives the whole gradient."""
    trace = np.zeros(5 * (max_steps + 1))
    steps, nc = C.c_int(0), C.c_int(0)
    n = len(dirs)
    arr = (C.c_void_p * max(n, 1))(*[x.handle for x in dirs])
    grad = np.zeros(max(n, 1))
    _check(lib().imsrg_gpu_magnus_decouple_adjoint(
        HS.handle, G.handle, Hbar.handle if Hbar is not None else None, float(s_max), float(ds), int(max_steps),
        PREC[precision], n, arr, _dp(grad), _dp(trace), C.byref(steps), C.byref(nc)), "magnus_decouple_adjoint")
    k = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, grad=grad[:n], trace=trace[:5 * k].reshape(k, 5))


def magnus_decouple_batch(HS: list, G: list, s_max: float = 50.0, ds: float = 0.5, max_steps: int = 1000,
                          precision: str = "fp64"):
    """Independent flows (one basis each) advanced together: a list of dicts
    as magnus_decouple returns, each with the instance's status."""
    n = len(HS)
    traces = [np.zeros(5 * (max_steps + 1)) for _ in range(n)]
    tp = (C.POINTER(C.c_double) * n)(*[_dp(t) for t in traces])
    hs = (C.c_void_p * n)(*[h.handle for h in HS])
    gs = (C.c_void_p * n)(*[g.handle for g in G])
    steps, nc, st = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
    rc = lib().imsrg_gpu_magnus_decouple_batch(n, hs, gs, float(s_max), float(ds), int(max_steps), PREC[precision],
                                               tp, steps, nc, st)
    out = []
    for i in range(n):
        k = steps[i] + 1
        out.append(dict(steps=steps[i], ncomm=nc[i], status=st[i], trace=traces[i][:5 * k].reshape(k, 5)))
    if rc != 0 and all(o["status"] == 0 for o in out):
        _check(rc, "magnus_decouple_batch")
    return out


def magnus_decouple_tangent(HS: Operator, dHS: Operator, G: Operator, dG: Operator, s_max: float = 50.0,
                            ds: float = 0.5, max_steps: int = 1000, precision: str = "fp64"):
    """The flow of HS with its derivative along dHS; dtrace[:, 2] is dE0."""
    trace, dtrace = np.zeros(5 * (max_steps + 1)), np.zeros(5 * (max_steps + 1))
    steps, nc = C.c_int(0), C.c_int(0)
    _check(lib().imsrg_gpu_magnus_decouple_tangent(HS.handle, dHS.handle, G.handle, dG.handle, float(s_max),
                                                   float(ds), int(max_steps), PREC[precision], _dp(trace),
                                                   _dp(dtrace), C.byref(steps), C.byref(nc)),
           "magnus_decouple_tangent")
    n = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, trace=trace[:5 * n].reshape(n, 5),
                dtrace=dtrace[:5 * n].reshape(n, 5))


GENERATORS = {"white": 0, "atan": 1, "w2": 2}


def build_gs_atan(H: Operator, ETA: Operator):
    _check(lib().imsrg_gpu_build_gs_atan(H.handle, ETA.handle), "build_gs_atan")


def build_gs_w2(H: Operator, ETA: Operator, precision: str = "fp64"):
    _check(lib().imsrg_gpu_build_gs_w2(H.handle, ETA.handle, PREC[precision]), "build_gs_w2")


def magnus_decouple_gen(HS: Operator, G: Operator, generator: str = "white", s_max: float = 50.0, ds: float = 0.5,
                        max_steps: int = 1000, precision: str = "fp64"):
    trace = np.zeros(5 * (max_steps + 1))
    steps, nc = C.c_int(0), C.c_int(0)
    _check(lib().imsrg_gpu_magnus_decouple_gen(HS.handle, G.handle, GENERATORS[generator], float(s_max), float(ds),
                                               int(max_steps), PREC[precision], _dp(trace), C.byref(steps),
                                               C.byref(nc)), "magnus_decouple_gen")
    n = steps.value + 1
    return dict(steps=steps.value, ncomm=nc.value, trace=trace[:5 * n].reshape(n, 5))


def checkpoint_name(directory: str, prefix: str, s: float) -> str:
    """The reference's Omega checkpoint file name for flow parameter s."""
    buf = C.create_string_buffer(512)
    _check(lib().imsrg_gpu_checkpoint_name(directory.encode(), prefix.encode(), float(s), buf, 512), "checkpoint_name")
    return buf.value.decode()


def normal_order(H: Operator):
    _check(lib().imsrg_gpu_normal_order(H.handle), "normal_order")


class Batch:
    """Independent commutators, one per basis, whose split-precision products
    run as one persistent launch (imsrg_gpu_batch_*)."""

    def __init__(self, bases: list):
        self.bases = list(bases)
        arr = (C.c_void_p * len(self.bases))(*[b.handle.value for b in self.bases])
        self._h = C.c_void_p()
        _check(lib().imsrg_gpu_batch_create(len(self.bases), arr, C.byref(self._h)), "batch_create")

    def commutator(self, L: list, R: list, RES: list, precision: str = "ozaki", with_e0: bool = True):
        """RES[i] = [L[i], R[i]] for every basis; returns when all are done."""
        n = len(self.bases)
        assert len(L) == len(R) == len(RES) == n
        arrs = [(C.c_void_p * n)(*[o.handle.value for o in ops]) for ops in (L, R, RES)]
        _check(lib().imsrg_gpu_batch_commutator(self._h, *arrs, PREC[precision], int(with_e0)), "batch_commutator")

    def magnus_decouple(self, HS: list, G: list, s_max: float = 50.0, ds: float = 0.5, max_steps: int = 1000,
                        precision: str = "ozaki"):
        """The instances' Magnus flows in lockstep, each step one CUDA graph
        for all of them and one merged product launch per series term
        (imsrg_gpu_batch_magnus_decouple): a list of dicts as
        magnus_decouple_batch returns."""
        n = len(self.bases)
        assert len(HS) == len(G) == n
        traces = [np.zeros(5 * (max_steps + 1)) for _ in range(n)]
        tp = (C.POINTER(C.c_double) * n)(*[_dp(t) for t in traces])
        hs = (C.c_void_p * n)(*[h.handle for h in HS])
        gs = (C.c_void_p * n)(*[g.handle for g in G])
        steps, nc, st = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
        rc = lib().imsrg_gpu_batch_magnus_decouple(self._h, hs, gs, float(s_max), float(ds), int(max_steps),
                                                   PREC[precision], tp, steps, nc, st)
        out = []
        for i in range(n):
            k = steps[i] + 1
            out.append(dict(steps=steps[i], ncomm=nc[i], status=st[i], trace=traces[i][:5 * k].reshape(k, 5)))
        if rc != 0 and all(o["status"] == 0 for o in out):
            _check(rc, "batch_magnus_decouple")
        return out

    def close(self):
        if self._h:
            _check(lib().imsrg_gpu_batch_destroy(self._h), "batch_destroy")
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _nucleons(basis: Basis) -> int:
    # A = sum over hole orbits of (2j + 1)
    return int(sum(j + 1 for j, c in zip(basis.jj, basis.con) if c == 1))


def read_interaction(H: Operator, path: str, htype: int = 1, hw: float = 20.0, com_hw: float | None = None,
                     lawson_beta: float = 0.0, mass: int | None = None):
    """read_interaction (interaction_IO.f90:8-107): H (herm +1) is cleared and
    filled with the two-body elements of the ASCII file at `path`, plus the
    centre-of-mass / Lawson terms of `htype`, `lawson_beta`, `com_hw` (default
    hw).  `mass` defaults to the reference's nucleon count."""
    m = _nucleons(H.basis) if mass is None else int(mass)
    _check(lib().imsrg_gpu_read_interaction(H.handle, os.fsencode(path), int(htype), float(hw),
                                            float(hw if com_hw is None else com_hw), float(lawson_beta), m),
           "read_interaction")


def h0_harm_osc(H: Operator, htype: int = 1, hw: float = 20.0, com_hw: float | None = None,
                lawson_beta: float = 0.0, mass: int | None = None):
    """calculate_h0_harm_osc (basic_IMSRG.f90:2049-2147): the HO one-body part
    of H for `htype` 1-5."""
    m = _nucleons(H.basis) if mass is None else int(mass)
    _check(lib().imsrg_gpu_h0_harm_osc(H.handle, int(htype), float(hw), float(hw if com_hw is None else com_hw),
                                       float(lawson_beta), m), "h0_harm_osc")


def hartree_fock(H: Operator, tol: float = 1e-6, max_iter: int = 1000) -> dict:
    """calc_HF (HF_mod.f90:14-106) without a three-body force: H (T + V, not
    normal ordered) becomes the normal-ordered Hamiltonian in the HF basis.
    Returns e_hf, the iteration count and the coefficients D (norb x norb,
    D[a, i] = weight of HO orbit a in HF orbit i)."""
    n = H.basis.norb
    e = C.c_double()
    it = C.c_int()
    D = np.zeros(n * n)
    _check(lib().imsrg_gpu_hartree_fock(H.handle, float(tol), int(max_iter), C.byref(e), C.byref(it), _dp(D)),
           "hartree_fock")
    return {"e_hf": e.value, "iterations": it.value, "coefs": D.reshape(n, n, order="F")}


def transform_to_hf(Op: Operator, coefs: np.ndarray):
    """observable_to_HF for a scalar operator (HF_mod.f90:108-136): Op (HO
    basis, not normal ordered, Hermitian) into the normal-ordered HF basis of
    the coefficients a hartree_fock call returned, in place."""
    D = np.ascontiguousarray(np.asarray(coefs, np.float64).reshape(-1, order="F") if np.ndim(coefs) == 2 else coefs,
                             np.float64)
    _check(lib().imsrg_gpu_transform_to_hf(Op.handle, _dp(D)), "transform_to_hf")


def dhds(HS: Operator, DH: Operator, generator: str = "white", precision: str = "fp64"):
    _check(lib().imsrg_gpu_dhds(HS.handle, DH.handle, GENERATORS[generator], PREC[precision]), "dhds")


def ode_decouple(HS: Operator, generator: str = "white", precision: str = "fp64", ds: float = 0.1,
                 s_max: float = 0.0, max_steps: int = 10000, relerr: float = 1e-6, abserr: float = 1e-6):
    """decouple_hamiltonian (IMSRG_ODE.f90:9-178): the Shampine-Gordon flow of
    HS (advanced in place) in output steps of ds until |E_mbpt2| < 1e-6 (or
    s >= s_max > 0, or max_steps).  Returns steps, the trace rows (step, s, E0,
    E0 + E_mbpt2, |E_mbpt2|) and the number of derivative evaluations."""
    trace = np.zeros(5 * (max_steps + 1))
    st, nf = C.c_int(0), C.c_long(0)
    _check(lib().imsrg_gpu_ode_decouple(HS.handle, GENERATORS[generator], PREC[precision], float(ds), float(s_max),
                                        int(max_steps), float(relerr), float(abserr), _dp(trace), C.byref(st),
                                        C.byref(nf)), "ode_decouple")
    return dict(steps=st.value, trace=trace[:5 * (st.value + 1)].reshape(-1, 5), nfev=nf.value)


def transform_bch(Op: Operator, G: Operator, precision: str = "fp64") -> int:
    n = C.c_int(0)
    _check(lib().imsrg_gpu_transform_bch(Op.handle, G.handle, PREC[precision], C.byref(n)), "transform_bch")
    return n.value
