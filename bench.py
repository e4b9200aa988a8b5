#!/usr/bin/env python
"""Benchmark: J-coupled IMSRG(2) [Omega, H] commutators per second at emax = 6.

Workload: one scalar-scalar commutator [Omega, H] (Omega anti-Hermitian,
H Hermitian) in the 16O harmonic-oscillator basis with emax = 6 (56 j-orbits,
84 (2J,Tz,parity) blocks, 850,034 two-body doubles per operator), exactly the
sequence 110+220, 111, 121, 122, 222_pp_hh, 221, 222_ph with both Pandya
transforms.  Inputs are seeded synthetic operators (see imsrg_gpu.synth).
A step is one commutator; L2 is flushed (a 256 MiB write) between timed
steps, because one operator pair plus workspace is smaller than L2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs N independent replicas (one per GPU, launched by torchrun); the
commutator of one Hamiltonian does not shard.  Rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "eom-imsrg_full_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "emax=6 [Ω,H] commutators/s, split-prec vs FP64 GPU at |ΔE0|<1e-6 MeV"
UNIT = "commutators/s"
EMAX = 6
SPLIT_DIGITS = 5  # digits per operand of the split engine (set from --split-digits)


def _workload_flops(lay):
    """Algorithmic FLOPs of the dense contractions of one commutator: the
    twelve ladder products per block of 222_pp_hh plus WCC = LCC RCC^T per
    cross-coupled block (2mnk each)."""
    f = 0
    for b in lay.blocks:
        np_, nb, nh = b.npp, b.nph, b.nhh
        f += 2 * (np_ ** 3 + nh ** 3)
        f += 2 * (nh * nh * np_ + np_ * np_ * nh + 2 * np_ * nh * np_ + 2 * np_ * nh * nh)
        f += 2 * (nb * nb * nh + 2 * nb * nh * nh + nb * nb * np_ + 2 * np_ * nb * np_)
        f += 2 * (2 * nb * nh * np_ + 2 * np_ * nb * nh)
    return f


def _cc_flops(orb):
    """2 * rlen^2 * nph summed over cross-coupled blocks (222_ph product)."""
    import numpy as np
    nn, ll, jj, tz, con = (np.asarray(orb[k]) for k in ("nn", "ll", "jj", "itzp", "con"))
    N = len(jj)
    jtm = int(jj.max())
    f = 0
    for q1 in range(4 * (jtm + 1)):
        JC = (q1 % (jtm + 1)) * 2
        PAR = q1 // (2 * jtm + 2)
        TZ = (q1 % (2 * jtm + 2)) // (jtm + 1)
        r = nb = 0
        for i in range(N):
            for j in range(N):
                if not (abs(jj[i] - jj[j]) <= JC <= jj[i] + jj[j]):
                    continue
                if (ll[i] + ll[j]) % 2 != PAR or abs(tz[i] - tz[j]) // 2 != TZ:
                    continue
                r += 1
                nb += int(con[i] == 0 and con[j] == 1)
        f += 2 * r * r * nb
    return f


def _compulsory_bytes(lay):
    """Read L and R, write RES: 3 x nfull doubles."""
    return 3 * lay.nfull * 8


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]
        return False

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x: float, device: str) -> float:
    """The largest x over the ranks of the default process group (x itself
    without one): each replica's timed region, so the whole job is as slow as
    its slowest replica."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(steps_per_rank: int, world: int, max_ms: float) -> float:
    """Commutators per second of all replicas together (weak scaling: each
    rank runs `steps_per_rank` steps of its own Hamiltonian)."""
    return world * steps_per_rank / (max_ms / 1e3)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_oracle(orb, threads: int):
    """The fastest CPU configuration of the oracle (the C restatement of the
    reference's CPU path) on `threads` OpenMP threads: its timed build
    (-O3, contraction allowed) with its own blocked GEMM, or with numpy's
    bundled OpenBLAS dgemm (the reference links a system BLAS).  Each is timed
    for about two seconds on the emax=6 commutator; returns (oracle, label,
    {label: commutators/s})."""
    from oracle import oracle
    from imsrg_gpu.layout import Layout
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    oracle.set_threads(threads)
    lay = Layout(**orb)
    Hh, Oh = synth_hamiltonian(lay, 1), synth_omega(lay, 1)
    rates = {}
    for label in ("own blocked GEMM", "OpenBLAS"):
        if label == "OpenBLAS":
            desc = oracle.use_blas(threads)
            if desc is None:
                break
            label = "OpenBLAS dgemm (" + " ".join(desc.split()[:2]) + ", numpy's ILP64 build)"
        orc = oracle.Oracle(**orb, variant="fast")
        orc.commutator(Oh, -1, Hh, 1)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 2.0:
            orc.commutator(Oh, -1, Hh, 1)
            n += 1
        rates[label] = n / (time.perf_counter() - t0)
    best = max(rates, key=rates.get)
    if not best.startswith("OpenBLAS"):
        oracle.lib("fast").orc_set_dgemm(None)
    return oracle.Oracle(**orb, variant="fast"), best, rates


def cpu_baseline(orb, lay, seconds: float = 12.0, threads: int | None = None):
    """The oracle (C restatement of the reference CPU path) on host cores, in
    its fastest configuration (cpu_oracle)."""
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    threads = threads or os.cpu_count()
    orc, blas, rates = cpu_oracle(orb, threads)
    Hh, Oh = synth_hamiltonian(lay, 1), synth_omega(lay, 1)
    orc.commutator(Oh, -1, Hh, 1)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        orc.commutator(Oh, -1, Hh, 1)
        n += 1
        dt = time.perf_counter() - t0
        if dt >= seconds or n >= 400:
            break
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} emax=6 [Omega,H] commutators in {dt:.1f} s (OpenMP C oracle, -O3 -ffp-contract=fast, "
                      f"{blas})",
            "blas": blas, "calibration_rates": rates}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from imsrg_gpu.layout import Layout, ho_basis
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    from oracle import oracle
    orb = ho_basis(EMAX)
    lay = Layout(**orb)
    threads = os.cpu_count()
    orc, blas, rates = cpu_oracle(orb, threads)
    Hh, Oh = synth_hamiltonian(lay, 1), synth_omega(lay, 1)
    for _ in range(args.warmup):
        orc.commutator(Oh, -1, Hh, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.commutator(Oh, -1, Hh, 1)
    dt = time.perf_counter() - t0
    value = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "emax=6 [Omega,H] commutator, 16O, 56 j-orbits", "emax": EMAX},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} commutators after {args.warmup} warm-up (OpenMP C oracle, "
                                   f"-O3 -ffp-contract=fast, {blas})", "blas": blas, "calibration_rates": rates},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, world, rank, local):
    import numpy as np
    import torch

    from imsrg_gpu import api
    from imsrg_gpu.layout import Layout, ho_basis
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    orb = ho_basis(EMAX)
    lay = Layout(**orb)
    B = api.Basis.from_dict(orb)
    B.set_split_digits(SPLIT_DIGITS)
    Hh, Oh = synth_hamiltonian(lay, 1 + rank), synth_omega(lay, 1 + rank)
    O, H, RES = api.Operator(B, -1, Oh), api.Operator(B, 1, Hh), api.Operator(B, 1)
    RES64 = api.Operator(B, 1)
    stream = torch.cuda.ExternalStream(B.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    precision = args.precision
    if args.split_schedule is not None and precision != "fp64":
        B.set_split_schedule(args.split_schedule)
    if precision == "auto":
        try:
            api.commutator(O, H, RES, precision="ozaki")
            B.synchronize()
            precision = "ozaki"
        except api.ImsrgError:
            precision = "fp64"

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            api.commutator(O, H, RES, precision=prec)
        B.synchronize()
        launches0 = B.launch_count()
        total = 0.0
        with ClockSampler(local) as clk:
            for _ in range(steps):
                flush.fill_(1.0)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                api.commutator(O, H, RES, precision=prec)
                e1.record(stream)
                e1.synchronize()
                total += e0.elapsed_time(e1)
        launches = B.launch_count() - launches0
        # per-kernel times: a profiled pass of the same workload right after
        # (CUDA events around every kernel class on the library's streams;
        # profiling replays the launches one by one instead of the cached graph)
        B.profile_reset()
        B.profile(True)
        for _ in range(min(steps, 200)):
            # the flush runs on the library's stream, in order with the
            # commutators (overlapping none of their kernels); while it runs
            # the host enqueues the commutator's launches, so the kernel times
            # carry no host launch latency (profiling replays launches one by
            # one instead of the cached graph)
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            api.commutator(O, H, RES, precision=prec)
        B.synchronize()
        prof = B.profile_read()
        B.profile(False)
        return total, launches, prof, clk.summary()

    if world > 1:
        torch.distributed.barrier()
    total_ms, launches, prof, clocks = timed(precision, args.steps, args.warmup)
    total_ms = max_over_ranks(total_ms, "cuda")
    value = whole_job_rate(args.steps, world, total_ms)

    # FP64 path beside the split-precision one, and their difference
    extra = {}
    if precision != "fp64":
        n64 = max(min(args.steps // 2, 500), 3)
        t64, _, prof64, _ = timed("fp64", n64, 3)
        extra["fp64_value"] = n64 / (t64 / 1e3)
        api.commutator(O, H, RES, precision=precision)
        api.commutator(O, H, RES64, precision="fp64")
        a, b_ = RES.download(), RES64.download()
        extra["split_vs_fp64"] = {"abs_dE0_MeV": abs(float(a[0] - b_[0])),
                                  "max_rel_elem": float(np.max(np.abs(a - b_)) / np.max(np.abs(b_)))}
    else:
        extra["fp64_value"] = value

    # roofline of the dominant kernel class: the class with the most device
    # time per commutator, timed live with CUDA events on the library's stream
    # (the profiled pass issues every launch on that one stream, so each event
    # pair times its kernels alone).  A class may launch more than one kernel
    # per commutator (slicing: three parts; two-body assembly: recoupling
    # inputs + assembly), so times and work are per commutator.
    n_prof = min(args.steps, 200)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6795.5)
    bf16_peak = peaks.get("bf16_tflops", 1951.5)
    comp = _compulsory_bytes(lay)
    alg_flops = _workload_flops(lay) + _cc_flops(orb)
    # the split engine keeps digit products d_s d_t with s + t <= S + 1
    nprod = SPLIT_DIGITS * (SPLIT_DIGITS + 1) // 2

    def roof_of(k, per):
        """One class against its bound: the contraction kernel against the
        tensor peak with the BF16 flops its 21 digit products execute (and the
        FP64-equivalent algorithmic flops beside them), the gather kernels
        against HBM with the compulsory bytes of one commutator."""
        if k.startswith("ozaki_mma"):
            return {"bound": "tensor", "achieved": nprod * alg_flops / per / 1e12, "peak": bf16_peak,
                    "unit": "TFLOP/s", "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)",
                    "achieved_fp64_equiv_tflops": alg_flops / per / 1e12,
                    "algorithmic_per_launch": nprod * alg_flops,
                    "work_note": f"executed BF16 flops = {nprod} digit products (S(S+1)/2, S = {SPLIT_DIGITS} "
                                 f"digits) x {alg_flops:.3e} FP64-equivalent flop"}
        if k == "gemm_fp64":
            return {"bound": "fp64", "achieved": alg_flops / per / 1e12, "peak": _fp64_peak_tflops(),
                    "unit": "TFLOP/s", "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (FP64 pipe)",
                    "algorithmic_per_launch": alg_flops}
        return {"bound": "hbm", "achieved": comp / per / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)", "algorithmic_per_launch": comp,
                "work_note": "compulsory bytes of one commutator: read L and R, write RES"}

    per_comm = {k: (ms_k / 1e3) / n_prof for k, (ms_k, n_k) in prof.items() if n_k}
    kname = max(per_comm, key=per_comm.get)
    roof = {"kernel": kname}
    roof.update(roof_of(kname, per_comm[kname]))
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["traffic"] = _traffic_from_profiles(kname)
    roof["per_launch_us"] = per_comm[kname] * 1e6
    roof["all_kernels"] = {}
    for k, per in per_comm.items():
        r = roof_of(k, per)
        roof["all_kernels"][k] = {"bound": r["bound"], "per_launch_us": per * 1e6, "event_pairs_per_commutator":
                                  prof[k][1] / n_prof, "achieved": r["achieved"], "unit": r["unit"],
                                  "frac": r["achieved"] / r["peak"], "traffic": _traffic_from_profiles(k)}
    roof["kernel_share"] = {k: round(v / max(sum(per_comm.values()), 1e-12), 4) for k, v in per_comm.items()}
    if precision != "fp64":
        # the FP64 arm's classes (the denominator of split vs FP64): its
        # contraction kernel against the live cuBLAS DGEMM rate
        n_prof64 = min(n64, 200)
        per64 = {k: (ms_k / 1e3) / n_prof64 for k, (ms_k, n_k) in prof64.items() if n_k}
        extra["fp64_roofline"] = {}
        for k, per in per64.items():
            r = roof_of(k, per)
            extra["fp64_roofline"][k] = {"bound": r["bound"], "per_launch_us": per * 1e6, "achieved": r["achieved"],
                                         "unit": r["unit"], "peak": r["peak"], "frac": r["achieved"] / r["peak"],
                                         "peak_source": r["peak_source"]}

    # end to end through the C ABI with pinned host buffers, in both host
    # layouts of the reference's operators: the flat sq_op arrays
    # (imsrg_gpu_commutator_host) and the packed vectorize vector
    # (imsrg_gpu_commutator_host_packed, independent elements only); one call
    # per step copies Omega and H in, runs the commutator and copies RES out,
    # returning when RES is in host memory
    def pinned(n):
        return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    n_e2e = max(min(args.steps // 2, 500), 3)
    e2e_modes = {}
    for mode in ("flat", "packed"):
        if mode == "flat":
            nel, call = lay.nfull, api.commutator_host
            src_o, src_h = Oh, Hh
        else:
            nel, call = B.neq, api.commutator_host_packed
            src_o, src_h = O.download_packed(), H.download_packed()
        pin_o, pin_h, pin_r = pinned(nel), pinned(nel), pinned(nel)
        pin_o[:], pin_h[:] = src_o, src_h
        for _ in range(2):
            call(B, pin_o, -1, pin_h, 1, pin_r, precision=precision)
        B.synchronize()
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            call(B, pin_o, -1, pin_h, 1, pin_r, precision=precision)
        dt_ = time.perf_counter() - t0
        e2e_modes[mode] = {"value": world * n_e2e / dt_, "unit": UNIT, "h2d_bytes_per_step": 2 * nel * 8,
                           "d2h_bytes_per_step": nel * 8,
                           "call": "imsrg_gpu_commutator_host" + ("_packed" if mode == "packed" else "")}
    best = max(e2e_modes, key=lambda m: e2e_modes[m]["value"])
    e2e = dict(e2e_modes[best])
    e2e["host_layout"] = best
    e2e["other_layout"] = e2e_modes["packed" if best == "flat" else "flat"]

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precision == "fp64" else "bf16-slices/f64",
            "data": "synthetic (seeded HO basis, hw=20 MeV, N(0,1) MeV two-body, N(0,0.05) Omega)",
            "config": {"workload": "emax=6 [Omega,H] commutator, 16O, 56 j-orbits", "emax": EMAX,
                       "precision": precision, "split_digits": args.split_digits if precision == "ozaki" else None,
                       "parallelism": f"replicas x{world}",
                       "l2": "flushed between timed steps (256 MiB write)", "nfull": lay.nfull},
            "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
        }
        if precision == "ozaki":
            choice, us = B.split_schedule()
            line["split_schedule_autotune"] = {"chosen_model": choice, "candidate_us": us,
                                               "pinned": args.split_schedule is not None}
        line.update(extra)
        if not args.no_flows:
            line["flow"] = flow_emax6(api, orb, lay, args.split_digits)
            line["fp64_class"] = fp64_class_extra(api, orb, lay, flush)
            line["ode"] = ode_emax6(api, orb, lay)
            line["hartree_fock"] = hf_emax6(api, orb, lay)
            line["batch"] = batch_flows(api, args.batch)
            line["batched_commutators"] = batched_commutators(api)
            line["adjoint"] = adjoint_extra(api)
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(orb, lay, seconds=args.cpu_seconds)
            # the same oracle on one core (the reference itself threads only
            # the Pandya transform and 222_ph)
            line["cpu_baseline_1thread"] = cpu_baseline(orb, lay, seconds=args.cpu_seconds / 2, threads=1)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def fp64_class_extra(api, orb, lay, flush, steps=100):
    """Eight-digit split precision (every digit level exact: FP64-class
    accuracy) beside the FP64 path on the benchmark's commutator: each path's
    commutators/s (CUDA events on the library's stream, the L2 flushed between
    steps), the eight-digit result's largest element difference from the FP64
    path, and the emax = 6 flow to s = 50 at eight digits against the FP64
    oracle flow (flow_emax6)."""
    import numpy as np
    import torch
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    B = api.Basis.from_dict(orb)
    B.set_split_digits(8)
    O, H = api.Operator(B, -1, synth_omega(lay, 1)), api.Operator(B, 1, synth_hamiltonian(lay, 1))
    res = {p: api.Operator(B, 1) for p in ("ozaki", "fp64")}
    stream = torch.cuda.ExternalStream(B.stream())
    out = {"split_digits": 8, "steps": steps, "l2": "flushed between timed steps"}
    for prec in ("ozaki", "fp64"):
        for _ in range(5):
            api.commutator(O, H, res[prec], precision=prec)
        B.synchronize()
        total = 0.0
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            api.commutator(O, H, res[prec], precision=prec)
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1) / 1e3
        out[prec + "_commutators_per_s"] = steps / total
    a, b = res["ozaki"].download(), res["fp64"].download()
    out["max_rel_elem_vs_fp64"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    out["abs_dE0_vs_fp64_MeV"] = abs(float(a[0] - b[0]))
    out["speedup_vs_fp64"] = out["ozaki_commutators_per_s"] / out["fp64_commutators_per_s"]
    f = flow_emax6(api, orb, lay, 8)
    out["flow"] = {k: f["ozaki"][k] for k in ("steps", "commutators", "seconds", "commutators_per_s",
                                             "max_abs_dE0_vs_oracle_MeV", "omega_norm_rel_err_vs_oracle")}
    return out


def flow_emax6(api, orb, lay, digits=5):
    """The emax = 6 Magnus flow to s = 50 (graph-captured steps) of the
    normal-ordered seed-13 synthetic H in split precision and in FP64: steps,
    commutators, wall time, and each flow's errors against the FP64 oracle
    flow of the same H (tests/golden/emax6_flow.npz, written by
    tests/golden/make_golden.py and checked against the oracle by
    tests/test_gpu_parity_headline.py): the largest |dE0| over all steps and
    the relative error of the final Omega's norm (mat_frob_norm)."""
    import numpy as np
    from imsrg_gpu.synth import synth_hamiltonian
    B = api.Basis.from_dict(orb)
    B.set_split_digits(digits)
    H0 = api.Operator(B, 1, synth_hamiltonian(lay, 13))
    api.normal_order(H0)
    Hh = H0.download()
    ref = np.load(os.path.join(ROOT, "tests", "golden", "emax6_flow.npz"))
    out = {"emax": EMAX, "s_max": 50.0, "ds": 0.5, "graph_steps": True, "split_digits": digits,
           "reference": "FP64 oracle flow (tests/golden/emax6_flow.npz)",
           "oracle_steps": int(ref["steps"]), "oracle_e0_MeV": float(ref["trace"][-1, 2]),
           "oracle_omega_norm": float(ref["omega_norm"])}
    for prec in ("ozaki", "fp64"):
        HS, G = api.Operator(B, 1, Hh), api.Operator(B, -1)
        api.magnus_decouple_graph(HS, G, s_max=0.5, ds=0.5, precision=prec)  # builds the step graph
        HS.upload(Hh)
        B.synchronize()
        t0 = time.perf_counter()
        r = api.magnus_decouple_graph(HS, G, s_max=50.0, ds=0.5, precision=prec)
        dt = time.perf_counter() - t0
        tr = r["trace"]
        same = tr.shape == ref["trace"].shape
        nrm = api.mat_frob_norm(G)
        out[prec] = {"steps": r["steps"], "commutators": r["ncomm"], "e0_MeV": float(tr[-1, 2]),
                     "seconds": dt, "commutators_per_s": r["ncomm"] / dt,
                     "max_abs_dE0_vs_oracle_MeV": float(np.max(np.abs(tr[:, 2] - ref["trace"][:, 2])))
                     if same else None,
                     "omega_norm": nrm,
                     "omega_norm_rel_err_vs_oracle": abs(nrm - float(ref["omega_norm"])) / float(ref["omega_norm"])}
    out["abs_dE0_split_vs_fp64_MeV"] = abs(out["ozaki"]["e0_MeV"] - out["fp64"]["e0_MeV"])
    return out


def adjoint_extra(api):
    """dE0/dc_k for H(c) = T + sum_k c_k V_k (imsrg_gpu.synth.adjoint_terms,
    c = 1) of the Magnus flow to |E_mbpt2| < 1e-6 (s_max 50, ds 0.5): one
    backward sweep of imsrg_gpu_magnus_decouple_adjoint for all four c_k
    against four tangent-linear flows, at emax = 4 (gradients compared with the
    oracle's central differences, tests/golden/adjoint_fd_emax4.npz) and
    emax = 6 (timing).  Wall times after a short warm-up flow of each kind."""
    import numpy as np
    from imsrg_gpu.layout import Layout, ho_basis
    from imsrg_gpu.synth import adjoint_terms
    ref = np.load(os.path.join(ROOT, "tests", "golden", "adjoint_fd_emax4.npz"))
    out = {"workload": "H(c) = T + sum_k c_k V_k, four N(0,1) MeV two-body V_k, c = 1",
           "reference": "FP64 oracle central differences, h = 1e-4 (tests/golden/adjoint_fd_emax4.npz)"}
    for emax in (4, 6):
        orb = ho_basis(emax)
        lay = Layout(**orb)
        B = api.Basis.from_dict(orb)
        B.set_split_digits(SPLIT_DIGITS)
        T, V = adjoint_terms(lay)
        H = api.Operator(B, 1, T + sum(V))
        api.normal_order(H)
        H0 = H.download()
        dirs = []
        for v in V:
            d = api.Operator(B, 1, v)
            api.normal_order(d)
            dirs.append(d)
        for prec in ("fp64", "ozaki"):
            api.magnus_decouple_adjoint(api.Operator(B, 1, H0), api.Operator(B, -1), dirs, s_max=1.0,
                                        precision=prec)
            api.magnus_decouple_tangent(api.Operator(B, 1, H0), api.Operator(B, 1, dirs[0].download()),
                                        api.Operator(B, -1), api.Operator(B, -1), s_max=1.0, precision=prec)
            B.synchronize()
            t0 = time.perf_counter()
            adj = api.magnus_decouple_adjoint(api.Operator(B, 1, H0), api.Operator(B, -1), dirs, s_max=50.0,
                                              precision=prec)
            t_adj = time.perf_counter() - t0
            tan = []
            t0 = time.perf_counter()
            for d in dirs:
                r = api.magnus_decouple_tangent(api.Operator(B, 1, H0), api.Operator(B, 1, d.download()),
                                                api.Operator(B, -1), api.Operator(B, -1), s_max=50.0,
                                                precision=prec)
                tan.append(float(r["dtrace"][-1, 2]))
            t_tan = time.perf_counter() - t0
            rec = {"steps": adj["steps"], "flow_commutators": adj["ncomm"], "adjoint_s": t_adj,
                   "tangent_x4_s": t_tan, "adjoint_speedup": t_tan / t_adj,
                   "dE0_dc": [float(x) for x in adj["grad"]],
                   "max_rel_diff_adjoint_vs_tangent": float(np.max(np.abs(adj["grad"] - tan) / np.abs(tan)))}
            if emax == 4:
                rec["max_rel_err_vs_oracle_fd"] = float(np.max(np.abs(adj["grad"] - ref["fd"]) / np.abs(ref["fd"])))
            out[f"emax{emax}_{prec}"] = rec
    return out


def ode_emax6(api, orb, lay):
    """The emax = 6 ODE flow (decouple_hamiltonian with the Shampine-Gordon
    solver, ds = 0.1, tolerances 1e-6) to |E_mbpt2| < 1e-6 in split precision
    and in FP64: E0 difference, output steps, derivative evaluations (one
    generator + one commutator each), wall time."""
    from imsrg_gpu.synth import synth_hamiltonian
    B = api.Basis.from_dict(orb)
    # six digits: the adaptive step control feeds rounding differences back
    # into the step sizes (|dE0| vs FP64 measured 1.2e-7 MeV with six digits,
    # 1.3e-6 MeV with five)
    B.set_split_digits(6)
    Hh = synth_hamiltonian(lay, 13)
    out = {"emax": EMAX, "ds": 0.1, "relerr": 1e-6, "abserr": 1e-6, "split_digits": 6}
    for prec in ("ozaki", "fp64"):
        HS = api.Operator(B, 1, Hh)
        api.ode_decouple(api.Operator(B, 1, Hh), precision=prec, s_max=0.1)  # warm-up (plans, graphs)
        B.synchronize()
        t0 = time.perf_counter()
        r = api.ode_decouple(HS, precision=prec, max_steps=2000)
        dt = time.perf_counter() - t0
        out[prec] = {"steps": r["steps"], "s": float(r["trace"][-1, 1]), "derivatives": r["nfev"],
                     "e0_MeV": float(r["trace"][-1, 2]), "seconds": dt, "derivatives_per_s": r["nfev"] / dt}
    out["abs_dE0_MeV"] = abs(out["ozaki"]["e0_MeV"] - out["fp64"]["e0_MeV"])
    return out


def hf_emax6(api, orb, lay):
    """The setup before the flow at emax = 6: the synthetic two-body part
    written as an ASCII interaction file, read back with the centre-of-mass
    terms (htype 1), the HO one-body part, Hartree-Fock to 1e-6, then the
    split-precision Magnus flow to s = 50 from the HF basis (wall times)."""
    import tempfile
    from imsrg_gpu.synth import synth_hamiltonian, write_vrenorm
    V = synth_hamiltonian(lay, 13, sigma2=0.5)
    V[:lay.off_fpp + lay.P * lay.P] = 0.0
    B = api.Basis.from_dict(orb)
    B.set_split_digits(SPLIT_DIGITS)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "v.int")
        nlines = write_vrenorm(lay, V, path, seed=13)
        H = api.Operator(B, 1)
        t0 = time.perf_counter()
        api.read_interaction(H, path, htype=1, hw=20.0)
        t1 = time.perf_counter()
    api.h0_harm_osc(H, htype=1, hw=20.0)
    B.synchronize()
    t2 = time.perf_counter()
    r = api.hartree_fock(H, tol=1e-6)
    t3 = time.perf_counter()
    G = api.Operator(B, -1)
    f = api.magnus_decouple_graph(H, G, s_max=50.0, ds=0.5, precision="ozaki")
    t4 = time.perf_counter()
    return {"emax": EMAX, "file_lines": nlines, "read_s": t1 - t0, "hf_s": t3 - t2, "hf_iterations": r["iterations"],
            "e_hf_MeV": r["e_hf"], "flow_steps": f["steps"], "flow_s": t4 - t3,
            "e0_after_flow_MeV": float(f["trace"][-1, 2])}


def batched_commutators(api, n=64, reps=20):
    """n independent Hamiltonians (hbar*omega ~ U[12,28] MeV, two-body scale
    ~ U[0.5,2] MeV, emax cycling 2, 4, 6): [Omega_i, H_i] for all of them per
    step, (a) as one batch (the split-precision products of every instance in
    one persistent launch, or in FP64 one grouped FP64 launch; one graph per
    step) and (b) as n single commutators
    issued back to back on the instances' own streams (each its own graph),
    then a synchronisation.  Same results (bit for bit); wall time per step."""
    import numpy as np
    from imsrg_gpu.layout import Layout, ho_basis
    from imsrg_gpu.synth import synth_hamiltonian, synth_omega
    rng = np.random.default_rng(64)
    bases, L, R, RES, emaxes = [], [], [], [], []
    t0 = time.perf_counter()
    for k in range(n):
        emax = (2, 4, 6)[k % 3]
        orb = ho_basis(emax)
        lay = Layout(**orb)
        B = api.Basis.from_dict(orb)
        B.set_split_digits(SPLIT_DIGITS)
        hw, sig = float(rng.uniform(12.0, 28.0)), float(rng.uniform(0.5, 2.0))
        bases.append(B)
        L.append(api.Operator(B, -1, synth_omega(lay, 2000 + k)))
        R.append(api.Operator(B, 1, synth_hamiltonian(lay, 2000 + k, hw=hw, sigma2=sig)))
        RES.append(api.Operator(B, 1))
        emaxes.append(emax)
    setup_s = time.perf_counter() - t0
    batch = api.Batch(bases)
    out = {"instances": n, "emax_counts": {e: emaxes.count(e) for e in (2, 4, 6)}, "setup_s": setup_s,
           "precision": "ozaki", "reps": reps}

    def timed(prec):
        for _ in range(3):  # graphs, autotuning of each instance's own schedule
            batch.commutator(L, R, RES, precision=prec)
            for i in range(n):
                api.commutator(L[i], R[i], RES[i], precision=prec)
            for B in bases:
                B.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            batch.commutator(L, R, RES, precision=prec)
        tb = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            for i in range(n):
                api.commutator(L[i], R[i], RES[i], precision=prec)
            for B in bases:
                B.synchronize()
        ts = (time.perf_counter() - t0) / reps
        return tb, ts

    tb, ts = timed("ozaki")
    out.update({"batch_ms_per_step": tb * 1e3, "batch_commutators_per_s": n / tb,
                "single_calls_ms_per_step": ts * 1e3, "single_calls_commutators_per_s": n / ts})
    # FP64: the products of every instance in one grouped FP64 launch
    tb, ts = timed("fp64")
    out["fp64"] = {"batch_ms_per_step": tb * 1e3, "batch_commutators_per_s": n / tb,
                   "single_calls_ms_per_step": ts * 1e3, "single_calls_commutators_per_s": n / ts}
    batch.close()
    return out


def batch_flows(api, n):
    """n independent seeded Hamiltonians (hbar*omega ~ U[12,28] MeV, two-body
    scale ~ U[0.5,2] MeV, emax cycling 2, 4, 6), Magnus flows to s = 50 in
    split precision advanced together, two ways:
    (a) interleaved: one step graph per instance per round, each instance's
        products in its own launches (imsrg_gpu_magnus_decouple_batch);
    (b) lockstep: one graph per step for all instances, every series term's
        products of all instances in one merged launch
        (imsrg_gpu_batch_magnus_decouple), timed on a second call that reuses
        the step graph (the first call's time, capture included, beside it).
    Both give each instance's unbatched flow bit for bit (checked here)."""
    import numpy as np
    from imsrg_gpu.layout import Layout, ho_basis
    from imsrg_gpu.synth import synth_hamiltonian
    rng = np.random.default_rng(64)
    H0, bases, emaxes = [], [], []
    for k in range(n):
        emax = (2, 4, 6)[k % 3]
        orb = ho_basis(emax)
        lay = Layout(**orb)
        B = api.Basis.from_dict(orb)
        B.set_split_digits(SPLIT_DIGITS)
        hw, sig = float(rng.uniform(12.0, 28.0)), float(rng.uniform(0.5, 2.0))
        H0.append(synth_hamiltonian(lay, 1000 + k, hw=hw, sigma2=sig))
        bases.append(B)
        emaxes.append(emax)
    HS = [api.Operator(B, 1, h) for B, h in zip(bases, H0)]
    G = [api.Operator(B, -1) for B in bases]
    t0 = time.perf_counter()
    res = api.magnus_decouple_batch(HS, G, s_max=50.0, ds=0.5, precision="ozaki")
    dt = time.perf_counter() - t0
    nc = sum(r["ncomm"] for r in res)
    out = {"instances": n, "emax": emaxes, "precision": "ozaki", "commutators": nc,
           "steps": sum(r["steps"] for r in res), "ok": sum(r["status"] == 0 for r in res),
           "interleaved": {"seconds": dt, "commutators_per_s": nc / dt,
                           "note": "includes step-graph capture of every instance"},
           "note": "instances whose BCH series does not converge stop with IMSRG_ERR_NOT_CONVERGED as the "
                   "reference STOPs"}
    # lockstep on fresh bases (each keeps its own workspace)
    lb = []
    for emax in emaxes:
        B = api.Basis.from_dict(ho_basis(emax))
        B.set_split_digits(SPLIT_DIGITS)
        lb.append(B)
    batch = api.Batch(lb)
    HS2 = [api.Operator(B, 1, h) for B, h in zip(lb, H0)]
    G2 = [api.Operator(B, -1) for B in lb]
    t0 = time.perf_counter()
    batch.magnus_decouple(HS2, G2, s_max=50.0, ds=0.5, precision="ozaki")
    first = time.perf_counter() - t0
    for op, h in zip(HS2, H0):
        op.upload(h)
    for B in lb:
        B.synchronize()
    t0 = time.perf_counter()
    res2 = batch.magnus_decouple(HS2, G2, s_max=50.0, ds=0.5, precision="ozaki")
    dt2 = time.perf_counter() - t0
    nc2 = sum(r["ncomm"] for r in res2)
    same = all(r["status"] == q["status"] and r["steps"] == q["steps"] and np.array_equal(r["trace"], q["trace"])
               for r, q in zip(res, res2))
    out["lockstep"] = {"seconds": dt2, "commutators_per_s": nc2 / dt2, "first_call_seconds": first,
                       "equal_to_interleaved_bit_for_bit": bool(same)}
    out["commutators_per_s"] = max(nc / dt, nc2 / dt2)
    batch.close()
    return out


_FP64_PEAK = []


def _fp64_peak_tflops():
    """cuBLAS DGEMM 8192^3 through torch.matmul, best of three (measured once
    per run): the FP64 pipe's rate on this GPU."""
    if _FP64_PEAK:
        return _FP64_PEAK[0]
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    _FP64_PEAK.append(2 * n ** 3 / (best / 1e3) / 1e12)
    return _FP64_PEAK[0]


def _traffic_from_profiles(kname):
    """DRAM bytes per launch of a kernel class from the committed ncu summary
    (profiles/dram_traffic.md, a two-column markdown table), or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "dram_traffic.md")):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 2 and cells[0] == kname and cells[1].isdigit():
                return int(cells[1])
    except OSError:
        pass
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "ozaki", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-flows", action="store_true", help="skip the flow and batched-flow extras")
    ap.add_argument("--batch", type=int, default=64, help="instances of the batched-flow extra")
    ap.add_argument("--split-digits", type=int, default=5, choices=[4, 5, 6],
                    help="digits per operand of the split engine (6: 21 BF16 products, 5: 15, 4: 10); "
                         "five meets |dE0| < 1e-6 MeV by five orders of magnitude")
    ap.add_argument("--split-schedule", type=int, default=None,
                    help="pin the split engine's CTA schedule model instead of autotuning it "
                         "(for profiler runs, whose serialised launches distort the tuner's timings)")
    ap.add_argument("--batched-only", type=int, default=0, metavar="N",
                    help="only the batched-commutator extra with N instances (for profiling the grouped launch)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    global SPLIT_DIGITS
    SPLIT_DIGITS = args.split_digits
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.batched_only:
        from imsrg_gpu import api
        print(json.dumps({"batched_commutators": batched_commutators(api, n=args.batched_only, reps=args.steps)}))
        return 0
    return run_gpu(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
