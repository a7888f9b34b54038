#!/usr/bin/env python
"""bench.py -- gam_4 integrals/s of the fused direct-SCF gam_4 Fock build.

One step = one GAM4_DSCF Fock build (gam4_DSCF_OMP.f:2-320): every one of
the ng4 = nebf^8 npbf^2 gam_4 elements is assembled from GAM_ee and GAM_2s
(24 ket permutations x 6 pair products, gam_4_OMP.f:712-1192) and contracted
with the electronic and nuclear densities into focke, fockp and E_gam4,
without storing gam_4.  FP64 throughout.

  value    device-resident inputs, K timed steps (CUDA events, barrier and
           synchronize on both sides, L2 flushed between steps).
  e2e      the public C-ABI call with HOST arrays (neoxc_gam4_dscf): the
           host->device copies of GAM_ee/GAM_2s/DE/DP and the device->host
           read of the Fock matrices and energy are inside the timed region.
  roofline the gam_4 kernel against the FP64 FMA rate measured on the same
           GPU by neoxc_probe_fp64 (the kernel is FP64-pipe bound; its DRAM
           traffic is the two input tables).
  cpu_baseline  the oracle's restatement of the reference loop on all host
           cores over a bounded contiguous sample of the same tuples.
  factored the factorised Fock build (same focke/fockp/E for the
           pair-symmetric tables the reference produces, O(nebf^4 npbf^2 +
           nebf^5) work) at this shape and at nebf=60/npbf=24, labelled
           separately; its "equivalent" rate is ng4 / time.

--impl reference times that CPU implementation alone (all host threads),
with the same metric and config.  With --gpus N (torchrun), every rank runs
one independent replica of the workload (weak scaling); value is the total
over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "neo-rxchf_gb300"))

NEBF, NPBF, NGTG, NPRIM = 12, 8, 3, 3
# FP64 operations of one element as the kernel evaluates it: 42 products
# accumulated by FMA (the factored form of the 24 x 6 products of
# symm_gam4), 4 operations combining the coefficient classes and 1 scaling,
# the density weight (2 multiplies) and its FMA; 2 FLOP per FMA.
FLOP_PER_ELEMENT = 2 * 42 + 7 + 1 + 2 + 2
METRIC = "gam_4 integrals/s"
UNIT = "integrals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nebf", type=int, default=NEBF)
    ap.add_argument("--npbf", type=int, default=NPBF)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true",
                    help="with --only gam2 / gam3 / gam3_batch / factored_tc: a small case "
                         "(for ncu captures)")
    ap.add_argument("--only", choices=["open_shell", "xcuhf_scf", "rx_scf", "config1", "gam3",
                                       "factored_tc", "gam3_batch", "gam2"],
                    default=None,
                    help="run one side section and print its JSON (no headline line)")
    return ap.parse_args()


def workload_config(ne, np_):
    return {
        "workload": ("XCHF RHF fused direct-SCF gam_4 Fock build (GAM4_DSCF): "
                     "nebf=%d contracted electronic functions (%d primitives each), "
                     "npbf=%d nuclear functions, NG=%d geminal terms" % (ne, NPRIM, np_, NGTG)),
        "nebf": ne, "npbf": np_, "ng4_per_step": ne ** 8 * np_ ** 2,
        "inputs": "GAM_ee (nebf^4) and GAM_2s (nebf^4 npbf^2) FP64 tables, DE, DP",
        "l2": "flushed between timed steps (256 MiB device write)",
        "parallelism": "replicas (one independent system per GPU)",
    }


def synthetic_inputs(ne, np_, seed=2024):
    """Seeded tables with the layouts and the pair-exchange symmetry of
    GAM_ee ((ab|cd) = (cd|ab)) and GAM_2s (gs(p;ab;cd) = gs(p;cd;ab), the
    GAM2_IC1 symmetrisation), and densities from two doubly occupied
    orbitals (the element kernel's work is data independent)."""
    from neoxc import basis
    rng = np.random.Generator(np.random.PCG64(seed))
    ee = rng.uniform(0.0, 1.0, (ne,) * 4)
    gee = np.ascontiguousarray((0.5 * (ee + ee.transpose(2, 3, 0, 1))).ravel())
    gs = rng.uniform(0.0, 1.0, (np_, np_) + (ne,) * 4)
    g2s = np.ascontiguousarray((0.5 * (gs + gs.transpose(0, 1, 4, 5, 2, 3))).ravel())
    DE = basis.random_density(ne, 2, seed + 1, 2.0)
    DP = basis.random_density(np_, 1, seed + 2, 1.0)
    return gee, g2s, DE, DP


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(backend):
    import torch.distributed as dist
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return dist, ws, rank, local


def replica_time(dist, ws, seconds, device=None):
    """Max over ranks of each rank's timed seconds (replica runs)."""
    if ws == 1:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(ne, np_, gee, g2s, DE, DP, target_s=12.0):
    """Oracle restatement of the reference loop on all host threads over a
    contiguous sample of the tuple space sized to about ``target_s``."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    L = O.lib()
    de = np.ascontiguousarray(DE.ravel(order="F"))
    dp = np.ascontiguousarray(DP.ravel(order="F"))
    fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    ng4 = ne ** 8 * np_ ** 2
    n = min(ng4, 4_000_000)
    t0 = time.perf_counter()
    L.orc_gam4_dscf_sample(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(de), O.ptr(dp), 0, n,
                           O.ptr(fe), O.ptr(fp), O.ptr(E))
    dt = time.perf_counter() - t0
    n2 = int(min(ng4, max(n, n * target_s / max(dt, 1e-6))))
    t0 = time.perf_counter()
    L.orc_gam4_dscf_sample(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(de), O.ptr(dp), 0, n2,
                           O.ptr(fe), O.ptr(fp), O.ptr(E))
    dt = time.perf_counter() - t0
    return {"value": n2 / dt, "unit": UNIT, "cores": int(L.orc_num_threads()),
            "kind": "port", "seconds": round(dt, 3),
            "sample": "first %d of %d gam_4 elements in loop_map order (%.2e %%), "
                      "oracle restatement of thread_gam4_DSCF with OpenMP" % (n2, ng4, 100.0 * n2 / ng4)}


def read_traffic(ne, np_):
    """Per-launch DRAM bytes of the gam_4 kernel from the committed ncu
    summary (profiles/gam4_dscf_traffic.txt), scaled to this workload by
    the table bytes it reads; None when no capture is recorded."""
    p = os.path.join(ROOT, "profiles", "gam4_dscf_traffic.txt")
    if not os.path.exists(p):
        return None
    kv = {}
    for ln in open(p):
        if "=" in ln and not ln.startswith("#"):
            k, v = ln.split("=", 1)
            kv[k.strip()] = v.strip()
    try:
        cap_ne, cap_np = int(kv["nebf"]), int(kv["npbf"])
        cap_bytes = float(kv["dram_bytes_per_launch"])
    except (KeyError, ValueError):
        return None
    scale = (ne ** 4 * np_ ** 2 + ne ** 4) / (cap_ne ** 4 * cap_np ** 2 + cap_ne ** 4)
    return cap_bytes * scale


def run_reference(args):
    dist, ws, rank, _ = dist_init("gloo")
    if rank != 0:
        return
    ne, np_ = args.nebf, args.npbf
    gee, g2s, DE, DP = synthetic_inputs(ne, np_)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    L = O.lib()
    de = np.ascontiguousarray(DE.ravel(order="F"))
    dp = np.ascontiguousarray(DP.ravel(order="F"))
    ng4 = ne ** 8 * np_ ** 2
    # size each step so that warm-up + timed steps take about two minutes
    fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    n = min(ng4, 4_000_000)
    t0 = time.perf_counter()
    L.orc_gam4_dscf_sample(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(de), O.ptr(dp), 0, n,
                           O.ptr(fe), O.ptr(fp), O.ptr(E))
    rate = n / (time.perf_counter() - t0)
    per_step = int(min(ng4, max(n, rate * 120.0 / (args.steps + args.warmup))))
    for _ in range(args.warmup):
        L.orc_gam4_dscf_sample(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(de), O.ptr(dp), 0,
                               per_step, O.ptr(fe), O.ptr(fp), O.ptr(E))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.orc_gam4_dscf_sample(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(de), O.ptr(dp), 0,
                               per_step, O.ptr(fe), O.ptr(fp), O.ptr(E))
    dt = time.perf_counter() - t0
    value = per_step * args.steps / dt
    cores = int(L.orc_num_threads())
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(ne, np_),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "first %d of %d gam_4 elements per step (the reference "
                                   "is Fortran and cannot be compiled here; the oracle "
                                   "restates its loop)" % (per_step, ng4)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


FACTORED_LARGE = (60, 24)   # nebf, npbf of the mixed-precision XCHF shape
FACTORED_LAUNCHES = 14      # kernels of one factorised build (k_gam4f.cu)


def time_factored(neoxc, torch, dev, stream, ne, np_, d_gee, d_g2s, d_DE, d_DP,
                  warmup=2, steps=5, fn=None):
    f64 = torch.float64
    fn = fn or neoxc.dev_gam4_fock_factored
    d_fe = torch.zeros(ne * ne, dtype=f64, device=dev)
    d_fp = torch.zeros(np_ * np_, dtype=f64, device=dev)
    d_E = torch.zeros(1, dtype=f64, device=dev)
    sp = stream.cuda_stream
    for _ in range(warmup):
        fn(sp, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_fe, d_fp, d_E)
    torch.cuda.synchronize(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn(sp, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_fe, d_fp, d_E)
    b.record(stream)
    torch.cuda.synchronize(dev)
    return a.elapsed_time(b) / steps, float(d_E.item())


def factored_section(neoxc, torch, dev, stream, ne, np_, gee, g2s, DE, DP,
                     d_gee, d_g2s, d_DE, d_DP, elem_ms, elem_E):
    """The factorised gam_4 Fock build (k_gam4f.cu): same focke/fockp/E as
    GAM4_DSCF for pair-symmetric tables at O(nebf^4 npbf^2 + nebf^5) work.
    Reported beside the element-wise number, not instead of it."""
    ms, E = time_factored(neoxc, torch, dev, stream, ne, np_, d_gee, d_g2s, d_DE, d_DP)
    t0 = time.perf_counter()
    n_e2e = 5
    for _ in range(n_e2e):
        neoxc.gam4_fock_factored(ne, np_, gee, g2s, DE, DP)
    e2e_ms = 1e3 * (time.perf_counter() - t0) / n_e2e
    out = {"api": "neoxc_dev_gam4_fock_factored (device), neoxc_gam4_fock_factored (host arrays)",
           "label": ("algorithm change, not the reference's loop: the same focke, fockp and "
                     "E_gam4 as GAM4_DSCF for pair-symmetric tables, from O(nebf^4 npbf^2 + "
                     "nebf^5) contractions instead of nebf^8 npbf^2 elements; the "
                     "'equivalent' rate divides the element count by this time"),
           "nebf": ne, "npbf": np_, "ms_per_build": ms, "e2e_ms_per_build": e2e_ms,
           "equivalent_gam4_integrals_per_s": ne ** 8 * np_ ** 2 / (ms * 1e-3),
           "speedup_vs_element_kernel": elem_ms / ms,
           "E_rel_diff_vs_element_kernel": abs(E - elem_E) / max(abs(elem_E), 1e-300),
           "kernel_launches_per_build": FACTORED_LAUNCHES}
    # the larger XCHF shape: tables generated on the device (60 GB of GAM_2s)
    nl, pl = FACTORED_LARGE
    n4 = nl ** 4
    need = 8 * (n4 * pl * pl + 9 * n4)
    free, _ = torch.cuda.mem_get_info(dev)
    if free < 1.2 * need:
        out["large"] = {"nebf": nl, "npbf": pl, "skipped": "needs %.1f GB free" % (need / 1e9)}
        return out
    f64 = torch.float64
    gen = torch.Generator(device=dev)
    gen.manual_seed(2025)
    lg2s = torch.empty(n4 * pl * pl, dtype=f64, device=dev)
    for p in range(pl * pl):
        t = torch.rand((nl,) * 4, generator=gen, dtype=f64, device=dev)
        lg2s[p * n4:(p + 1) * n4].view((nl,) * 4).copy_(0.5 * (t + t.permute(2, 3, 0, 1)))
        del t
    t = torch.rand((nl,) * 4, generator=gen, dtype=f64, device=dev)
    lgee = (0.5 * (t + t.permute(2, 3, 0, 1))).contiguous().view(-1)
    del t
    from neoxc import basis
    lDE = torch.tensor(np.ascontiguousarray(basis.random_density(nl, 5, 11, 2.0).ravel(order="F")),
                       dtype=f64, device=dev)
    lDP = torch.tensor(np.ascontiguousarray(basis.random_density(pl, 1, 12, 1.0).ravel(order="F")),
                       dtype=f64, device=dev)
    lms, lE = time_factored(neoxc, torch, dev, stream, nl, pl, lgee, lg2s, lDE, lDP)
    tms, tE = time_factored(neoxc, torch, dev, stream, nl, pl, lgee, lg2s, lDE, lDP,
                            fn=neoxc.dev_gam4_fock_factored_tc)
    table_bytes = 8 * n4 * pl * pl
    # GAM_2s is read twice (G = DP.GAM_2s, fockp = GAM_2s.W): the HBM floor
    hbm_bytes = 2 * table_bytes
    peak = read_hbm_peak()
    out["large"] = {"nebf": nl, "npbf": pl, "ms_per_build": lms,
                    "equivalent_gam4_integrals_per_s": nl ** 8 * pl * pl / (lms * 1e-3),
                    "GAM_2s_GB": table_bytes / 1e9,
                    "roofline": {"bound": "hbm", "algorithmic_bytes": hbm_bytes,
                                 "achieved": hbm_bytes / (lms * 1e-3) / 1e9, "unit": "GB/s",
                                 "peak": peak,
                                 "frac": (hbm_bytes / (lms * 1e-3) / 1e9) / peak if peak else None,
                                 "note": "whole build timed; bytes = the two passes over GAM_2s"},
                    "E": lE,
                    "tensor_core": {
                        "api": "neoxc_dev_gam4_fock_factored_tc (tcgen05 kind::tf32, 3xTF32 "
                               "products, FP32 accumulation per 64-wide K tile, FP64 across "
                               "tiles; GAM_2s passes, traces, gradients FP64)",
                        "ms_per_build": tms,
                        "speedup_vs_fp64_build": lms / tms,
                        "E": tE, "E_rel_err_vs_fp64": abs(tE - lE) / max(abs(lE), 1e-300),
                        "roofline": {"bound": "hbm", "algorithmic_bytes": hbm_bytes,
                                     "achieved": hbm_bytes / (tms * 1e-3) / 1e9, "unit": "GB/s",
                                     "peak": peak,
                                     "frac": (hbm_bytes / (tms * 1e-3) / 1e9) / peak
                                     if peak else None}}}
    del lg2s, lgee
    torch.cuda.empty_cache()
    return out


def factored_tc_only(neoxc, torch, dev, ne, np_):
    """FP64 and tensor-core factorised gam_4 builds on device-generated
    pair-symmetric tables (ne^4 np^2 GAM_2s), timed with CUDA events."""
    f64 = torch.float64
    stream = torch.cuda.current_stream(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(2025)
    n4 = ne ** 4
    g2s = torch.empty(n4 * np_ * np_, dtype=f64, device=dev)
    for p in range(np_ * np_):
        t = torch.rand((ne,) * 4, generator=gen, dtype=f64, device=dev)
        g2s[p * n4:(p + 1) * n4].view((ne,) * 4).copy_(0.5 * (t + t.permute(2, 3, 0, 1)))
    t = torch.rand((ne,) * 4, generator=gen, dtype=f64, device=dev)
    gee = (0.5 * (t + t.permute(2, 3, 0, 1))).contiguous().view(-1)
    from neoxc import basis
    DE = torch.tensor(np.ascontiguousarray(basis.random_density(ne, 5, 11, 2.0).ravel(order="F")),
                      dtype=f64, device=dev)
    DP = torch.tensor(np.ascontiguousarray(basis.random_density(np_, 1, 12, 1.0).ravel(order="F")),
                      dtype=f64, device=dev)
    ms, E = time_factored(neoxc, torch, dev, stream, ne, np_, gee, g2s, DE, DP)
    tms, tE = time_factored(neoxc, torch, dev, stream, ne, np_, gee, g2s, DE, DP,
                            fn=neoxc.dev_gam4_fock_factored_tc)
    hbm = 2 * 8 * n4 * np_ * np_
    peak = read_hbm_peak()
    return {"nebf": ne, "npbf": np_, "fp64_ms": ms, "tc_ms": tms, "E_fp64": E, "E_tc": tE,
            "E_rel_err": abs(tE - E) / max(abs(E), 1e-300),
            "hbm_floor_ms": hbm / (peak * 1e9) * 1e3,
            "tc_frac_of_hbm_floor": (hbm / (peak * 1e9) * 1e3) / tms}


def open_shell_section(neoxc, torch, dev, stream):
    """XCUHF in-core contractions (k_spin.cu): one neoxc_dev_xcuhf_omg call
    gives FAE_OMGk, FAE_OMGk for beta and UFP_OMGk (three reference routines)
    from one pass over the stored tensor.  Tensors larger than L2, seeded on
    the device; NAE = NBE = 2.  The tensor is read once (algorithmic bytes,
    reported against HBM), but the bound is the FP64 pipe: ncu shows 90 %
    FP64-pipe activity and 3.5 % DRAM for rank 3
    (profiles/spin_kernel_rank3_open_shell.md)."""
    f64 = torch.float64
    peak = read_hbm_peak()
    out = {"api": "neoxc_dev_xcuhf_omg (device)", "peak_gbs": peak}
    sp = stream.cuda_stream
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)
    for k, ne, np_ in ((2, 40, 4), (3, 12, 4), (4, 10, 2)):
        n = ne ** (2 * k) * np_ ** 2
        ntens = 2 if k == 2 else 1
        free, _ = torch.cuda.mem_get_info(dev)
        if free < 1.5 * 8 * n * ntens:
            out["omg%d" % k] = {"skipped": "needs %.1f GB free" % (8e-9 * n * ntens)}
            continue
        G = torch.rand(n, generator=gen, dtype=f64, device=dev)
        Gs = torch.rand(n, generator=gen, dtype=f64, device=dev) if k == 2 else None
        A = torch.rand((ne, ne), generator=gen, dtype=f64, device=dev)
        DA = (A @ A.T).contiguous().view(-1) / ne
        B = torch.rand((ne, ne), generator=gen, dtype=f64, device=dev)
        DB = (B @ B.T).contiguous().view(-1) / ne
        DP = torch.eye(np_, dtype=f64, device=dev).view(-1)
        FA = torch.zeros(ne * ne, dtype=f64, device=dev)
        FB, FP = torch.zeros_like(FA), torch.zeros(np_ * np_, dtype=f64, device=dev)
        S = [torch.zeros_like(FA), torch.zeros_like(FA), torch.zeros_like(FP)] if k == 2 \
            else [None, None, None]
        E = torch.zeros(6, dtype=f64, device=dev)

        def call():
            neoxc.dev_xcuhf_omg(sp, k, ne, np_, 2, 2, G, Gs, DA, DB, DP, FA, FB, FP,
                                S[0], S[1], S[2], E)
        for _ in range(2):
            call()
        torch.cuda.synchronize(dev)
        steps = 5
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            call()
        b.record(stream)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / steps
        nbytes = 8 * n * ntens
        gbs = nbytes / (ms * 1e-3) / 1e9
        out["omg%d" % k] = {"nebf": ne, "npbf": np_, "tensor_GB": nbytes / 1e9,
                            "ms_per_call": ms, "elements_per_s": n / (ms * 1e-3),
                            "hbm": {"achieved": gbs, "unit": "GB/s", "peak": peak,
                                    "frac": gbs / peak if peak else None,
                                    "algorithmic_bytes": nbytes},
                            "bound": "fp64",
                            "launches_per_call": 5}
        del G, Gs
        torch.cuda.empty_cache()
    return out


def xcuhf_scf_section(neoxc):
    """XCUHF (open-shell) SCF on the reference's examples/xcuhf system
    (fixture tests/golden/xcuhf_example.json): core-Hamiltonian guesses for
    both spins and the proton, every integral including the raw OMG4_ICR
    tensor built on the GPU, UHF_FOCK / UROOTHAN with DIIS there.  The
    converged energy is compared with XCUHF.log's."""
    import re
    from neoxc import basis
    with open(os.path.join(ROOT, "tests", "golden", "xcuhf_example.json")) as f:
        g = json.load(f)
    s = basis.parse_inp(g["inp"], name="examples/xcuhf")
    m = re.search(r"&XCUHF\s*nae=(\d+),\s*nbe=(\d+)", g["inp"], re.I)
    nae, nbe = int(m.group(1)), int(m.group(2))
    E_log = g["final"]["E_TOTAL"]
    out = {"workload": "examples/xcuhf XCUHF (nebf=%d, npebf=%d, npbf=%d, NG=%d, NAE=%d, "
                       "NBE=%d), core-Hamiltonian guesses" % (s.nebf, s.npebf, s.npbf, s.ngtg,
                                                              nae, nbe),
           "api": "neoxc_xcuhf_scf (host arrays; integrals and SCF on the GPU)"}
    neoxc.xcuhf_scf(s, nae, nbe, maxit=2)   # warm-up
    for name, mixed in (("diis", False), ("diis_mixed", True)):
        t0 = time.perf_counter()
        r = neoxc.xcuhf_scf(s, nae, nbe, diis=True, mixed=mixed)
        dt = time.perf_counter() - t0
        t1 = time.perf_counter()
        neoxc.xcuhf_scf(s, nae, nbe, maxit=1, mixed=mixed)
        dt1 = time.perf_counter() - t1
        out[name] = {"solves_per_s": 1.0 / dt, "ms_per_solve": 1e3 * dt,
                     "iterations": r["niter"], "converged": r["converged"],
                     "ms_integrals_plus_first_iteration": 1e3 * dt1,
                     "ms_per_iteration": 1e3 * (dt - dt1) / max(1, r["niter"] - 1),
                     "E_total": r["final"]["E_total"],
                     "E_err_vs_log": r["final"]["E_total"] - E_log}
    return out


RX_BENCH = (("rxchf_ne", dict(nae=2)), ("rxcuhf_ne", dict(nalp=1, nbet=2)),
            ("rxcuhf_ae", dict(nalp=1, nbet=2)))


def rx_scf_section(neoxc, with_cpu: bool):
    """One-special-electron RXCHF SCF (neoxc_rx_scf) on the reference's
    examples/rxchf/one_special_electron and examples/rxcuhf/rxchf-{ne,ae}
    (fixture tests/golden/rx_examples.json): every integral on the GPU,
    UROOTHAN + OCBSE2 iterations there.  The converged energies are compared
    with the logs'.  The CPU leg times the oracle's restatement of the
    RXCHF-ne solve (C tables with OpenMP + the numpy SCF) on the host cores."""
    from neoxc import basis
    with open(os.path.join(ROOT, "tests", "golden", "rx_examples.json")) as f:
        g = json.load(f)
    out = {"api": "neoxc_rx_scf (host arrays; integrals and SCF on the GPU)"}
    for name, kw in RX_BENCH:
        s = basis.parse_inp(g[name]["inp"], name=name)
        neoxc.rx_scf(s, name, **kw)   # warm-up
        t0 = time.perf_counter()
        r = neoxc.rx_scf(s, name, **kw)
        dt = time.perf_counter() - t0
        out[name] = {"workload": "%s (nebf=%d, npebf=%d, npbf=%d, NG=%d)" % (
                         g[name]["source"], s.nebf, s.npebf, s.npbf, s.ngtg),
                     "solves_per_s": 1.0 / dt, "ms_per_solve": 1e3 * dt,
                     "iterations": r["niter"], "converged": r["converged"],
                     "micro_iterations": int(r["history"][:, 1].sum()),
                     "E_total": r["final"]["E_total"],
                     "E_err_vs_log": r["final"]["E_total"] - g[name]["final_energy"]}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        import rxne
        O.build()
        s = basis.parse_inp(g["rxchf_ne"]["inp"], name="rxchf_ne")
        t0 = time.perf_counter()
        ints = rxne.RxIntegrals(s)
        _, fin, hist, ok = rxne.rx_scf(ints, nae=2)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"kind": "port", "cores": os.cpu_count(),
                               "sample": "one full RXCHF-ne solve of "
                                         "examples/rxchf/one_special_electron",
                               "solves_per_s": 1.0 / dt, "seconds": dt,
                               "E_err_vs_log": fin["E_total"] - g["rxchf_ne"]["final_energy"]}
        out["gpu_vs_cpu_rxchf_ne"] = out["rxchf_ne"]["solves_per_s"] / (1.0 / dt)
    return out


def scf_section(neoxc, with_cpu: bool):
    """XCHF RHF SCF solves/s on the reference's examples/xchf system (inputs
    from the committed fixture tests/golden/xchf_example.json: exam_xchf.inp
    and guessCE.inp), through neoxc_xchf_scf with host arrays: every integral
    (overlaps, core, GAM_ep, GAM_1, GAM_ee, gam_2, gam_3) is built on the GPU
    and the Roothaan loop (plain, as xcscf.f, and with DIIS) runs there.  The
    converged energy is compared with XCHF.log's."""
    from neoxc import basis
    with open(os.path.join(ROOT, "tests", "golden", "xchf_example.json")) as f:
        g = json.load(f)
    s = basis.parse_inp(g["inp"], name="examples/xchf")
    DE = basis.density(basis.read_mo_file(g["guessCE"], s.nebf), s.nelec // 2, 2.0)
    E_log = g["final"]["E_TOTAL"]
    out = {"workload": "examples/xchf XCHF RHF (nebf=%d, npebf=%d, npbf=%d, NG=%d, nelec=%d), "
                       "guessCE start, core-Hamiltonian proton guess" % (
                           s.nebf, s.npebf, s.npbf, s.ngtg, s.nelec),
           "api": "neoxc_xchf_scf (host arrays; integrals and SCF on the GPU)"}
    neoxc.xchf_scf(s, DE, maxit=3)   # warm-up (module load, allocator)
    E_fp64 = None
    for name, diis, mixed in (("roothan", False, False), ("diis", True, False),
                              ("diis_mixed_gam3", True, "gam3"), ("diis_mixed", True, True)):
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            r = neoxc.xchf_scf(s, DE, diis=diis, mixed=mixed)
        dt = (time.perf_counter() - t0) / reps
        t1 = time.perf_counter()
        neoxc.xchf_scf(s, DE, maxit=1, diis=diis, mixed=mixed)
        dt1 = time.perf_counter() - t1
        out[name] = {"solves_per_s": 1.0 / dt, "ms_per_solve": 1e3 * dt,
                     "iterations": r["niter"], "converged": r["converged"],
                     "ms_integrals_plus_first_iteration": 1e3 * dt1,
                     "ms_per_iteration": 1e3 * (dt - dt1) / max(1, r["niter"] - 1),
                     "E_total": r["final"]["E_total"],
                     "E_err_vs_log": r["final"]["E_total"] - E_log}
        if mixed:
            out[name]["E_err_vs_fp64_Eh"] = r["final"]["E_total"] - E_fp64
            out[name]["precision"] = ("%s MD tables FP32 (Boys function, seeds, sums over "
                                      "primitives and geminal terms FP64%s); one-body, "
                                      "GAM_1, GAM_ee, contractions, Fock assembly and "
                                      "diagonalisation FP64"
                                      % (("gam_3", "") if mixed == "gam3" else
                                         ("gam_2, gam_3", "; gam_2 items above the "
                                          "recompute threshold in FP64")))
        else:
            E_fp64 = r["final"]["E_total"]
    out["config1"] = config1_section(neoxc)
    out["xcuhf"] = xcuhf_scf_section(neoxc)
    out["rx"] = rx_scf_section(neoxc, with_cpu)
    out["batch"] = scf_batch_section(neoxc, s, DE)
    out["gam3_batch"] = gam3_batch_section(neoxc)
    out["serving"] = scf_serving_section(neoxc, s, DE)
    if with_cpu:
        out["cpu_baseline"] = scf_cpu_baseline(s, DE, out["roothan"]["iterations"])
    return out


CONFIG1 = dict(seed=2024, nat=3, nebf=12, nprim=3, npbf=8, ngtg=3, lmax_e=1, lmax_p=2)


def config1_section(neoxc):
    """The seeded XCHF RHF system of the first configuration: 3 nuclei in
    [-1.5,1.5]^3 bohr, 4 electrons, the proton on nucleus 0, 12 contracted
    s/p electronic functions of 3 primitives (exponents log-uniform in
    [0.1,20]), 8 even-tempered s/p/d nuclear primitives (4-32), NG=3.  One
    solve = every integral built on the GPU (gam_2 and the 1.9e8-element
    gam_3 tensor included) from core-Hamiltonian guesses and DIIS SCF to
    the reference's convergence rule, through neoxc_xchf_scf with host
    arrays.  Mixed (FP32 McMurchie-Davidson tables for gam_2 and gam_3 with
    FP64 Boys function, seeds and sums, the large gam_2 items re-evaluated
    in FP64; Fock assembly and diagonalisation FP64), then FP64; the mixed
    energy is reported against the FP64 one."""
    from neoxc import basis
    s = basis.synthetic(**CONFIG1)
    out = {"workload": "XCHF RHF, seeded synthetic system (seed %d): nebf=%d (s/p, 3 primitives), "
                       "npbf=%d (s/p/d), NG=%d, nelec=%d; ng3=%.3g" % (
                           CONFIG1["seed"], s.nebf, s.npbf, s.ngtg, s.nelec, s.ng3),
           "api": "neoxc_xchf_scf (host arrays; core-Hamiltonian guesses, DIIS)"}
    E = {}
    for name, mixed in (("mixed", True), ("fp64", False)):
        t0 = time.perf_counter()
        r = neoxc.xchf_scf(s, None, diis=True, mixed=mixed)
        dt = time.perf_counter() - t0
        E[name] = r["final"]["E_total"]
        out[name] = {"solves_per_s": 1.0 / dt, "ms_per_solve": 1e3 * dt,
                     "iterations": r["niter"], "converged": r["converged"],
                     "E_total": r["final"]["E_total"],
                     "E_init": r["initial"]["E_total"]}
    out["mixed"]["E_err_vs_fp64_Eh"] = E["mixed"] - E["fp64"]
    out["mixed"]["E_init_err_vs_fp64_Eh"] = out["mixed"]["E_init"] - out["fp64"]["E_init"]
    out["mixed"]["gam2_recompute_threshold"] = neoxc.get_mixed_threshold()
    out["mixed_over_fp64_solves_per_s"] = out["mixed"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    return out


def gam3_section(neoxc, kw=None):
    """The gam_3 builder (GAM3_IC1: the dense contracted gam_3 tensor, packed
    index_GAM_3PK order, six-permutation symmetrised) on the seeded system of
    the first configuration, FP64 and mixed (FP32 tables, FP64 Boys
    function, seeds and sums).  Device time of the build from CUDA events
    (the copy of the 1.5 GB tensor to the host excluded).  Units: contracted
    gam_3 integrals/s (ng3 / t) and composite-bra x pair-ket Coulomb
    evaluations/s (k_gam3.cu: 2 passes x pair-canonical (Pp, P1, P2) x
    primitive bras x geminal pairs x primitive kets)."""
    from neoxc import basis
    kw = kw or CONFIG1
    s = basis.synthetic(**kw)
    nPe = s.nebf * (s.nebf + 1) // 2
    nPp = s.npbf * (s.npbf + 1) // 2
    k = np.array(s.KPEEND) - np.array(s.KPESTR) + 1
    ket_pairs = sum(int(k[i] * k[j]) for i in range(s.nebf) for j in range(i + 1))
    # per pass: CTAs (Pp, Pa, Pb) x bras (prim pairs of Pa x of Pb x NG^2) x kets
    pp_of = [int(k[i] * k[j]) for i in range(s.nebf) for j in range(i + 1)]
    evals = 2 * nPp * sum(pp_of) ** 2 * s.ngtg ** 2 * ket_pairs
    out = {"workload": "GAM3_IC1 on the seeded nebf=%d (s/p, %d primitives), npbf=%d (s/p/d), "
                       "NG=%d system: ng3=%d" % (s.nebf, s.npebf // s.nebf, s.npbf, s.ngtg, s.ng3),
           "api": "neoxc_gam3_ic1_opts (device time from CUDA events)",
           "canonical_tuples": nPp * nPe ** 3, "primitive_pair_kets": ket_pairs,
           "coulomb_evaluations": evals}
    for name, mixed in (("mixed", True), ("fp64", False)):
        x, sec = neoxc.gam3_ic1(s, mixed=mixed, timing=True)
        out[name] = {"seconds": sec, "gam3_integrals_per_s": s.ng3 / sec,
                     "coulomb_evaluations_per_s": evals / sec, "absmax": float(np.abs(x).max())}
        out[name + "_tensor"] = x
    diff = float(np.abs(out["mixed_tensor"] - out["fp64_tensor"]).max())
    out["mixed"]["max_abs_diff_vs_fp64"] = diff
    out["mixed"]["max_rel_diff_vs_fp64"] = diff / max(out["fp64"]["absmax"], 1e-300)
    del out["mixed_tensor"], out["fp64_tensor"]
    return out


def gam2_section(neoxc, small=False):
    """The gam_2 build (GM2ICR / GM2sICR, k_md.cu) in FP64 and in the mixed
    precision (FP32 tables, FP64 Boys function, seeds and sums, items above
    the recompute threshold re-evaluated in FP64), timed as a one-iteration
    XCHF SCF of a two-electron system (no gam_3: the gam_2 build dominates;
    the one-body, GAM_1 and GAM_ee builds and one Fock build are included).
    System: the first configuration's seeded basis with 2 electrons, or with
    small=True the seeded nebf=8 (s/p, 3 primitives), npbf=4 (s/p/d) one."""
    from neoxc import basis
    if small:
        kw = dict(seed=6, nat=3, nebf=8, nprim=3, npbf=4, ngtg=3, lmax_e=1, lmax_p=2, nelec=2)
    else:
        kw = dict(CONFIG1, nelec=2)
    s = basis.synthetic(**kw)
    out = {"workload": "one-iteration XCHF SCF, seeded nebf=%d (s/p), npbf=%d (s/p/d), NG=%d, "
                       "nelec=2: ng2=%d" % (s.nebf, s.npbf, s.ngtg, s.nebf ** 4 * s.npbf ** 2),
           "api": "neoxc_xchf_scf (maxit 1; host arrays)",
           "gam2_recompute_threshold": neoxc.get_mixed_threshold()}
    neoxc.xchf_scf(s, None, maxit=1, mixed="gam2")   # warm-up
    E = {}
    for name, mixed in (("mixed", "gam2"), ("fp64", False)):
        t0 = time.perf_counter()
        r = neoxc.xchf_scf(s, None, maxit=1, mixed=mixed)
        dt = time.perf_counter() - t0
        E[name] = r["initial"]["E_total"]
        out[name] = {"seconds": dt, "E_init": E[name]}
    out["mixed"]["E_err_vs_fp64_Eh"] = E["mixed"] - E["fp64"]
    out["fp64_over_mixed_time"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    return out


def gam3_batch_section(neoxc, nsys=48):
    """Many uneven systems' gam_3 in persistent launches
    (neoxc_gam3_ic1_batch): seeded molecules of 3-6 nuclei with the proton
    basis on nucleus 0, nebf 4-7 (s/p, 2-3 primitives), npbf 2-4 (s/p/d),
    NG 3-4, mixed precision.  Device time of the batched build against the
    sum of the per-system builds' device times (neoxc_gam3_ic1_opts), the
    autotuner's choices, and the largest deviation of a batched tensor from
    its separate build."""
    from neoxc import basis
    rng = np.random.Generator(np.random.PCG64(44))
    systems = []
    for k in range(nsys):
        systems.append(basis.synthetic(seed=1000 + k, nat=int(rng.integers(3, 7)),
                                       nebf=int(rng.integers(4, 8)), nprim=(2, 3),
                                       npbf=int(rng.integers(2, 5)), ngtg=int(rng.integers(3, 5)),
                                       lmax_e=1, lmax_p=2, name="batch%d" % k))
    neoxc.gam3_ic1_batch(systems[:2], mixed=True)            # warm-up (tunes the class)
    outs, t_batch = neoxc.gam3_ic1_batch(systems, mixed=True)
    t_sep, dev = 0.0, 0.0
    for s, x in zip(systems, outs):
        y, t = neoxc.gam3_ic1(s, mixed=True, timing=True)
        t_sep += t
        dev = max(dev, float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)))
    return {"workload": "%d seeded systems, nebf 4-7 (s/p), npbf 2-4 (s/p/d), NG 3-4, mixed" % nsys,
            "api": "neoxc_gam3_ic1_batch (one persistent launch per angular class)",
            "total_ng3": int(sum(s.ng3 for s in systems)),
            "batched_s": t_batch, "separate_builds_s": t_sep,
            "speedup": t_sep / t_batch if t_batch > 0 else None,
            "systems_per_s": nsys / t_batch if t_batch > 0 else None,
            "max_rel_dev_vs_separate": dev,
            "autotuner": neoxc.gam3_batch_tuning()}


# Precision of the mixed arms of the examples/xchf scans: gam_3 in FP32
# tables (0.15 microhartree from FP64 on this system), gam_2 in FP64.  Most
# gam_2 items of this basis (tight s primitives) lie above the dynamic-
# precision threshold, where the mixed gam_2 build costs more than the FP64
# one (52.0 vs 43.7 ms per DIIS solve).
SCAN_MIXED = "gam3"


def scf_serving_section(neoxc, s, DE):
    """Poisson arrivals of proton-scan requests (seeded) into the
    continuous-batching server (8 worker streams, DIIS): p50/p99 time from
    submission to converged energy, and completed solves/s, per rate."""
    from neoxc import basis
    out = {"workload": "examples/xchf proton-scan requests, Poisson arrivals, 8 workers, DIIS",
           "mixed_mode": SCAN_MIXED}
    for mixed, rates, n in ((SCAN_MIXED, (5.0, 10.0, 20.0, 40.0), 40), (False, (2.0,), 16)):
        for lam in rates:
            rng = np.random.Generator(np.random.PCG64(int(lam * 100) + (1 if mixed else 0)))
            gaps = rng.exponential(1.0 / lam, n)
            systems = basis.proton_scan(s, n, 0.5, seed=int(lam))
            srv = neoxc.XchfServer(nworkers=8, diis=True, mixed=mixed)
            try:
                t0 = time.perf_counter()
                tickets = []
                for k in range(n):
                    target = t0 + gaps[:k + 1].sum()
                    dt = target - time.perf_counter()
                    if dt > 0:
                        time.sleep(dt)
                    tickets.append(srv.submit(systems[k], DE))
                res = [srv.wait(t) for t in tickets]
            finally:
                srv.stop()
            lat = np.array([r["t_end"] - r["t_submit"] for r in res])
            span = max(r["t_end"] for r in res) - min(r["t_submit"] for r in res)
            out["%s_rate%g" % ("mixed" if mixed else "fp64", lam)] = {
                "requests": n, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                "solves_per_s": n / span, "converged": sum(r["converged"] for r in res)}
    return out


def scf_batch_section(neoxc, s, DE, njobs=48):
    """A proton-position scan (proton basis centre displaced uniformly within
    +-0.5 bohr, seeded) of njobs independent solves through
    neoxc_xchf_scf_batch: solves/s with one worker stream and with eight."""
    from neoxc import basis
    systems = basis.proton_scan(s, njobs, 0.5, seed=11)
    DEs = [DE] * njobs
    out = {"workload": "%d-point proton-position scan of examples/xchf, DIIS" % njobs,
           "mixed_mode": SCAN_MIXED}
    neoxc.xchf_scf_batch(systems[:2], DEs[:2], nworkers=2, diis=True, mixed=SCAN_MIXED)
    for mixed in (False, SCAN_MIXED):
        for nw in (1, 8):
            t0 = time.perf_counter()
            res = neoxc.xchf_scf_batch(systems, DEs, nworkers=nw, diis=True, mixed=mixed)
            dt = time.perf_counter() - t0
            key = "%s_workers%d" % ("mixed" if mixed else "fp64", nw)
            out[key] = {"solves_per_s": njobs / dt, "seconds": dt,
                        "converged": sum(r["converged"] for r in res)}
    return out


def scf_cpu_baseline(s, DE, niter):
    """The oracle's restatement (C integrals with OpenMP + numpy xcscf) of the
    same solve, timed in full: every integral and every Roothaan iteration
    to convergence."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import xchf_scf as X
    O.build()
    t0 = time.perf_counter()
    ints = X.XchfIntegrals(s)
    t_int = time.perf_counter() - t0
    t1 = time.perf_counter()
    hist, _, _, _, ok = X.xchf_scf(ints, DE)
    t_scf = time.perf_counter() - t1
    total = t_int + t_scf
    return {"solves_per_s": 1.0 / total, "unit": "SCF solves/s", "kind": "port",
            "cores": int(O.lib().orc_num_threads()), "converged": bool(ok),
            "sample": "one full solve: integrals %.1f s + %d Roothaan iterations %.1f s "
                      "(the GPU run took %d)" % (t_int, len(hist) - 1, t_scf, niter)}


def read_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import neoxc
    dist, ws, rank, local = dist_init("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    neoxc.lib()
    if not neoxc.device_ok():
        raise SystemExit("no usable GB300: " + neoxc.lib().neoxc_last_error().decode())
    if args.only == "open_shell":
        print(json.dumps(open_shell_section(neoxc, torch, dev, torch.cuda.current_stream(dev))))
        return
    if args.only == "xcuhf_scf":
        print(json.dumps(xcuhf_scf_section(neoxc)))
        return
    if args.only == "rx_scf":
        print(json.dumps(rx_scf_section(neoxc, not args.no_cpu_baseline)))
        return
    if args.only == "config1":
        print(json.dumps(config1_section(neoxc)))
        return
    if args.only == "gam3":
        kw = dict(CONFIG1, nebf=6, npbf=4) if args.small else None
        print(json.dumps(gam3_section(neoxc, kw)))
        return
    if args.only == "gam2":
        print(json.dumps(gam2_section(neoxc, args.small)))
        return
    if args.only == "gam3_batch":
        print(json.dumps(gam3_batch_section(neoxc, 8 if args.small else 48)))
        return
    if args.only == "factored_tc":
        print(json.dumps(factored_tc_only(neoxc, torch, dev, 24 if args.small else 60,
                                          8 if args.small else 24)))
        return
    ne, np_ = args.nebf, args.npbf
    ng4 = ne ** 8 * np_ ** 2
    gee, g2s, DE, DP = synthetic_inputs(ne, np_)
    f64 = torch.float64
    d_gee = torch.tensor(gee, dtype=f64, device=dev)
    d_g2s = torch.tensor(g2s, dtype=f64, device=dev)
    d_DE = torch.tensor(np.ascontiguousarray(DE.ravel(order="F")), dtype=f64, device=dev)
    d_DP = torch.tensor(np.ascontiguousarray(DP.ravel(order="F")), dtype=f64, device=dev)
    d_fe = torch.zeros(ne * ne, dtype=f64, device=dev)
    d_fp = torch.zeros(np_ * np_, dtype=f64, device=dev)
    d_E = torch.zeros(1, dtype=f64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step():
        neoxc.dev_gam4_dscf(sp, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_fe, d_fp, d_E)

    peak = neoxc.probe_fp64_tflops()
    for _ in range(max(args.warmup, 0)):
        flush.zero_()
        step()
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    clk = clocks.stop()
    total_s = t_start.elapsed_time(t_end) / 1e3
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = replica_time(dist, ws, total_s, dev)
    value = ws * ng4 * args.steps / total_s
    # ---- e2e through the host-array C-ABI call
    e2e_steps = max(1, min(args.steps, 2))
    neoxc.gam4_dscf(ne, np_, gee, g2s, DE, DP)       # warm the host path
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        fe, fp, E = neoxc.gam4_dscf(ne, np_, gee, g2s, DE, DP)
    e2e_s = replica_time(dist, ws, time.perf_counter() - t0, dev)
    e2e = {"value": ws * ng4 * e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": 8 * (ne ** 4 + ne ** 4 * np_ ** 2 + ne * ne + np_ * np_),
           "d2h_bytes_per_step": 8 * (ne * ne + np_ * np_ + 1),
           "api": "neoxc_gam4_dscf (host arrays)"}
    if rank != 0:
        return
    mean_ms = float(np.mean(kern_ms))
    achieved = FLOP_PER_ELEMENT * ng4 / (mean_ms * 1e-3) / 1e12
    traffic = read_traffic(ne, np_)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded tables with the GAM_ee / GAM_2s layouts)",
        "config": workload_config(ne, np_),
        "e2e": e2e,
        "gpu_launches": 3 * args.steps,
        "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "peak_source": "neoxc_probe_fp64 on this GPU (measured DFMA rate, a "
                                    "builder-measured lower bound of the FP64 peak: the "
                                    "kernel can exceed it); "
                                    "MEASURED_PEAKS.json has no FP64 figure",
                     "flop_per_element": FLOP_PER_ELEMENT,
                     "kernel_ms_mean": mean_ms},
    }
    line["factored"] = factored_section(neoxc, torch, dev, stream, ne, np_, gee, g2s, DE, DP,
                                        d_gee, d_g2s, d_DE, d_DP, mean_ms, float(d_E.item()))
    line["open_shell"] = open_shell_section(neoxc, torch, dev, stream)
    line["scf"] = scf_section(neoxc, not args.no_cpu_baseline and ws == 1)
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"] = cpu_baseline(ne, np_, gee, g2s, DE, DP)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
