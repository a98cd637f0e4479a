#!/usr/bin/env python
"""Powder-averaged muon polarisation throughput on one GB300.

Workload (the 24-dimensional powder configuration): spins mu, e, 1H, 14N
(Hilbert dimension 24) with seeded random anisotropic hyperfine, dipolar and
quadrupolar couplings, 10,000 ZCW-style orientations, 4096 times on
0-20 us, B = 0.01 T, T = inf, muon polarised along z -- the muon-first
fast path.  Synthetic inputs stand in for a real material; see
muspinsim_gb300/workloads.py.

Metric: P(t) samples/s, one sample = one (orientation, time) value before the
orientation average.  ``value`` is the mixed-precision pipeline (FP32
Householder + QL eigensolve + double-word refinement + FP32 phase sum) with
inputs resident in HBM; the
all-FP64 pipeline is timed beside it (``fp64``) and the max |dP| between the
two is reported.  ``e2e`` runs the public ``powder_average`` call on host
inputs (host->device copies and the device->host result inside the timed
region).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "powder-avg P(t) samples/s, mixed-prec vs FP64 GPU at max|ΔP|≤1e-6, 1×GB300"
WORKLOAD = "mu_e_1H_14N_dim24_powder_10k_orient_4096_t"
L2_BYTES = 129 * 1024 * 1024
# FP32 FMA lanes per SM on GB300 (152 SMs); the FP32 SIMT roofline is
# 152 * 128 * 2 flop * SM clock.  MEASURED_PEAKS.json carries HBM and bf16
# tensor figures only.
SMS, FP32_FMA_PER_SM = 152, 128
# DRAM bytes (read + write) per snapshot of each stage's kernel, from ncu
# --set full captures of the 2,000-orientation x 4,096-time case
# (dram__bytes_read.sum + dram__bytes_write.sum per launch / 2,000): the
# eigensolve reads the system matrices (L2-resident; its reflectors and
# eigenvectors go through the L2-resident scratch), the refinement its
# eigenvectors (4.6 KB a snapshot), the phase sum the pair records (6.6 KB);
# their outputs stay in the 129 MB L2.  Traffic scales with the snapshot
# count.
TRAFFIC_PER_SNAPSHOT = {"eigensolve": 0.117e6 / 2000, "snapshots": 9.458e6 / 2000,
                        "phase": 13.288e6 / 2000}
# Batches of at least this many snapshots take the Householder + QL
# eigensolve (smaller ones the warp Jacobi)
QL_MIN_SNAPSHOTS = 4096


def parse_args():
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--orientations", type=int, default=10000)
    p.add_argument("--times", type=int, default=4096)
    p.add_argument("--fp64-steps", type=int, default=3)
    p.add_argument("--cpu-orientations", type=int, default=2500,
                   help="orientations in the bounded CPU-baseline sample (~10 s)")
    p.add_argument("--ref-orientations", type=int, default=400,
                   help="orientations per step of the --impl reference arm")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--celio-orient", type=int, default=8,
                   help="celio workload: orientations (19 random states each)")
    p.add_argument("--celio-times", type=int, default=50, help="celio workload: time samples")
    p.add_argument("--celio-nuclei", type=int, default=4,
                   help="celio workload: vanadium nuclei (4: dim 8192 in shared memory; "
                        "5: dim 65536 from global memory)")
    p.add_argument("--celio-states", type=int, default=19,
                   help="celio workload: random states per orientation")
    p.add_argument("--c4-systems", type=int, default=512,
                   help="config4: systems (the full configuration: 4096)")
    p.add_argument("--c4-orientations", type=int, default=32,
                   help="config4: orientations per system (the full configuration: 256)")
    p.add_argument("--c3-fields", type=int, default=2000,
                   help="config3 workload: fields of the ALC scan (a smaller scan for profiling)")
    p.add_argument("--c4-graph", choices=["on", "off"], default="on",
                   help="config4 workload: replay the batch from a CUDA graph")
    p.add_argument("--c4-dims", default="4,8,12,24,48,96,192",
                   help="config4 workload: dimensions drawn for the systems")
    p.add_argument("--workload", default="config2",
                   choices=["config1", "config2", "config3", "config4", "config5", "lindblad",
                            "celio"],
                   help="config2 (default) is the headline; the others print their own line")
    return p.parse_args()


# ---------------------------------------------------------------- distributed

def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gb300" and torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_model():
    """Host CPU model name (lscpu / /proc/cpuinfo), or None."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


# ---------------------------------------------------------------- workload

def build_workload(args):
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300 import workloads
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.config2(n_orient=args.orientations, n_times=args.times)
    sy = wl.system()
    qs, ws = orientation_rows_to_quats(wl.orientations)
    N = len(qs)
    ws = ws * (N / ws.sum())
    p = wl.polarization / np.linalg.norm(wl.polarization)
    B_lab = Q.rotate(qs, wl.fields[0])
    p_lab = Q.rotate(qs, p)
    return wl, sy, B_lab, p_lab, ws / N


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """SM clock and clock-event reasons sampled during the timed region.

    Polls NVML (read-only queries through ctypes: no Python NVML package is
    needed) every 5 ms from a thread; falls back to ``nvidia-smi -lms 200``
    when NVML cannot be loaded."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.samples, self.max_mhz, self.reasons = [], None, set()
        self.proc = self.thread = None
        self.source = "none"
        if self._start_nvml(gpu_index):
            return
        self.path = tempfile.mktemp(suffix=".csv")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
            self.source = "nvidia-smi"
        except (OSError, FileNotFoundError):
            self.proc = None

    def _start_nvml(self, gpu_index):
        import ctypes
        import threading

        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return False
            h = ctypes.c_void_p()
            uuid = None
            try:
                import torch

                uuid = str(getattr(torch.cuda.get_device_properties(gpu_index), "uuid", "") or "")
            except Exception:
                uuid = None
            ok = False
            if uuid:
                key = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
                ok = lib.nvmlDeviceGetHandleByUUID(key.encode(), ctypes.byref(h)) == 0
            if not ok and lib.nvmlDeviceGetHandleByIndex_v2(gpu_index, ctypes.byref(h)) != 0:
                return False
            mx = ctypes.c_uint(0)
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        except (OSError, AttributeError):
            return False
        self._stop = threading.Event()

        def poll():
            clk, rs = ctypes.c_uint(0), ctypes.c_ulonglong(0)
            while not self._stop.is_set():
                if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0:
                    self.samples.append(float(clk.value))
                if get_reasons(h, ctypes.byref(rs)) == 0:
                    for bit, name in self.REASONS.items():
                        if rs.value & bit:
                            self.reasons.add(name)
                self._stop.wait(0.005)

        self.thread = threading.Thread(target=poll, daemon=True)
        self.thread.start()
        self.source = "nvml"
        return True

    def stop(self):
        if self.thread is not None:
            self._stop.set()
            self.thread.join(timeout=5)
            if not self.samples:
                return None
            return {"sm_mhz": statistics.median(self.samples),
                    "sm_max_mhz": self.max_mhz or max(self.samples),
                    "reasons": sorted(self.reasons), "samples": len(self.samples),
                    "source": self.source}
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm), "source": self.source}


# ---------------------------------------------------------------- CPU reference

def cpu_reference_rate(sy, B_lab, p_lab, times, n_orient, threads, wscale=None):
    """Samples/s of the reference's fast path on the host: per orientation
    H = Hsys + b.Z, numpy eigh, A = |U^dag (sigma (x) 1) U|^2, W, and the
    reference's own Cython cosine sum compiled from its sources
    (oracle/_ref), with all host threads; the C restatement
    (oracle/fast_cos_sum.c) when the reference kernel is absent.  Also
    returns the weighted average P(t) of those orientations (weights
    wscale, renormalised over the sample), for the parity check."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import build as obuild
    from oracle import port

    kind = "port"
    kernel = None
    try:
        path = obuild.build_ref()
        if path:
            import importlib.util

            spec = importlib.util.spec_from_file_location(obuild.REF_MODULE, path)
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            kernel = mod.parallel_fast_time_evolve
            kind = "reference"
    except Exception:
        kernel = None
    obuild.build_port()
    Hsys = sy.hamiltonian_matrix()
    Z = sy.zeeman_operators()
    d = Hsys.shape[0] // 2
    t = np.ascontiguousarray(times, dtype=np.float64)
    w = np.ones(n_orient) if wscale is None else np.asarray(wscale[:n_orient], dtype=float)
    t0 = time.perf_counter()
    acc = np.zeros(len(t))
    for k in range(n_orient):
        H = Hsys + np.einsum("a,aij->ij", B_lab[k], Z)
        A, W, _ = port.fast_amplitudes(H, port.sigma_mu(p_lab[k]), d)
        if kernel is not None:
            r = np.asarray(kernel(t, d, np.ascontiguousarray(A), np.ascontiguousarray(W)))
        else:
            r = port.fast_cos_sum(t, d, A, W, threads)
        acc += w[k] * 0.5 * r
    dt = time.perf_counter() - t0
    return n_orient * len(t) / dt, dt, kind, acc / w.sum()


def cpu_evolve_rate(spins, sy, B_lab, p_lab, times, n_orient):
    """Samples/s of the reference's general evolve on the host, per
    orientation: numpy eigh, rho0' and O' basis changes and the per-time loop
    of Hamiltonian.evolve (oracle.port.evolve_per_time restates it,
    muspinsim/hamiltonian.py:40-117), with numpy's default threads; and the
    largest deviation from the fast path's P(t) on the same orientations."""
    from oracle import port
    from tests.helpers import oracle_system

    osy = oracle_system(list(spins), [])
    Hsys, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    t = np.asarray(times, dtype=float)
    Smu = [port.embed(osy.Is, {0: a}) for a in "xyz"]
    dt = 0.0
    for k in range(n_orient):
        H = Hsys + np.einsum("a,aij->ij", B_lab[k], Z)
        rho = port.rho0(osy, B_lab[k], p_lab[k], np.inf)
        O = sum(p_lab[k][a] * Smu[a] for a in range(3))
        t0 = time.perf_counter()
        port.evolve_per_time(H, rho, t, [O])
        dt += time.perf_counter() - t0
    return n_orient * len(t) / dt, dt


# ---------------------------------------------------------------- main arms

def run_reference(args, world, rank):
    if rank != 0:
        return 0
    wl, sy, B_lab, p_lab, _ = build_workload(args)
    threads = os.cpu_count() or 1
    n = min(args.ref_orientations, len(B_lab))
    rates = []
    for step in range(args.warmup + args.steps):
        rate, dt, kind, _ = cpu_reference_rate(sy, B_lab, p_lab, wl.times, n, threads)
        if step >= args.warmup:
            rates.append((rate, dt))
    value = statistics.median([r for r, _ in rates])
    ms = statistics.median([d for _, d in rates]) * 1e3
    sample = f"{n} of {len(B_lab)} orientations x {len(wl.times)} times per step"
    ev_n = 4
    ev_rate, ev_dt = cpu_evolve_rate(wl.spins, sy, B_lab, p_lab, wl.times, ev_n)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "orientations": len(B_lab), "times": len(wl.times),
                   "dim": 24, "l2": "n/a (host)"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": kind,
                         "cpu_model": cpu_model(), "sample": sample},
        "evolve": {"value": ev_rate, "unit": "samples/s", "seconds": ev_dt,
                   "sample": f"{ev_n} orientations x {len(wl.times)} times",
                   "path": "Hamiltonian.evolve restated per time step (oracle.port."
                           "evolve_per_time), numpy default threads"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gb300(args, world, rank, local):
    import torch

    from muspinsim_gb300 import _lib, kernels
    from muspinsim_gb300.powder import powder_average

    torch.cuda.set_device(local)
    wl, sy, B_lab, p_lab, wscale = build_workload(args)
    S, T = len(B_lab), len(wl.times)
    Hsys, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    n = Hsys.shape[0]
    slot = np.zeros(S, dtype=np.int32)

    def plan(prec):
        return kernels.PowderPlan(n, Hsys, Z, B_lab, p_lab, wscale, slot, 1, wl.times,
                                  mode=_lib.MODE_FAST, precision=prec, dims=list(sy.dimension),
                                  mu_index=sy.muon_index, gammas=sy.gammas)

    mixed, fp64 = plan(_lib.PREC_MIXED), plan(_lib.PREC_FP64)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(pl, steps, timer=None):
        times_ms = []
        for _ in range(steps):
            flush.fill_(1.0)  # evict L2 between iterations (outside the events)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            pl.run(timer)
            ev1.record(stream)
            ev1.synchronize()
            times_ms.append(ev0.elapsed_time(ev1))
        return times_ms

    # warm-up
    for _ in range(args.warmup):
        mixed.run()
    fp64.run()
    torch.cuda.synchronize()

    timer = kernels.StageTimer()
    timer.read()
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    ms_mixed = timed(mixed, args.steps, timer)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    stages, runs = timer.read()
    res_mixed = mixed.out.clone()
    st_mixed = int(mixed.status[:S].max().item())

    ms_fp64 = timed(fp64, max(1, args.fp64_steps))
    res_fp64 = fp64.out.clone()
    st_fp64 = int(fp64.status[:S].max().item())
    dP = float((res_mixed - res_fp64).abs().max().item())

    # e2e through the public API, host inputs
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = powder_average(sy, wl.orientations, wl.fields[0], wl.polarization, wl.times,
                           precision="mixed")
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    dP_e2e = float(np.abs(r - res_fp64[0].cpu().numpy()).max())
    # per call: the orientation rows go up (the system's Hsys and Z stay on
    # the device after the first call, like a model's weights, and the time
    # grid is re-uploaded only when it changes, which it does not here); the
    # powder average and the per-snapshot status come back
    h2d = int(np.asarray(wl.orientations).nbytes)
    d2h = T * 8 + S * 4

    t_mixed = statistics.median(ms_mixed)
    t_fp64 = statistics.median(ms_fp64)
    t_e2e = statistics.median(e2e_ms)
    t_mixed_max = max_over_ranks(world, t_mixed)
    samples = S * T
    value = world * samples / (t_mixed_max * 1e-3)

    # roofline per stage (live CUDA-event stage times; each stage is one
    # kernel on this path) and of the dominant one
    per_run = {k: v / max(runs, 1) for k, v in stages.items()}
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    fp32_peak = SMS * FP32_FMA_PER_SM * 2 * 2070e6 / 1e12
    bf16 = peaks.get("bf16_tflops")
    tf32_peak = (bf16 if bf16 else 1900.0) / 2.0  # dense TF32 runs at half the bf16 rate
    tf32_src = ("measured bf16 burst / 2 (MEASURED_PEAKS.json)" if bf16
                else "fallback 1.9 PF/s bf16 / 2")
    # algorithmic work per snapshot: eigensolve 36 n^3 (six Jacobi sweeps) or
    # 19 n^3 (Householder 16/3 n^3, QL rotations 6 n^3 at ~n^2 rotations,
    # back-transformation 8 n^3), eigenbasis products 32 n^3; per time
    # sample 4 n^2 + 2 (phase sum + accumulation)
    ql = S >= QL_MIN_SNAPSHOTS
    kernels_rl = {
        "eigensolve": (("msp_ql_warp_kernel<24,4> (Householder + QL, four matrices a warp)"
                        if ql else "msp_jacobi_warp_kernel<24>"),
                       (19.0 if ql else 36.0) * n**3 * S, "fp32-pipe", fp32_peak,
                       "nominal FP32 FMA pipe (152 x 128 x 2 x 2070 MHz)"),
        "snapshots": ("msp_snap_fast_kernel<float,true,true> (refinement + amplitudes)",
                      32.0 * n**3 * S, "fp32-pipe", fp32_peak,
                      "nominal FP32 FMA pipe (152 x 128 x 2 x 2070 MHz)"),
        "phase": ("msp_phase_tcw_kernel<32> (tcgen05 kind::tf32, 3xTF32, A in tensor memory, "
                  "warp-specialised)",
                  (4.0 * n * n) * samples, "tensor", tf32_peak, tf32_src),
        "reduce": ("msp_reduce_kernel", 2.0 * samples, "fp32-pipe", fp32_peak,
                   "nominal FP32 FMA pipe"),
    }
    rl_all = {}
    for k, (kn, fl, bound, pk, src) in kernels_rl.items():
        if per_run.get(k, 0.0) > 0.0:
            ach = fl / (per_run[k] * 1e-3) / 1e12
            rl_all[k] = {"kernel": kn, "ms": per_run[k], "achieved_tflops": ach,
                         "peak_tflops": pk, "frac": ach / pk, "bound": bound,
                         "peak_source": src}
    dom = max(rl_all, key=lambda k: rl_all[k]["ms"])
    kn, fl, bound, pk, src = kernels_rl[dom]
    achieved = rl_all[dom]["achieved_tflops"]
    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_mixed_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Householder + QL eigensolve, 3xTF32 phase sum) + double-word f32 "
                 "(refinement, eigenvalues, phase records, item reduction); f64 only in the "
                 "final per-time sums",
        "data": "synthetic (seeded couplings, ZCW-style grid)",
        "config": {"workload": WORKLOAD, "orientations": S, "times": T, "dim": n,
                   "precision": "mixed", "l2": "flushed between timed steps (258 MB write)",
                   "parallelism": f"replicas x{world}"},
        "max_abs_dP_mixed_vs_fp64": dP,
        "fp64": {"value": world * samples / (max_over_ranks(world, t_fp64) * 1e-3),
                 "unit": "samples/s", "ms_per_step": t_fp64, "steps": len(ms_fp64)},
        "mixed_over_fp64": t_fp64 / t_mixed,
        "status_max": {"mixed": st_mixed, "fp64": st_fp64},
        "e2e": {"value": world * samples / (max_over_ranks(world, t_e2e) * 1e-3),
                "unit": "samples/s", "ms_per_step": t_e2e, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "api": "muspinsim_gb300.powder_average",
                "max_abs_dP_vs_fp64": dP_e2e,
                "h2d": "orientation rows (time grid cached on the device)"},
        "stage_ms_per_step": per_run,
        "roofline": {
            "bound": bound, "kernel": kn, "achieved": achieved, "peak": pk, "unit": "TFLOP/s",
            "frac": achieved / pk,
            "traffic": TRAFFIC_PER_SNAPSHOT.get(dom, 0.0) * S or None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                              "scaled per snapshot",
            "algorithmic": {"eigensolve": ("19 n^3" if ql else "36 n^3") + " per snapshot",
                            "snapshots": "32 n^3 per snapshot",
                            "phase": "4 n^2 per sample", "reduce": "2 per sample"}[dom],
            "peak_source": src,
            "stages": rl_all,
        },
        "clocks": clk,
        # double-word split of the system matrices, eigensolve, refinement,
        # schedule, phase sum, reduction
        "gpu_launches": 6 * args.steps,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        nc = min(args.cpu_orientations, S)
        rate, dt, kind, ref_avg = cpu_reference_rate(sy, B_lab, p_lab, wl.times, nc, threads,
                                                     wscale)
        line["cpu_baseline"] = {"value": rate, "unit": "samples/s", "cores": threads,
                                "kind": kind, "cpu_model": cpu_model(), "seconds": dt,
                                "sample": f"{nc} of {S} orientations x {T} times"}
        # parity at the benchmark's size: both GPU forms on the same sample of
        # orientations (weights renormalised over it) against the reference's
        # own P(t), on the full time grid
        sub_w = wscale[:nc] / wscale[:nc].sum()
        par = {}
        for name, prec in (("mixed", _lib.PREC_MIXED), ("fp64", _lib.PREC_FP64)):
            pl = kernels.PowderPlan(n, Hsys, Z, B_lab[:nc], p_lab[:nc], sub_w,
                                    np.zeros(nc, dtype=np.int32), 1, wl.times,
                                    mode=_lib.MODE_FAST, precision=prec)
            got = pl.run()[0].cpu().numpy()
            par[name] = float(np.abs(got - ref_avg).max())
        line["max_abs_dP_vs_reference"] = {
            **par, "sample": f"{nc} of {S} orientations x {T} times", "reference": kind,
            "gates": {"mixed": 1e-6, "fp64": 1e-10}}
    if rank == 0:
        print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- CPU pools

def _pool_init():
    # one BLAS / OpenMP thread per worker process: the pool supplies the
    # parallelism
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"


def _snapshot_task(task):
    """Worker: the oracle's per-snapshot path (numpy eigh + the reference's
    arithmetic) for a chunk of (spins, couplings, orientation row, field,
    polarisation, times, y) items; returns the weighted sum of results."""
    from oracle import port
    from tests.helpers import oracle_system

    spins, couplings, rows, fields, pol, times, y, weights = task
    osy = oracle_system(spins, couplings)
    Hn, Zn = osy.hamiltonian(), osy.zeeman_operators()
    acc = 0.0
    for row, B, w in zip(rows, fields, weights):
        q = port.orientation_quat(row)[0]
        r = port.snapshot(osy, Hn, Zn, q, 1.0, np.asarray(B, float), pol, np.inf, np.zeros(3),
                          times, y=y)
        acc = acc + w * np.asarray(r)
    return acc


def _lindblad_task(task):
    """Worker: the oracle's dissipative powder average (numpy eig of the
    Lindbladian per snapshot) over a chunk of orientation rows."""
    from oracle import port
    from tests.helpers import oracle_system

    spins, couplings, rows, field, pol, temperature, times, diss = task
    osy = oracle_system(spins, couplings)
    return port.powder_average(osy, rows, field, pol, temperature, times, dissipation=diss)


def cpu_pool_map(tasks, threads, fn=None):
    """Run fn (default _snapshot_task) over tasks in a spawn pool of
    `threads` processes (spawn: no process is forked from one that holds a
    CUDA context)."""
    import multiprocessing as mp

    with mp.get_context("spawn").Pool(threads, initializer=_pool_init) as pool:
        return pool.map(fn or _snapshot_task, tasks)


def _chunks(items, k):
    n = len(items)
    return [items[i * n // k:(i + 1) * n // k] for i in range(k) if i * n // k < (i + 1) * n // k]


# ---------------------------------------------------------------- other workloads

def _events_ms(fn, steps, flush=None):
    """Median milliseconds of fn() over `steps` runs, CUDA events on the
    current stream, L2 flushed before each run when `flush` is given."""
    import torch

    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def _wall_ms(fn, steps):
    import torch

    ts = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        ts.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(ts)


def _line(metric, value, unit, ms, args, world, workload, config, **extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded couplings, ZCW-style grid)",
            "config": dict({"workload": workload}, **config)}
    line.update(extra)
    return line


def run_config1(args, world, rank, local):
    """mu + e (dim 4), 1 orientation, 1000 times: the reference's own
    CPU-sized case, plain FP64 as the reference computes it."""
    import torch

    from muspinsim_gb300 import _lib, kernels, workloads
    from muspinsim_gb300.powder import powder_average

    wl = workloads.config1()
    sy = wl.system()
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()
    B = np.atleast_2d(wl.fields[0])
    p = np.atleast_2d(wl.polarization)
    T = len(wl.times)
    plan = kernels.PowderPlan(4, Hs, Z, B, p, np.ones(1), np.zeros(1, np.int32), 1, wl.times,
                              precision=_lib.PREC_FP64, dims=list(sy.dimension))
    for _ in range(args.warmup):
        plan.run()
    ms = _events_ms(plan.run, args.steps)
    call = lambda: powder_average(sy, wl.orientations, wl.fields[0], wl.polarization, wl.times)
    for _ in range(args.warmup):
        call()
    e2e = _wall_ms(call, args.steps)
    line = _line("P(t) samples/s, plain FP64", T / (ms * 1e-3), "samples/s", ms, args, world,
                 "mu_e_dim4_1_orient_1000_t", {"orientations": 1, "times": T, "dim": 4},
                 dtype="f64",
                 e2e={"value": T / (e2e * 1e-3), "unit": "samples/s", "ms_per_step": e2e,
                      "h2d_bytes_per_step": int(np.asarray(wl.orientations).nbytes) + T * 8,
                      "d2h_bytes_per_step": T * 8 + 4, "api": "muspinsim_gb300.powder_average"},
                 gpu_launches=4 * args.steps,
                 note="launch-bound: one snapshot of a 4x4 Hamiltonian")
    if not args.no_cpu_baseline:
        from oracle import port
        from tests.helpers import oracle_system

        threads = os.cpu_count() or 1
        reps, total, kind = 200, 0.0, "port"
        for _ in range(reps):
            _, dt, kind, _ = cpu_reference_rate(sy, B, p, wl.times, 1, threads)
            total += dt
        line["cpu_baseline"] = {"value": reps * T / total, "unit": "samples/s", "cores": threads,
                                "kind": kind, "cpu_model": cpu_model(),
                                "sample": f"{reps} runs of the fast path (numpy eigh + the "
                                          "reference's OpenMP cosine sum)"}
    return line


def run_config3(args, world, rank, local):
    """ALC field scan: mu, e, 3 x 1H (dim 32), 2000 fields x 1000
    orientations, decaying integral with tau = MU_TAU.  Unit: one
    (field, orientation) integral."""
    import torch

    from muspinsim_gb300 import _lib, kernels, workloads
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.constants import MU_TAU
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.config3(n_fields=args.c3_fields)
    sy = wl.system()
    qs, ws = orientation_rows_to_quats(wl.orientations)
    No = len(qs)
    ws = ws * (No / ws.sum())
    Nf = len(wl.fields)
    p_or = Q.rotate(qs, wl.polarization)
    R = Q.rotation_matrix(qs)  # (No, 3, 3)
    B_lab = np.einsum("oab,fb->foa", R, wl.fields).reshape(-1, 3)
    p_lab = np.broadcast_to(p_or, (Nf, No, 3)).reshape(-1, 3)
    wsc = np.broadcast_to(ws / No, (Nf, No)).reshape(-1)
    slot = np.repeat(np.arange(Nf, dtype=np.int32), No)
    units = Nf * No
    Hs, Z = sy.hamiltonian_matrix(), sy.zeeman_operators()

    def plan(prec, sub=None):
        sl = slice(None) if sub is None else slice(0, sub * No)
        nslots = Nf if sub is None else sub
        return kernels.PowderPlan(32, Hs, Z, B_lab[sl], p_lab[sl], wsc[sl], slot[sl], nslots,
                                  np.array([np.inf]), mode=_lib.MODE_INTEGRAL, precision=prec,
                                  dims=list(sy.dimension), mu_index=0, gammas=sy.gammas,
                                  tau=MU_TAU)

    mixed = plan(_lib.PREC_MIXED)
    for _ in range(args.warmup):
        mixed.run()
    ms = _events_ms(mixed.run, args.steps)
    sub = min(100, Nf)  # FP64 on 100 fields x all orientations (5% of the full scan)
    f64 = plan(_lib.PREC_FP64, sub)
    f64.run()
    ms64 = _events_ms(f64.run, max(1, args.fp64_steps))
    dP = float((mixed.out[:sub] - f64.out).abs().max().item())
    line = _line("ALC (field, orientation) integrals/s, mixed precision", units / (ms * 1e-3),
                 "integrals/s", ms, args, world, f"mu_e_3H_dim32_alc_{Nf}_fields_{No}_orient",
                 {"fields": Nf, "orientations": No, "dim": 32, "tau_us": MU_TAU,
                  "l2": "inputs (96 MB of field/polarisation) resident; not flushed"},
                 dtype="f32 Householder + QL + double-word f32 refinement and integral sums",
                 fp64={"value": sub * No / (ms64 * 1e-3), "unit": "integrals/s",
                       "ms_per_step": ms64, "sample": f"{sub} of {Nf} fields x {No} orientations"},
                 max_abs_dIntegral_mixed_vs_fp64=dP,
                 status_max=int(mixed.status[:units].max().item()),
                 # double-word split, eigensolve, refinement + integrals,
                 # schedule, reduction
                 gpu_launches=5 * args.steps)
    if not args.no_cpu_baseline:
        from oracle import port
        from tests.helpers import oracle_system

        threads = os.cpu_count() or 1
        nsamp = 200 * threads
        items = [((k * 10) % Nf, (k * 37) % No) for k in range(nsamp)]
        tasks = [(list(wl.spins), wl.couplings, [wl.orientations[o] for _, o in c],
                  [wl.fields[f] for f, _ in c], wl.polarization, np.array([np.inf]),
                  "integral", np.ones(len(c))) for c in _chunks(items, threads)]
        cpu_pool_map(tasks[:1], threads)  # start-up and imports outside the timing
        t0 = time.perf_counter()
        cpu_pool_map(tasks, threads)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nsamp / dt, "unit": "integrals/s", "cores": threads,
                                "kind": "port", "cpu_model": cpu_model(),
                                "sample": f"{nsamp} (field, orientation) units over {threads} "
                                          "processes (numpy eigh + the reference's integral)"}
    return line


def run_config4(args, world, rank, local):
    """Heterogeneous batch: spin systems of dimension 4 ... 192, one output
    row each, through msp_multi_run (size buckets, persistent launches,
    concurrent streams, CUDA graph).  Scaled by default to 512 systems x 32
    orientations (the 4,096 x 256 configuration, --c4-systems 4096
    --c4-orientations 256, has the same per-snapshot mix: about 11 s per
    step in mixed precision, two minutes in FP64; --fp64-steps 0 skips the
    FP64 comparison)."""
    import torch

    from muspinsim_gb300 import workloads
    from muspinsim_gb300.multi import MultiSystemBatch

    n_sys, n_or = args.c4_systems, args.c4_orientations
    dims = tuple(int(x) for x in args.c4_dims.split(","))
    graph = args.c4_graph == "on"
    wls = workloads.config4(n_systems=n_sys, n_orient=n_or, dims=dims)
    systems = [w.system() for w in wls]
    T = len(wls[0].times)
    out = {}
    for prec in ("mixed", "fp64") if args.fp64_steps > 0 else ("mixed",):
        b = MultiSystemBatch(systems, wls[0].orientations, wls[0].fields[0],
                             wls[0].polarization, wls[0].times, precision=prec)
        for _ in range(max(1, args.warmup if prec == "mixed" else 1)):
            b.run(graph=graph)
        torch.cuda.synchronize()
        # every timed step of the mixed batch; the FP64 batch (~1.8 s a step
        # at 512 x 32) for --fp64-steps of them
        nsteps = max(1, args.steps if prec == "mixed" else args.fp64_steps)
        ms = _events_ms(lambda: b.run(graph=graph), nsteps)
        out[prec] = (ms, b.plan.out.clone(), b.plan.info())
        b.plan.close()
    ms, res, info = out["mixed"]
    samples = n_sys * n_or * T
    dP = float((res - out["fp64"][1]).abs().max().item()) if "fp64" in out else None
    buckets = [{k: bi[k] for k in ("n", "num_systems", "num_snap", "num_chunks",
                                    "snap_threads", "grid")} for bi in info]
    cfg = {"systems": n_sys, "orientations": n_or, "times": T, "dims": list(dims),
           "graph": graph}
    if (n_sys, n_or) != (4096, 256):
        cfg["scaled_from"] = "4096 systems x 256"
    return _line("heterogeneous-batch P(t) samples/s, mixed precision", samples / (ms * 1e-3),
                 "samples/s", ms, args, world,
                 f"{min(dims)}_to_{max(dims)}_dim_systems_{n_sys}x{n_or}_orient_{T}_t", cfg,
                 dtype="f32 (Jacobi for n <= 64, Householder + QL for n > 64 and for "
                       "n <= 32 buckets of 4,096+ snapshots; double-word refinement; phase sum)",
                 fp64=({"value": samples / (out["fp64"][0] * 1e-3),
                        "ms_per_step": out["fp64"][0]} if "fp64" in out else None),
                 max_abs_dP_mixed_vs_fp64=dP, buckets=buckets)


def run_config5(args, world, rank, local):
    """Differentiable fit: F-mu-F (dim 8), 2000 orientations, 1000 times:
    loss + analytic gradient (forward powder average and the adjoint
    kernel) evaluations per second."""
    import torch

    from muspinsim_gb300 import workloads
    from muspinsim_gb300.adjoint import GradientFitter, TorchSpinHamiltonian

    wl = workloads.config5()
    r = [np.asarray(v, dtype=float) for _, _, v in wl.couplings]
    th = TorchSpinHamiltonian(wl.spins)
    d = th.device
    dirs = [torch.as_tensor(r[k] / np.linalg.norm(r[k]), device=d) for k in range(2)]
    fixed = th.dipolar(1, 2, r[2])
    B0 = torch.zeros(3, dtype=torch.float64, device=d)

    def model(ps):
        return th.dipolar(0, 1, ps[0] * dirs[0]) + th.dipolar(0, 2, ps[1] * dirs[1]) + fixed, B0

    rng = np.random.default_rng(1005)
    data = 0.5 * np.cos(np.linspace(0, 3, wl.times.size)) + rng.normal(0, 0.01, wl.times.size)
    fits = {p: GradientFitter(model, th.Z, wl.orientations, wl.times, data, wl.polarization,
                              precision=p) for p in ("mixed", "fp64")}
    ps = [torch.tensor(float(np.linalg.norm(r[k])), dtype=torch.float64, device=d,
                       requires_grad=True) for k in range(2)]

    def step(prec="mixed"):
        L, g = fits[prec].loss_and_grad(ps)
        return L, g

    for _ in range(args.warmup):
        step()
        step("fp64")
    ms = _wall_ms(step, args.steps)
    ms64 = _wall_ms(lambda: step("fp64"), args.steps)
    Lm, gm = step()
    Ld, gd = step("fp64")
    gm = np.array([float(g) for g in gm])
    gd = np.array([float(g) for g in gd])
    # central finite differences of the FP64 loss
    fd = []
    with torch.no_grad():
        for k in range(2):
            h = 1e-5 * float(ps[k])
            lo = [p.detach().clone() for p in ps]
            hi = [p.detach().clone() for p in ps]
            lo[k] -= h
            hi[k] += h
            fd.append((float(fits["fp64"].loss(hi)) - float(fits["fp64"].loss(lo))) / (2 * h))
    fd = np.array(fd)
    line = _line("loss + gradient evaluations/s (mixed forward, FP64 adjoint)", 1e3 / ms,
                 "evaluations/s", ms, args, world, "F_mu_F_dim8_2000_orient_1000_t_fit",
                 {"orientations": len(wl.orientations), "times": len(wl.times), "dim": 8,
                  "parameters": 2},
                 dtype="f32 Jacobi + double-word refinement (forward), f64 (adjoint)",
                 fp64={"value": 1e3 / ms64, "ms_per_step": ms64},
                 loss_rel_diff_mixed_vs_fp64=float(abs(float(Lm) - float(Ld)) / abs(float(Ld))),
                 grad_rel_diff_mixed_vs_fp64=float(np.abs(gm - gd).max() / np.abs(gd).max()),
                 grad_rel_err_fp64_vs_central_fd=float(np.abs(gd - fd).max() / np.abs(fd).max()),
                 e2e={"value": 1e3 / ms, "unit": "evaluations/s", "ms_per_step": ms,
                      "note": "wall clock of torch autograd loss + backward"})
    if not args.no_cpu_baseline:
        from oracle import port
        from tests.helpers import oracle_system

        threads = os.cpu_count() or 1
        rows = list(wl.orientations)
        tasks = [(list(wl.spins), wl.couplings, c, [np.zeros(3)] * len(c), wl.polarization,
                  wl.times, "asymmetry", np.ones(len(c)) / len(rows))
                 for c in _chunks(rows, threads)]
        cpu_pool_map(tasks[:1], threads)  # start-up and imports outside the timing
        t0 = time.perf_counter()
        cpu_pool_map(tasks, threads)
        dt = time.perf_counter() - t0
        # a central-difference gradient in 2 parameters costs 5 forward runs
        line["cpu_baseline"] = {"value": 1.0 / (5 * dt), "unit": "evaluations/s",
                                "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                                "sample": "one forward run over all orientations in "
                                          f"{threads} processes; loss + central-FD gradient = "
                                          "5 runs"}
    return line


def run_lindblad(args, world, rank, local):
    """Dissipative powder average (the Lindbladian branch of run_single):
    mu, e, 1H (n = 8, superoperator 64 x 64), dissipation on the electron
    and the proton, B = 3 mT, T = 20 K, 500 ZCW-style orientations, 1000
    times on 0-10 us.  FP64 (exp(2 pi L dt) propagation on the device)."""
    import torch

    from muspinsim_gb300 import _lib, kernels, workloads
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats, zcw_gen

    rng = np.random.default_rng(1006)
    wl = workloads.Workload(
        name="mu_e_H_lindblad", spins=["mu", "e", "H"],
        couplings=[("hyperfine", {"i": 1}, workloads.random_hyperfine(rng, 30.0)),
                   ("hyperfine", {"i": 3}, workloads.random_hyperfine(rng, 5.0))],
        orientations=zcw_gen(500), fields=np.array([[0.0, 0.0, 0.003]]),
        polarization=np.array([0.0, 0.0, 1.0]), times=np.linspace(0.0, 10.0, 1000),
        temperature=20.0)
    diss = {1: 2.0, 2: 0.3}
    sy = wl.system()
    qs, ws = orientation_rows_to_quats(wl.orientations)
    N = len(qs)
    ws = ws * (N / ws.sum())
    B_lab, p_lab = Q.rotate(qs, wl.fields[0]), Q.rotate(qs, wl.polarization)
    n = 8
    S_ops = np.array([[sy.operator({i: ax}).matrix.toarray() for ax in "xyz"]
                      for i in range(3)], dtype=complex)
    T = len(wl.times)

    def step(prec=_lib.PREC_MIXED):
        return kernels.lindblad_run(n, sy.hamiltonian_matrix(), sy.zeeman_operators(), S_ops,
                                    list(sy.dimension), 0, sy.gammas, diss, B_lab, p_lab, ws / N,
                                    np.zeros(N, np.int32), 1, wl.times,
                                    temperature=wl.temperature, precision=prec)[0]

    for _ in range(args.warmup):
        step()
        step(_lib.PREC_FP64)
    ms = _events_ms(step, max(1, args.steps))
    ms64 = _events_ms(lambda: step(_lib.PREC_FP64), max(1, min(args.steps, 3)))
    out = step().cpu().numpy()[0]
    out64 = step(_lib.PREC_FP64).cpu().numpy()[0]
    line = _line("dissipative powder P(t) samples/s, double-word FP32 propagation",
                 N * T / (ms * 1e-3), "samples/s", ms,
                 args, world, "mu_e_H_lindblad_500_orient_1000_t",
                 {"orientations": N, "times": T, "dim": n, "superoperator": n * n,
                  "dissipation_MHz": {"e": 2.0, "H": 0.3}, "temperature_K": 20.0},
                 dtype="f32 double-word (propagation), f64 (construction, measurement)",
                 gpu_launches=5 * max(1, args.steps),
                 fp64={"value": N * T / (ms64 * 1e-3), "ms_per_step": ms64},
                 mixed_over_fp64=ms64 / ms,
                 max_abs_dP_mixed_vs_fp64=float(np.abs(out - out64).max()),
                 note="each step uploads the orientation vectors (host inputs)")
    if not args.no_cpu_baseline:
        from oracle import port
        from tests.helpers import oracle_system

        osy = oracle_system(wl.spins, wl.couplings)
        sample = 20
        t0 = time.perf_counter()
        ref = port.powder_average(osy, wl.orientations[:sample], wl.fields[0], wl.polarization,
                                  wl.temperature, wl.times, dissipation=diss)
        dt = time.perf_counter() - t0
        gpu20 = kernels.lindblad_run(n, sy.hamiltonian_matrix(), sy.zeeman_operators(), S_ops,
                                     list(sy.dimension), 0, sy.gammas, diss, B_lab[:sample],
                                     p_lab[:sample],
                                     (ws[:sample] * (sample / ws[:sample].sum())) / sample,
                                     np.zeros(sample, np.int32), 1, wl.times,
                                     temperature=wl.temperature)[0].cpu().numpy()[0]
        line["max_abs_dP_vs_oracle_20_orient_fp64"] = float(np.abs(gpu20 - ref).max())
        # the timed baseline: the same oracle path on every host core, ~5 s
        # of work per process, timed after the (spawn) pool has started
        import multiprocessing as mp

        threads = os.cpu_count() or 1
        per = max(1, int(round(sample / dt * 5.0)))
        rows = [wl.orientations[k % N] for k in range(per * threads)]

        def tasks_of(rs):
            return [(list(wl.spins), wl.couplings, c, wl.fields[0], wl.polarization,
                     wl.temperature, wl.times, diss) for c in _chunks(rs, threads)]

        with mp.get_context("spawn").Pool(threads, initializer=_pool_init) as pool:
            pool.map(_lindblad_task, tasks_of(rows[:threads]))  # start-up and imports
            t0 = time.perf_counter()
            pool.map(_lindblad_task, tasks_of(rows))
            dtp = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(rows) * T / dtp, "unit": "samples/s",
                                "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                                "sample": f"{len(rows)} orientations over {threads} processes "
                                          "(numpy eig of L per snapshot)"}
    del out
    return line


def celio_flops(dims, batch):
    """Algorithmic flops of one msp_celio_run of `batch`: every factor
    application multiplies V / D groups by a D x D complex matrix (8 real
    flops per complex multiply-add), k passes per time step, T - 1 steps
    per state; the measurements (O(V) per sample) are left out."""
    V = int(np.prod(dims))
    per_pass = sum(8 * V * (dims[d0] * (dims[d1] if d1 >= 0 else 1)) for d0, d1 in batch.digits)
    return per_pass * batch.k * (batch.T - 1) * batch.S * batch.averages


def run_celio(args, world, rank, local):
    """Celio's method with averaged random initial states (the reference's
    native fast variant, muspinsim/celio.py:318-476): mu + 4 51V (I = 7/2,
    dimension 8192), the shape of the reference's own Celio example;
    8 ZCW-style orientations x 19 random states = 152 states (one per SM),
    k = 10, 50 times on 0-10 us.  States stay in shared memory; the line's
    value is the double-word FP32 form, with the FP64 form beside it."""
    from muspinsim_gb300 import celio, workloads
    from muspinsim_gb300 import quaternion as Q
    from muspinsim_gb300.orientations import orientation_rows_to_quats

    wl = workloads.celio_v3si(n_orient=args.celio_orient, n_times=args.celio_times,
                              n_vanadium=args.celio_nuclei, averages=args.celio_states)
    k, A = wl.meta["celio"]
    steps = max(1, min(args.steps, 10))
    sy = wl.system(celio_k=k)
    qs, ws = orientation_rows_to_quats(wl.orientations)
    N = len(qs)
    ws = ws * (N / ws.sum())
    B_lab, p_lab = Q.rotate(qs, wl.fields[0]), Q.rotate(qs, wl.polarization)
    T = len(wl.times)
    Tk = np.full(N, np.inf)
    rows = np.zeros(N, dtype=np.int64)
    batches, ms, outs = {}, {}, {}
    for prec in ("fp64", "mixed"):
        np.random.seed(1234)  # the same random states for both forms
        b = celio.CelioBatch(sy, k, A, B_lab, p_lab, Tk, ws / N, rows, 1, wl.times,
                             precision=prec)
        for _ in range(args.warmup):
            b.run()
        ms[prec] = _events_ms(b.run, steps if prec == "mixed" else max(1, min(steps, 3)))
        outs[prec] = b.run().cpu().numpy()[0]
        batches[prec] = b

    def e2e():
        out = celio.CelioBatch(sy, k, A, B_lab, p_lab, Tk, ws / N, rows, 1, wl.times,
                               precision="mixed").run()
        return out.cpu().numpy()

    e2e()
    e2e_ms = _wall_ms(e2e, steps)
    batch = batches["mixed"]
    dims = list(sy.dimension)
    V = int(np.prod(dims))
    flops = celio_flops(dims, batch)
    cmacs = flops / 8
    fp32_peak = 152 * 128 * 2 * 2.07  # GFLOP/s, nominal FP32 FMA rate at 2.07 GHz
    achieved = flops / (ms["mixed"] * 1e-3) / 1e9
    pipe_ops = cmacs * 24 / (ms["mixed"] * 1e-3) / 1e9  # FP32 ops issued per second (12 f32x2)
    samples = N * T
    line = _line(f"Celio P(t) samples/s (orientation x time, {A} random states each), "
                 "double-word FP32", samples / (ms["mixed"] * 1e-3), "samples/s", ms["mixed"],
                 args, world,
                 f"celio_muV{args.celio_nuclei}_dim{V}_{N}_orient_{A}_states_{T}_t_k{k}",
                 {"orientations": N, "states_per_orientation": A, "times": T, "dim": V,
                  "trotter_k": k, "factors_per_pass": len(batch.digits),
                  "l2": ("states resident in shared memory; HBM traffic is the inputs only"
                         if V <= 8192 else "states in global memory (L2-resident): one launch "
                                           "per factor application")},
                 dtype="f32 double-word", gpu_launches=steps,
                 state_steps_per_s=N * A * (T - 1) / (ms["mixed"] * 1e-3),
                 fp64={"value": samples / (ms["fp64"] * 1e-3), "ms_per_step": ms["fp64"],
                       "achieved_gflops": flops / (ms["fp64"] * 1e-3) / 1e9,
                       "fp64_peak_gflops": 1250.0,
                       "frac": flops / (ms["fp64"] * 1e-3) / 1e9 / 1250.0},
                 mixed_over_fp64=ms["fp64"] / ms["mixed"],
                 max_abs_dP_mixed_vs_fp64=float(np.abs(outs["mixed"] - outs["fp64"]).max()),
                 roofline={"bound": "fp32", "achieved": pipe_ops, "peak": fp32_peak,
                           "unit": "GFLOP/s", "frac": pipe_ops / fp32_peak, "traffic": None,
                           "algorithmic_gflops": achieved,
                           "note": "achieved = FP32 operations issued (12 packed f32x2 "
                                   "instructions = 24 FP32 ops per complex multiply-add of "
                                   "the anchored double-word product) per second; peak = "
                                   "nominal FP32 "
                                   "(152 SMs x 128 lanes x 2 x 2.07 GHz), no measured FP32 "
                                   "figure on this pool"},
                 e2e={"value": samples / (e2e_ms * 1e-3), "unit": "samples/s",
                      "ms": e2e_ms, "h2d_bytes_per_step": int(batch.phases.numel() * 8 +
                                                             batch.mats.numel() * 16),
                      "d2h_bytes_per_step": T * 8,
                      "note": "host factor exponentials, np.random.rand states and uploads "
                              "inside the timed region"})
    if not args.no_cpu_baseline:
        from oracle import port
        from tests.helpers import oracle_system

        osy = oracle_system(wl.spins, wl.couplings)
        fac = port.celio_snapshot_factors(osy, None, wl.times[1] - wl.times[0], k)
        np.random.seed(99)
        one = celio.CelioBatch(sy, k, 2, B_lab[:1], p_lab[:1], Tk[:1], np.ones(1), rows[:1], 1,
                               wl.times)
        gpu = one.run().cpu().numpy()[0]
        one.precision = batch.precision
        gpu_mixed = one.run().cpu().numpy()[0]
        ph = one.phases.cpu().numpy()[0]
        sig = port.sigma_mu(p_lab[0])
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = port.celio_fast_evolve_c(fac, dims, sig, wl.times, k, ph, nthreads=threads)
        dt = time.perf_counter() - t0
        line["max_abs_dP_vs_oracle_1_orient_2_states"] = {
            "fp64": float(np.abs(gpu - ref).max()), "mixed": float(np.abs(gpu_mixed - ref).max())}
        # one state took dt / 2; an orientation sample needs A states
        line["cpu_baseline"] = {"value": T / (dt / 2 * A), "unit": "samples/s", "cores": threads,
                                "kind": "port",
                                "sample": "1 orientation x 2 random states through oracle/celio.c "
                                          "(the reference's native loop restated, OpenMP inside "
                                          "each factor application)"}
    return line


def main():
    args = parse_args()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    elif args.workload != "config2":
        import torch

        torch.cuda.set_device(local)
        fn = {"config1": run_config1, "config3": run_config3, "config4": run_config4,
              "config5": run_config5, "lindblad": run_lindblad, "celio": run_celio}[args.workload]
        line = fn(args, world, rank, local)
        if rank == 0:
            print(json.dumps(line))
        rc = 0
    else:
        rc = run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
