"""Benchmark of the GB300 probit Gibbs sampler.

A step is one sweep of the sampler (latent Z + beta for both colours, the
Omega Wishart draw, the posterior accumulators) over the brain-sized study:
91x109x91 grid, ellipsoidal mask of about 230k voxels, N = 1000 subjects,
P = 5 covariates, single chain, FP32 sweep with FP64 Omega/accumulators.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is subject*voxel updates per second with the
study resident in HBM (device time of the K timed sweeps, L2 flushed between
sweeps); `e2e` is the same metric through the C ABI with host buffers: each
step is one bsg_step_host call that uploads the chain's Omega from host
memory (as the reference's updateSpatCoefGPU does, covarGPU.cu:540), runs the
sweep and reads the new Omega and the column means back
(covarGPU.cu:582,1106-1108).  With N > 1 (torchrun) every
rank runs an independent chain on its own GPU (replicas, weak scaling).
`--impl reference` times the reference's CPU sweep (the oracle's timing port
of covar.cpp's updateZ / updateSpatCoef / updateSpatCoefPrec) on all host
cores, one chain per core; each step is a bounded sample of the study (the
first voxels of each colour), sized so that the timed steps take about
90 s in all.  The `cpu_baseline` of the GPU arm is one such sample of about
10 s.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("subj·voxel updates/s & sweeps/s, batched-split vs plain GPU form, "
          "≤0.5 MCSE err")
UNIT = "subject-voxel updates/s"
WORKLOAD = "brain-sized plain FP32 GPU form: 91x109x91 grid, ellipsoid mask, N=1000, P=5"
C_TN = 40          # FP32 flops of one truncated-normal draw's accept path
L2_FLUSH_BYTES = 512 << 20
L2_MB = 129  # GB300 L2
CPU_CAL_VOX = 2000      # voxels per colour of the CPU calibration sweep
CPU_BASELINE_S = 10.0   # seconds of CPU work in the cpu_baseline sample
CPU_REFERENCE_S = 90.0  # seconds of CPU work in a whole reference-arm run
# The ncu figures of the fused colour kernel on the brain-sized workload
# (DRAM bytes per colour launch, thread instructions per update) are read
# from the committed profile summary, which records the hash of the kernel
# sources it was captured on; the line says "stale" when the sources have
# changed since.
PROFILE = ROOT / "profiles" / "fused_colour_kernel_brain_c1.md"
KERNEL_SOURCES = ["bsg_fused.cuh", "bsg_device.cuh", "bsg_math.cuh", "bsg_wishart.cuh",
                  "bsg_internal.h", "bsg_fused_l1.cu", "bsg_mma.cuh", "bsg_fused_wide.cu"]


def kernel_sources_hash() -> str:
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        h.update((ROOT / "bsglmm_gb300" / "csrc" / f).read_bytes())
    return h.hexdigest()[:16]


def profile_inputs() -> dict:
    """The `bench-inputs` block of the profile summary: key: value lines
    between '<!-- bench-inputs' and '-->'."""
    out = {"source": str(PROFILE.relative_to(ROOT))}
    try:
        text = PROFILE.read_text()
        block = text.split("<!-- bench-inputs", 1)[1].split("-->", 1)[0]
    except (OSError, IndexError):
        return out
    for line in block.strip().splitlines():
        k, _, v = line.partition(":")
        v = v.strip()
        try:
            out[k.strip()] = float(v) if k.strip() != "kernel_sources_sha256" else v
        except ValueError:
            out[k.strip()] = v
    out["stale"] = out.get("kernel_sources_sha256") != kernel_sources_hash()
    return out


def fused_flops_per_update(P: int) -> int:
    """Algorithmic FP32 flops per subject-voxel update: eta = x'beta and the
    X'Z accumulation (2P each) plus the truncated-normal draw."""
    return 4 * P + C_TN


def sweep_bytes(N: int, V: int, P: int, S: int, kept: bool = True) -> int:
    """Minimum HBM bytes of one sweep: outcome bits, beta read+write, the
    Omega pass read of beta, FP64 accumulators (mean, M2, prb mean read and
    write) and 5 B of lattice metadata per voxel."""
    b = N * V // 8 + 8 * P * V + 4 * P * V + 5 * V
    if kept:
        b += 2 * 8 * (2 * P + S) * V
    return b


# ------------------------------------------------------------ utilities --
def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class _Nvml:
    """Read-only NVML queries through the driver's libnvidia-ml (ctypes): the
    SM clock, its maximum and the active clock-event reasons of one GPU."""

    SM = 1  # NVML_CLOCK_SM
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
            0x40: "hw_thermal_slowdown"}

    def __init__(self, target: str):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit_v2")
        self.h = C.c_void_p()
        if target.isdigit():
            st = self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(int(target)), C.byref(self.h))
        else:
            st = self.lib.nvmlDeviceGetHandleByUUID(target.encode(), C.byref(self.h))
        if st != 0:
            raise OSError("no NVML handle for GPU " + target)
        mx = C.c_uint()
        self.max_mhz = (float(mx.value) if self.lib.nvmlDeviceGetMaxClockInfo(
            self.h, self.SM, C.byref(mx)) == 0 else None)
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) \
            or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        clk, r = C.c_uint(), C.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, C.byref(clk)) != 0:
            return None
        bits = r.value if self.reasons_fn(self.h, C.byref(r)) == 0 else 0
        return float(clk.value), {n for b, n in self.BITS.items() if bits & b}


class Clocks:
    """Samples SM clocks and clock-event (throttle) reasons while the timed
    region runs: NVML every millisecond where the driver's library loads
    (a timed region of a few milliseconds still gets several readings), else
    nvidia-smi every 50 ms.  Only reads the settings."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        # the GPU as NVML and nvidia-smi number it: CUDA's device `index`
        # is an entry of CUDA_VISIBLE_DEVICES when that is set
        vis = [x.strip() for x in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
               if x.strip()]
        self.index = vis[index] if index < len(vis) else str(index)
        self.proc = None
        self.nvml = None
        self.lines = []
        self.samples = []
        self._stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.index)
        except (OSError, AttributeError):
            self.nvml = None
        if self.nvml:
            self._t = threading.Thread(target=self._poll, daemon=True)
            self._t.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.index, f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _poll(self):
        while True:
            x = self.nvml.sample()
            if x:
                self.samples.append(x)
            if self._stop.wait(0.001):
                return

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self._stop.set()
        if self.nvml:
            self._t.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml:
            sm = [c for c, _ in self.samples]
            reasons = set().union(*[r for _, r in self.samples]) if self.samples else set()
            return {"sm_mhz": statistics.median(sm) if sm else None,
                    "sm_max_mhz": self.nvml.max_mhz, "samples": len(sm),
                    "reasons": sorted(reasons), "source": "NVML, 1 ms"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": mx, "samples": len(sm), "reasons": sorted(reasons),
                "source": "nvidia-smi, 50 ms"}


def issue_roofline(device: int, updates_per_s: float, prof: dict):
    """The binding resource of the colour kernel is issue slots: thread
    instructions per second (ncu's instructions per update x the live update
    rate of a colour launch) against 4 warp instructions per clock per SM at
    the maximum SM clock."""
    ipu = prof.get("thread_inst_per_update")
    if ipu is None:
        return None
    try:
        import torch
        props = torch.cuda.get_device_properties(device)
        sms = props.multi_processor_count
        mhz = float(subprocess.run(
            ["nvidia-smi", "-i", str(device), "--query-gpu=clocks.max.sm",
             "--format=csv,noheader,nounits"], capture_output=True, text=True,
            timeout=20).stdout.strip().splitlines()[0])
    except Exception:
        return None
    achieved = ipu * updates_per_s / 1e12
    peak = 4 * 32 * sms * mhz * 1e6 / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "Tinst/s (thread instructions)",
            "frac": achieved / peak, "inst_per_update": ipu,
            "inst_source": prof["source"], "stale": prof.get("stale", True)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


# ------------------------------------------------------------ CPU legs ---
def cpu_port_rate(study, threads: int, steps: int, warmup: int, target_s: float):
    """The oracle's timing port of the reference CPU sweep, one independent
    chain per thread.  A short calibration sweep sizes each step to about
    `target_s` seconds: a step sweeps the first `nvox` voxels of each colour,
    up to the whole study.  `warmup` (at least one) untimed steps of that
    size precede the `steps` timed ones."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build_oracle()
    pb = oracle.Problem(study.mask, study.covar, study.data, study.nsubtypes)
    ports = [oracle.Port(pb, seed=1000 + t) for t in range(threads)]
    ncmax = max(pb.n0, pb.n1)

    def run(n, nvox):
        def work(pt):
            for _ in range(n):
                pt.sweep(nvox)
        ts = [threading.Thread(target=work, args=(pt,)) for pt in ports]
        t0 = time.perf_counter()
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        return time.perf_counter() - t0

    cal = min(CPU_CAL_VOX, ncmax)
    run(1, cal)  # first touch of the chains' state
    dt = run(1, cal)
    nvox = int(min(ncmax, max(cal, cal * target_s / max(dt, 1e-6))))
    upd = ports[0].updates(nvox)
    for _ in range(max(warmup, 1)):
        run(1, nvox)
    dt = run(steps, nvox)
    rate = upd * threads * steps / dt
    what = ("the whole study" if nvox >= ncmax else
            f"the first {nvox} voxels of each colour")
    sample = (f"{steps} sweep(s) per thread over {what} ({upd} subject-voxel "
              f"updates per sweep, {dt / steps:.1f} s per step), {threads} "
              f"independent chains")
    return rate, dt / steps, sample


# ---------------------------------------------------------------- arms ---
def run_reference(args, rank, world):
    if rank != 0:
        return
    from bsglmm_gb300 import synth
    study = synth.config1(seed=1)
    threads = os.cpu_count() or 1
    # each step a bounded sample, so that the whole --steps/--warmup run
    # stays within a couple of minutes
    per_step = min(10.0, max(0.25, CPU_REFERENCE_S / max(args.steps, 1)))
    rate, sec_per_step, sample = cpu_port_rate(study, threads, args.steps,
                                               args.warmup, per_step)
    ref_gpu = reference_gpu_timing() if args.gpus >= 1 else None
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec_per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 Wishart)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "V": study.V, "N": study.N, "P": study.P,
                   "sample": sample},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line))


REFGPU_TIMEOUT_S = 240


def reference_gpu_timing() -> dict:
    """The reference's own GPU form on this GPU (its covarGPU.cu kernels,
    compiled to PTX from its source tree and driven as its launchers do,
    oracle/refgpu_run.py), in a child process under a time limit: the
    brain-sized study (2 warm-up + 10 timed sweeps) and the 20^3 study (20 +
    200).  Each entry is that run's JSON line, or why it is missing."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    if not oracle.refgpu_available():
        return {"unavailable": "oracle/_ref/covarGPU.ptx was not built (the reference "
                               "tree was not mounted where the repository was built)"}
    out = {"form": "the reference's covarGPU.cu kernels (PTX JIT-compiled for this GPU), "
                   "driven as mcmc.cpp:314-394 drives them; host Wishart",
           "timing": "CUDA events around whole sweeps (host-synchronous launchers)"}
    for name, warm, timed in (("c1", 2, 10), ("c0", 20, 200)):
        try:
            r = subprocess.run([sys.executable, str(ROOT / "oracle" / "refgpu_run.py"), name,
                                str(warm), str(timed)], capture_output=True, text=True,
                               timeout=REFGPU_TIMEOUT_S)
            last = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else ""
            out[name] = (json.loads(last) if r.returncode == 0 and last else
                         {"unavailable": f"exit {r.returncode}: {r.stderr.strip()[-300:]}"})
        except subprocess.TimeoutExpired:
            out[name] = {"unavailable": f"timed out after {REFGPU_TIMEOUT_S} s"}
    return out


def flush_l2(buf):
    buf.zero_()


def reduce_max(x: float, world: int) -> float:
    """Max over ranks (the slowest replica sets the job's time)."""
    if world > 1:
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())
    return float(x)


def chain_seed(rank: int) -> int:
    """Each replica runs an independent chain."""
    return 1 + rank


def run_ours(args, rank, world, local):
    import torch
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    study = synth.config1(seed=1)
    N, P, S, V = study.N, study.P, study.nsubtypes, study.V
    s = bsg.Sampler(local)
    ds = s.add_dataset(study.mask, study.covar, study.data, S)
    ch = s.add_chain(ds, seed=chain_seed(rank), burnin=0, thin=1)
    if args.lpv or args.threads:
        s.set_tuning(args.lpv, args.threads)
    lpv, thr = s.tuning()
    step = s.step_subjects()
    flushbuf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")

    # warm-up (also instantiates the one-sweep graph)
    for _ in range(args.warmup):
        s.run_timed(1)
    s.sync()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        s.sync()

    barrier()
    dev_ms = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush_l2(flushbuf)
            torch.cuda.synchronize()
            dev_ms.append(s.run_timed(1))
        s.sync()
        wall = time.perf_counter() - t0
    barrier()
    total_ms = reduce_max(sum(dev_ms), world)
    ms_per_step = total_ms / args.steps
    value = world * N * V * args.steps / (total_ms * 1e-3)

    # e2e through the C ABI with host buffers (Omega in, Omega + column means
    # out), wall time of each step from the host; L2 is flushed before each
    # step, outside its timed interval, as for `value`.  The step is one
    # bsg_step_host call; the same round trip as four calls (set Omega, run,
    # get Omega, get column means: what the covarGPU.cu shim does) is timed
    # beside it.
    om = s.omega(ch)
    h2d = om.nbytes
    d2h = om.nbytes + 4 * P
    out = (np.empty_like(om), np.empty(P, np.float32))
    barrier()

    def e2e_steps(one_call):
        nonlocal om
        t = 0.0
        for _ in range(args.steps):
            flush_l2(flushbuf)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if one_call:
                om = s.step_host(ch, om, 1, out=out)[0]
            else:
                s.set_omega(ch, om)
                s.run(1, sync=False)
                om = s.omega(ch)      # waits for the sweep
                _ = s.colmeans(ch)
            t += time.perf_counter() - t0
        s.sync()
        return world * N * V * args.steps / reduce_max(t, world)

    e2e = e2e_steps(True)
    e2e_calls = e2e_steps(False)

    # live per-kernel timing of the same sweep (CUDA events on the sampler's
    # stream, plain launches)
    kms, kl = s.profile(min(max(args.steps, 5), 50))
    s.sync()
    fused_avg_ms = (kms[0] + kms[1]) / (kl[0] + kl[1])
    flops_launch = N * V / 2 * fused_flops_per_update(P)
    achieved_tflops = flops_launch / (fused_avg_ms * 1e-3) / 1e12
    peak = None
    import ctypes as C
    pk = C.c_double()
    if s._L.bsg_fp32_peak(local, C.byref(pk)) == 0:
        peak = pk.value
    fused_share = (kms[0] + kms[1]) / kms[2]
    launches = s.launches_per_sweep() * args.steps
    prof = profile_inputs()

    if rank != 0:
        s.close()
        return
    s.close()
    batched = map_err = txz = None
    if world == 1 and not args.no_batched:
        batched = measure_batched(local)
    if world == 1 and not args.no_tensor_xz:
        txz = measure_tensor_xz(local, study)
    if world == 1 and not args.no_map_error:
        map_err = measure_map_error(local)
    cpu = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        crate, _, sample = cpu_port_rate(study, threads, 1, 1, CPU_BASELINE_S)
        cpu = {"value": crate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": sample}
    peaks = measured_peaks()
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 Omega/accumulators)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "V": V, "N": N, "P": P, "S": S,
                   "chains_per_gpu": 1,
                   "l2": "flushed between timed sweeps (value and e2e)",
                   "lanes_per_voxel": lpv, "block_threads": thr,
                   "subjects_per_step": step,
                   "parallelism": f"replicas x{world}"},
        "sweeps_per_s": 1e3 / ms_per_step,
        "wall_s": wall,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "form": "one bsg_step_host call per sweep (Omega in; Omega and column "
                        "means out)",
                "four_calls_value": e2e_calls},
        "gpu_launches": launches,
        "roofline": {
            "bound": "fp32", "kernel": "fused_colour_kernel",
            "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved_tflops / peak) if peak else None,
            "peak_source": "measured FP32 FMA microbenchmark (bsg_fp32_peak)",
            "traffic": prof.get("dram_bytes_per_launch"),
            "traffic_unit": "bytes per colour launch (ncu capture)",
            "traffic_source": prof["source"], "stale": prof.get("stale", True),
            "algorithmic_bytes_per_launch": sweep_bytes(N, V, P, S) / 2,
            "flops_per_update": fused_flops_per_update(P),
            "fused_avg_launch_ms": fused_avg_ms, "fused_share_of_sweep": fused_share,
            "hbm_bytes_per_sweep": sweep_bytes(N, V, P, S),
            "hbm_achieved_gbs": sweep_bytes(N, V, P, S) / (ms_per_step * 1e-3) / 1e9,
            "hbm_peak_gbs": peaks.get("hbm_gbs"),
            "issue": issue_roofline(local, N * V / 2 / (fused_avg_ms * 1e-3), prof),
        },
        "cpu_baseline": cpu,
        "clocks": clocks,
        "batched": batched,
        "map_error": map_err,
        "tensor_xz": txz,
    }
    print(json.dumps(line))


# ------------------------------------- headline: batched against plain ---
BATCH_SEGMENT = {"c4": 32, "c3": 100, "c0": 100}  # sweeps per timed segment
BATCH_MIN_MS = 1000.0  # device time of each batched measurement, at least


def _segments(smp, T: int, min_ms: float) -> float:
    """Device time per sweep of `smp` over graph segments of T sweeps
    (CUDA events on its stream), repeated until at least min_ms."""
    smp.run(T)  # instantiates the segment graphs
    total, n = 0.0, 0
    while total < min_ms or n < 2:
        total += smp.run_timed(T)
        n += 1
    smp.sync()
    return total / (n * T)


def batched_vs_plain(name: str, local: int, rhat=(None, None)) -> dict:
    """One workload of the headline metric: every chain / study in one
    context (one launch per colour and P group, P groups on parallel graph
    branches) against the plain single-chain form: each chain or study
    alone in its own context, advanced by bsg_run graph segments of the same
    length with no host synchronisation inside a segment (what a user of
    one chain runs), one after another.  Device time per sweep, with no L2
    flush inside a segment: the line states each form's working set against
    the 129 MB L2 (the 64-chain 20^3 study fits in it, so both forms run
    L2-resident there, as a chain that small does in steady state).  `rhat`
    = (burn-in, sweeps) of the c4 R-hat, None for the defaults."""
    import bsglmm_gb300 as bsg
    studies, nchains = batched_workload(name)
    rh_burnin = RHAT_BURNIN if rhat[0] is None else rhat[0]
    rh_sweeps = RHAT_SWEEPS if rhat[1] is None else rhat[1]
    T = BATCH_SEGMENT[name]
    upd = sum(st.N * st.V * c for st, c in zip(studies, nchains))
    # bytes a sweep touches per study: outcome bits (shared by its chains),
    # and per chain the coefficients and the FP64 running sums of kept sweeps
    ws = [st.N * st.V / 8 + c * (st.P * st.V * 4 + (2 * st.P + st.nsubtypes) * st.V * 8)
          for st, c in zip(studies, nchains)]
    with bsg.Sampler(local) as b:
        for k, (st, nc) in enumerate(zip(studies, nchains)):
            ds = b.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            for c in range(nc):
                b.add_chain(ds, seed=1000 * k + c + 1)
        with Clocks(local) as clk:
            t_b = _segments(b, T, BATCH_MIN_MS)
        launches = b.launches_per_sweep()
        # the 16 chains of one study: Gelman-Rubin R-hat of every coefficient
        # map entry across them (the convergence measure reported for it)
        rh = (cross_chain_rhat(b, sum(nchains), rh_burnin, rh_sweeps)
              if name == "c4" else None)
    # plain: a lone chain of each study; identical chains of one study cost
    # the same, so a study's nc chains take nc times its lone chain's time
    t_p = 0.0
    for k, (st, nc) in enumerate(zip(studies, nchains)):
        with bsg.Sampler(local) as p:
            ds = p.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
            p.add_chain(ds, seed=1000 * k + 1)
            t_p += nc * _segments(p, T, 200.0 / len(studies))
    return {"workload": BATCHED[name], "chains": sum(nchains), "studies": len(studies),
            "updates_per_sweep": upd, "segment_sweeps": T,
            "batched": {"value": upd / (t_b * 1e-3), "ms_per_sweep": t_b,
                        "launches_per_sweep": launches},
            "plain": {"value": upd / (t_p * 1e-3), "ms_per_sweep": t_p,
                      "form": "each chain alone in its own context, bsg_run segments"},
            "batched_over_plain": t_p / t_b, "unit": UNIT, "timing": "device, CUDA events",
            "working_set_mb": {"batched": sum(ws) / 1e6, "plain_largest": max(ws) / 1e6,
                               "l2_mb": L2_MB},
            "clocks": clk.summary(), "rhat": rh}


def measure_batched(local: int) -> dict:
    out = {k: batched_vs_plain(k, local) for k in ("c4", "c3", "c0")}
    out["meets_3x"] = {k: out[k]["batched_over_plain"] >= 3.0 for k in ("c4", "c3", "c0")}
    return out


def measure_tensor_xz(local: int, brain) -> dict:
    """The A/B of the probit colour kernel's X'Z contraction: f32x2 FMAs
    (SIMT, the default) against the tensor cores (BF16x3 split product,
    bsg_set_tensor_xz), on the brain-sized study (N = 1000, P = 5) and the
    precision study (N = 2000, P = 8): device time per colour launch
    (CUDA events around plain launches) and per sweep (64-sweep segments,
    at least 0.5 s), same chain and variates."""
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    out = {"form": "mma.sync m16n8k16 BF16x3 (x_hi z_hi + x_hi z_lo + x_lo z_hi), "
                   "FP32 accumulation, one warp per 32 voxels"}
    for name, st in (("c1", brain), ("c2", synth.config2())):
        res = {"N": st.N, "P": st.P, "V": st.V}
        for mode, tc in (("simt", False), ("tensor", True)):
            with bsg.Sampler(local) as s:
                ds = s.add_dataset(st.mask, st.covar, st.data, st.nsubtypes)
                s.add_chain(ds, seed=7)
                s.set_tensor_xz(tc)
                s.run(2)
                kms, kl = s.profile(10)
                t = _segments(s, 64, 500.0)
            res[mode] = {"colour_ms": [kms[0] / kl[0], kms[1] / kl[1]], "ms_per_sweep": t,
                         "value": st.N * st.V / (t * 1e-3)}
        res["tensor_over_simt"] = res["simt"]["ms_per_sweep"] / res["tensor"]["ms_per_sweep"]
        out[name] = res
    return out


MAP_ERROR_FILE = ROOT / "tests" / "golden" / "map_error_fp64.json"


def measure_map_error(local: int) -> dict:
    """The FP32 maps' error against the FP64 GPU chain, live on the
    CPU-runnable study (20^3 sphere, N = 50, P = 3: 1000 burn-in + 20 x 100
    kept sweeps, batch-means MCSE), plus the committed results of the
    brain-sized studies (tests/golden/map_error_fp64.json)."""
    from bsglmm_gb300 import precision, synth
    live = precision.map_error_vs_fp64(synth.config0(0), seed=1, burnin=1000,
                                       batches=20, batch=100, device=local)
    out = {"c0_live": live}
    if MAP_ERROR_FILE.exists():
        out["committed"] = json.loads(MAP_ERROR_FILE.read_text())
        out["committed_source"] = str(MAP_ERROR_FILE.relative_to(ROOT))
    return out


# ------------------------------------------------- batched workloads ---
BATCHED = {
    "c0": "64 chains of the 20^3 sphere study (N=50, P=3) in one context",
    "c3": "64 replicate studies (cube side 32-64, N 40-400, P 2-6) in one context",
    "c4": "16 chains on a 182x218x182 ellipsoid (1.5M voxels, N=500, P=6)",
}


def batched_workload(name):
    from bsglmm_gb300 import synth
    if name == "c0":
        return [synth.config0(0)], [64]
    if name == "c3":
        sts = synth.config3()
        return sts, [1] * len(sts)
    if name == "c4":
        return [synth.config4()], [16]
    raise ValueError(name)


RHAT_BURNIN, RHAT_SWEEPS = 300, 200  # sweeps behind the c4 R-hat figure


def cross_chain_rhat(s, nchains: int, burnin: int, sweeps: int) -> dict:
    """Gelman-Rubin R-hat of every coefficient map entry across the chains
    of one study, from each chain's posterior mean and variance over
    `sweeps` sweeps after `burnin` more (the accumulators are reset in
    between)."""
    s.run(burnin)
    for c in range(nchains):
        s.reset_accumulators(c)
    s.run(sweeps)
    means, vars_ = [], []
    for c in range(nchains):
        m, v, _, n = s.posterior(c)
        means.append(m)
        vars_.append(v)
    m = np.stack(means)
    w = np.mean(np.stack(vars_), axis=0)
    b = n * np.var(m, axis=0, ddof=1)
    var_plus = (n - 1) / n * w + b / n
    r = np.sqrt(var_plus / w).ravel()
    return {"burnin": burnin, "sweeps": sweeps, "chains": nchains, "entries": int(r.size),
            "median": float(np.median(r)), "p99": float(np.percentile(r, 99)),
            "max": float(r.max())}


def run_batched(args, rank, world, local):
    """One batched workload on its own line (`--workload c0|c3|c4`): every
    chain / study in one context against the plain single-chain form, both
    timed as in the default line's `batched` object (batched_vs_plain: graph
    segments, device time); for c4 the cross-chain R-hat after
    `--rhat-burnin` + `--rhat-sweeps` sweeps per chain."""
    import torch
    torch.cuda.set_device(local)
    r = batched_vs_plain(args.workload, local, rhat=(args.rhat_burnin, args.rhat_sweeps))
    b = r["batched"]
    line = {
        "metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": 1,
        "steps": None, "warmup": None, "ms_per_step": b["ms_per_sweep"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 Omega/accumulators)", "data": "synthetic",
        "config": {"workload": r["workload"], "studies": r["studies"],
                   "chains": r["chains"], "updates_per_sweep": r["updates_per_sweep"],
                   "segment_sweeps": r["segment_sweeps"],
                   "l2": "no flush inside a segment; working set %.0f MB batched, %.0f MB for "
                         "the largest plain study, against a %d MB L2"
                         % (r["working_set_mb"]["batched"], r["working_set_mb"]["plain_largest"],
                            L2_MB),
                   "timing": r["timing"]},
        "sweeps_per_s": 1e3 / b["ms_per_sweep"], "gpu_launches_per_sweep": b["launches_per_sweep"],
        "plain": r["plain"], "batched_over_plain": r["batched_over_plain"],
        "rhat": r["rhat"], "clocks": r["clocks"],
    }
    if rank == 0:
        print(json.dumps(line))


def run_dic(args, rank, world, local):
    """The DIC / Qhat predictive pass on the brain-sized study with two
    indicator group columns (the two arms of the +-0.5 group column): device
    time per kept sweep with the pass on against off (every sweep kept, L2
    flushed before each sweep), and the on-demand pass."""
    import torch
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    torch.cuda.set_device(local)
    study = synth.config1(seed=1)
    covar = study.covar.copy()
    arm = covar[1] > 0
    covar[0], covar[1] = ~arm, arm
    N, P, V, S = study.N, study.P, study.V, 2
    flushbuf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    s = bsg.Sampler(local)
    ds = s.add_dataset(study.mask, covar, study.data, S)
    ch = s.add_chain(ds, seed=chain_seed(rank), burnin=0, thin=1)

    def timed(steps):
        ms = []
        for _ in range(steps):
            flush_l2(flushbuf)
            torch.cuda.synchronize()
            ms.append(s.run_timed(1))
        s.sync()
        return float(np.median(ms))

    for _ in range(args.warmup):
        s.run_timed(1)
    with Clocks(local) as clk:
        off = timed(args.steps)
        s.set_predictive(ch, True)
        for _ in range(args.warmup):
            s.run_timed(1)
        on = timed(args.steps)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.predict(ch)
        call = (time.perf_counter() - t0) / args.steps
    q, ed, npred = s.predictive(ch)
    dic = s.dic(ch)
    s.close()
    evals = N * V * S
    added = on - off
    line = {
        "metric": "subject-voxel-group log predictive evaluations/s (DIC/Qhat pass)",
        "value": evals / (added * 1e-3), "unit": "evaluations/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": added,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 sums)", "data": "synthetic",
        "config": {"workload": "brain-sized study, 91x109x91 grid, N=1000, P=5, "
                               "two indicator group columns (S=2)",
                   "V": V, "N": N, "P": P, "S": S,
                   "l2": "flushed between timed sweeps", "timing": "device, median"},
        "sweep_ms_off": off, "sweep_ms_on_every_sweep_kept": on,
        "predict_call_ms": call * 1e3, "gpu_launches_per_kept_sweep": 2,
        "npred": npred, "dic": dic, "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


VARIANTS = {
    "logit": "brain-sized study with the logistic link (t_8 scale mixture, "
             "logit_factor 0.634): 91x109x91 grid, N=1000, P=5",
    "t": "brain-sized study with the t_3 link (scale mixture of normals): "
         "91x109x91 grid, N=1000, P=5",
    "wm": "brain-sized study with a voxelwise WM map and the beta_WM update: "
          "91x109x91 grid, N=1000, P=5",
    "c2": "precision form: the brain-sized mask with N=2000, P=8 (FP32 sweep, "
          "FP64 Omega pair sums, Cholesky and accumulators), 1 chain",
}


def run_variant(args, rank, world, local):
    """One sweep of the brain-sized study on a model variant (the logistic
    link, or the beta_WM update), device time per sweep with L2 flushed,
    against the plain probit sweep of the same study in the same process."""
    import torch
    import bsglmm_gb300 as bsg
    from bsglmm_gb300 import synth
    torch.cuda.set_device(local)
    study = synth.config2() if args.workload == "c2" else synth.config1(seed=1)
    N, P, S, V = study.N, study.P, study.nsubtypes, study.V
    flushbuf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    wm = (np.random.default_rng(7).random(V).astype(np.float32)
          if args.workload == "wm" else None)

    def timed(setup):
        with bsg.Sampler(local) as s:
            ds = s.add_dataset(study.mask, study.covar, study.data, S, wm)
            ch = s.add_chain(ds, seed=chain_seed(rank), burnin=0, thin=1)
            if args.tensor_xz:
                s.set_tensor_xz(True)
            setup(s, ch)
            for _ in range(args.warmup):
                s.run_timed(1)
            s.sync()
            ms = []
            for _ in range(args.steps):
                flush_l2(flushbuf)
                torch.cuda.synchronize()
                ms.append(s.run_timed(1))
            s.sync()
            prof, nl = s.profile(min(args.steps, 20))
            return float(np.median(ms)), prof[0] / nl[0], prof[1] / nl[1], s.launches_per_sweep()

    with Clocks(local) as clk:
        base = timed(lambda s, ch: None)
        if args.workload in ("logit", "t"):
            link = "logistic" if args.workload == "logit" else "t"
            var = timed(lambda s, ch: s.set_model(ch, link))
        elif args.workload == "wm":
            var = timed(lambda s, ch: s.set_wm_update(ch, True))
        else:  # c2: the plain sweep of its own study
            var = base
    line = {
        "metric": "subject-voxel updates/s of one sweep (model variant)",
        "value": N * V / (var[0] * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": var[0],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 Omega/accumulators)", "data": "synthetic",
        "config": {"workload": VARIANTS[args.workload], "V": V, "N": N, "P": P, "S": S,
                   "l2": "flushed between timed sweeps", "timing": "device, median"},
        "colour_kernel_ms": [var[1], var[2]], "gpu_launches_per_sweep": var[3],
        "probit_same_study": {"ms_per_step": base[0], "value": N * V / (base[0] * 1e-3),
                              "colour_kernel_ms": [base[1], base[2]]},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--lpv", type=int, default=0)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-map-error", action="store_true")
    ap.add_argument("--no-tensor-xz", action="store_true")
    ap.add_argument("--tensor-xz", action="store_true",
                    help="model-variant workloads: X'Z on the tensor cores")
    ap.add_argument("--rhat-burnin", type=int, default=None,
                    help="--workload c4: burn-in sweeps per chain before the R-hat")
    ap.add_argument("--rhat-sweeps", type=int, default=None,
                    help="--workload c4: sweeps per chain behind the R-hat")
    ap.add_argument("--workload", default="brain",
                    choices=["brain", "dic"] + sorted(VARIANTS) + sorted(BATCHED))
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.workload == "dic" and args.impl == "ours":
        run_dic(args, rank, world, local)
        return
    if args.workload in VARIANTS and args.impl == "ours":
        run_variant(args, rank, world, local)
        return
    if args.workload != "brain" and args.impl == "ours":
        run_batched(args, rank, world, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
