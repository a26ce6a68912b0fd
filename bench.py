"""Benchmark: BP message updates/s on the 32x32 periodic PEPS norm network, D=8, d=2.

One *step* is one belief-propagation solve of that network: message reset to the
normalised identity, SWEEPS parallel-schedule sweeps (2E = 4096 message updates
each), and the Bethe log-norm.  ``value`` counts message updates per second of device
time of the sweeps with the site tensors resident in HBM; ``e2e`` is the same metric
through the C ABI with pinned host buffers (tensor upload, message upload, solve, log-norm,
message download inside the timed region for every step) as a serving loop runs it:
``itn_bp_solve_submit`` / ``itn_bp_solve_wait`` on E2E_CONTEXTS contexts, so that later steps'
uploads overlap earlier steps' solves.  ``e2e_single_call`` is the synchronous one-call form
``itn_bp_solve`` (one host wait per step) and ``e2e_separate_calls`` the same step as five
calls that each wait for their result.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--impl reference`` times the CPU restatement of the reference algorithm (the oracle,
plain FP32 arithmetic, OpenMP over the host cores) on the same workload.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "itensornetworksnext.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

LX = LY = 32
BOND = 8
PHYS = 2
SWEEPS = 30
SPLIT_SWEEPS = 3
SEED = 32
METRIC = "BP message updates/s (32x32, D=8) mixed vs plain FP32; grad time @1e-6 err"
# FP32 FMA rate of a GB300 at its maximum clock: 152 SMs x 128 lanes x 2 flops x 2.07 GHz
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
UNIT = "message updates/s"
# solves in flight in the serving form of the end-to-end measurement (one context each)
E2E_CONTEXTS = 8


def workload():
    from itn_gb300 import graphs as G
    g = G.square_lattice(LX, LY, BOND, periodic=True, phys=PHYS)
    rng = np.random.default_rng(SEED)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    return g, t


def flops_per_sweep(g) -> float:
    """Algorithmic flops of one sweep: sum over directed slots of 2 d P_u S_u, where
    P_u is the product and S_u the sum of the bond dims of the source vertex."""
    tot = 0.0
    for u in range(g.nv):
        legs = g.legs(u)
        P = float(np.prod(legs))
        S = float(np.sum(legs))
        tot += len(legs) * 2.0 * g.phys[u] * P * S
    return tot


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: let its first sample arrive before the
            # timed region begins
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def hbm_roofline(g, mode, sweep_ms, peaks):
    """Algorithmic bytes of one sweep against the measured copy bandwidth: every site tensor
    read once in the operand precision (BF16 2 B, TF32/FP32 4 B per entry) and, per message
    update, its z-1 incoming messages read and the result written (FP32)."""
    esz = 2 if mode == "bf16" else 4
    tensor_bytes = esz * float(g.toff[-1])
    msg_bytes = 0.0
    for u in range(g.nv):
        z = int(g.off[u + 1] - g.off[u])
        for s in range(int(g.off[u]), int(g.off[u + 1])):
            msg_bytes += 4.0 * float(g.moff[s + 1] - g.moff[s]) * z  # z-1 reads + 1 write
    total = tensor_bytes + msg_bytes
    gbs = total / (sweep_ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"algorithmic_bytes_per_sweep": total, "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak,
            "note": "within a solve the operands stay L2-resident; DRAM traffic per sweep is in traffic"}


def ncu_traffic():
    """Per-sweep DRAM bytes of the sweep kernels from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "bp_sweep_32x32_D8.md")
    if not os.path.exists(p):
        return None
    best = {}
    for ln in open(p):
        if ln.startswith("traffic_bytes_per_sweep"):
            k, v = ln.split(":", 1)
            try:
                best[k.strip()] = float(v.strip().split()[0])
            except ValueError:
                pass
    return best or None


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def barrier(pg, device):
    if pg is not None:
        import torch
        t = torch.zeros(1, device=f"cuda:{device}")
        pg.all_reduce(t)
        torch.cuda.synchronize(device)


def max_over_ranks(pg, x, device):
    """Replica timing: the slowest rank defines the job time (itn_gb300.distributed)."""
    if pg is None:
        return x
    from itn_gb300 import distributed as D
    return D.max_over_ranks(x, device=f"cuda:{device}")


def flush_l2(device):
    import torch
    buf = getattr(flush_l2, "buf", None)
    if buf is None:
        buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{device}")
        flush_l2.buf = buf
    buf.zero_()
    torch.cuda.synchronize(device)


def host_cpu():
    """Model name of the host cores (lscpu), else the machine type."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def cpu_baseline(g, t, seconds=12.0):
    """Oracle (CPU restatement of the reference algorithm), FP32 parallel sweeps with
    OpenMP over all host threads, on the same 32x32 D=8 network; a bounded sample."""
    from oracle import oracle as O
    from itn_gb300 import graphs as G
    t32 = t.astype(np.float32)
    m = G.identity_messages(g, np.float32)
    threads = O.max_threads()
    O.bp_sweeps(g, t32, m, 1, nthreads=threads)  # warm
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n == 0:
        O.bp_sweeps(g, t32, m, 1, nthreads=threads)
        n += 1
    dt = time.perf_counter() - t0
    # the same sweeps on one host core (bounded sample)
    n1, t1 = 0, time.perf_counter()
    while time.perf_counter() - t1 < seconds / 3 or n1 == 0:
        O.bp_sweeps(g, t32, m, 1, nthreads=1)
        n1 += 1
    dt1 = time.perf_counter() - t1
    return {"value": n * g.nslots / dt, "unit": UNIT, "cores": threads, "kind": "port", "cpu": host_cpu(),
            "sample": f"{n} parallel FP32 sweeps of the 32x32 D=8 norm network ({n * g.nslots} updates, {dt:.1f} s)",
            "one_core": {"value": n1 * g.nslots / dt1, "unit": UNIT,
                         "sample": f"{n1} sweeps on 1 thread ({dt1:.1f} s)"}}


def run_reference(args):
    rank, world, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return 0
    g, t = workload()
    from oracle import oracle as O
    from itn_gb300 import graphs as G
    t32 = t.astype(np.float32)
    threads = O.max_threads()
    sweeps_per_step = 2
    m = G.identity_messages(g, np.float32)
    for _ in range(args.warmup):
        O.bp_sweeps(g, t32, m, 1, nthreads=threads)
    times = []
    for _ in range(args.steps):
        m = G.identity_messages(g, np.float32)
        t0 = time.perf_counter()
        O.bp_sweeps(g, t32, m, sweeps_per_step, nthreads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    v = args.steps * sweeps_per_step * g.nslots / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded N(0,1)/sqrt(d D^4) PEPS)",
            "config": {"workload": f"peps {LX}x{LY} periodic norm network D={BOND} d={PHYS}, parallel schedule",
                       "step": f"{sweeps_per_step} sweeps (bounded CPU sample of the GPU step's {SWEEPS})"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "cpu": host_cpu(),
                             "sample": f"{args.steps} steps x {sweeps_per_step} FP32 sweeps, OpenMP"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    rank, world, local, pg = dist_setup(args.gpus)
    import torch
    device = local
    torch.cuda.set_device(device)
    from itn_gb300 import BPEngine
    g, t = workload()
    t32 = np.ascontiguousarray(t.astype(np.float32))
    m0 = np.ascontiguousarray(G_identity(g))
    upd_per_step = SWEEPS * g.nslots
    fps = flops_per_sweep(g)

    eng = BPEngine(g, device=device)
    eng.set_tensors(t32)
    mode = args.precision
    run_kw = dict(maxiter=SWEEPS)
    if mode != "native":
        run_kw.update(precision=mode, split_sweeps=SPLIT_SWEEPS)

    def device_step():
        eng.init_messages("identity_normalized")
        r = eng.run(**run_kw)
        logz = eng.bethe_free_energy()
        return r, logz

    # plain FP32 CUDA-core sweeps (the comparison point of the metric)
    def fp32_step():
        eng.init_messages("identity_normalized")
        return eng.run(maxiter=SWEEPS)

    for _ in range(max(args.warmup, 3)):
        device_step()
        fp32_step()
    barrier(pg, device)
    torch.cuda.synchronize(device)

    dev_ms, launches, fp32_ms = [], 0, []
    wall0 = time.perf_counter()
    with ClockSampler(device) as clk:
        for _ in range(args.steps):
            flush_l2(device)
            r, logz = device_step()
            dev_ms.append(r.device_ms)
            # + message init + the log-norm's kernels (vertex scalars, edge scalars, FP64
            # logs with per-block shares, the single-network sum)
            launches += r.kernel_launches + 1 + 4
        for _ in range(args.steps):
            flush_l2(device)
            fp32_ms.append(fp32_step().device_ms)
    torch.cuda.synchronize(device)
    barrier(pg, device)
    wall = time.perf_counter() - wall0
    ms_step = max_over_ranks(pg, sum(dev_ms) / len(dev_ms), device)
    ms_fp32 = max_over_ranks(pg, sum(fp32_ms) / len(fp32_ms), device)
    value = world * upd_per_step / (ms_step * 1e-3)
    fp32_value = world * upd_per_step / (ms_fp32 * 1e-3)

    # end to end through the C ABI with host buffers (pinned, as a serving caller keeps them)
    m_host = torch.empty(int(g.moff[-1]), dtype=torch.float32, pin_memory=True).numpy()
    t_pin = torch.empty(t32.size, dtype=torch.float32, pin_memory=True).numpy()
    t_pin[:] = t32
    m0_pin = torch.empty(m0.size, dtype=torch.float32, pin_memory=True).numpy()
    m0_pin[:] = m0
    # the one-call API (itn_bp_solve: upload, solve, log-norm, download, one host wait) ...
    e2e_times = []
    for _ in range(args.steps):
        flush_l2(device)
        t0 = time.perf_counter()
        eng.solve(t_pin, m0_pin, messages_out=m_host, **run_kw)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(pg, sum(e2e_times) / len(e2e_times), device)
    e2e_value = world * upd_per_step / e2e_s
    # ... and the serving form of the same call: E2E_CONTEXTS contexts, each step submitted with
    # itn_bp_solve_submit and collected with itn_bp_solve_wait E2E_CONTEXTS - 1 steps later, so
    # that later steps' uploads overlap earlier steps' solves; every step still copies its own
    # inputs in and its messages and log-norm out.  The contexts' buffers (~800 MB) exceed L2.
    engs = [eng] + [BPEngine(g, device=device) for _ in range(E2E_CONTEXTS - 1)]
    m_out = [m_host] + [torch.empty(int(g.moff[-1]), dtype=torch.float32, pin_memory=True).numpy()
                        for _ in range(E2E_CONTEXTS - 1)]
    for k in range(2 * E2E_CONTEXTS):  # warm-up of the other contexts (graph capture, operand image)
        engs[k % E2E_CONTEXTS].solve(t_pin, m0_pin, messages_out=m_out[k % E2E_CONTEXTS], **run_kw)
    barrier(pg, device)
    n_pipe = max(args.steps, 4 * E2E_CONTEXTS)
    t0 = time.perf_counter()
    for k in range(n_pipe):
        engs[k % E2E_CONTEXTS].solve_submit(t_pin, m0_pin, messages_out=m_out[k % E2E_CONTEXTS], **run_kw)
        if k >= E2E_CONTEXTS - 1:
            engs[(k - E2E_CONTEXTS + 1) % E2E_CONTEXTS].solve_wait()
    for k in range(n_pipe - E2E_CONTEXTS + 1, n_pipe):
        engs[k % E2E_CONTEXTS].solve_wait()
    pipe_s = max_over_ranks(pg, (time.perf_counter() - t0) / n_pipe, device)
    pipe_value = world * upd_per_step / pipe_s
    for e_ in engs[1:]:
        e_.close()
    # ... and the same step as five separate calls, each waiting for its own result
    sep_times = []
    for _ in range(args.steps):
        flush_l2(device)
        t0 = time.perf_counter()
        eng.set_tensors(t_pin)
        eng.set_messages(m0_pin)
        eng.run(**run_kw)
        eng.bethe_free_energy()
        eng.messages(m_host)
        sep_times.append(time.perf_counter() - t0)
    sep_s = max_over_ranks(pg, sum(sep_times) / len(sep_times), device)
    h2d = t_pin.nbytes + m0_pin.nbytes
    d2h = m_host.nbytes + 16 + 4  # messages, the (re, im) log-norm total and its flags

    # accuracy of this run against an FP64 GPU solve of the same network: total and
    # per-site (log Z_v) log-norm errors
    err = None
    site_err = None
    if rank == 0:
        eng.init_messages("identity_normalized")
        eng.run(**run_kw)
        lzv = eng.logscalars()["logzv"][:, 0]
        ref = BPEngine(g, device=device)
        ref.set_tensors(t)
        ref.init_messages("identity_normalized")
        ref.run(maxiter=SWEEPS)
        lz64 = ref.bethe_free_energy()
        lzv64 = ref.logscalars()["logzv"][:, 0]
        ref.close()
        err = abs(logz - lz64) / abs(lz64)
        site_err = float(np.max(np.abs(lzv - lzv64)))

    if rank != 0:
        # the batched workload shards across all ranks (the same call as rank 0's below)
        if args.extra:
            bench_batched(device, pg, rank, world)
        eng.close()
        return 0
    peaks, peak_kind = measured_peaks()
    sweep_ms = ms_step / SWEEPS
    achieved = fps / (sweep_ms * 1e-3) / 1e12
    peak = peaks["bf16_tflops"]
    traffic = ncu_traffic()
    tkey = "traffic_bytes_per_sweep_" + mode
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if mode == "native" else ("tf32 hi/lo" if mode == "tf32x3" else f"{mode}+split"),
        "data": "synthetic (seeded N(0,1)/sqrt(d D^4) PEPS)",
        "config": {"workload": f"peps {LX}x{LY} periodic norm network D={BOND} d={PHYS}, "
                               f"{SWEEPS} parallel sweeps per step (device-timed solve; the Bethe "
                               f"log-norm follows each step and is inside the e2e region)",
                   "precision": mode, "split_sweeps": SPLIT_SWEEPS if mode != "native" else 0,
                   "updates_per_step": upd_per_step,
                   "l2": "flushed between steps (256 MB write); the 33.5 MB of FP32 site tensors stay L2-resident within a step"},
        "fp32_plain": {"value": fp32_value, "ms_per_step": ms_fp32,
                       "speedup_of_value": value / fp32_value,
                       "kernel": "sweep_d8_kernel (FP32 CUDA cores, register-blocked, one CTA per half vertex)",
                       "achieved_tflops_alg": fps / (ms_fp32 / SWEEPS * 1e-3) / 1e12,
                       "fp32_peak_tflops": FP32_PEAK_TFLOPS,
                       "frac_of_fp32_peak": fps / (ms_fp32 / SWEEPS * 1e-3) / 1e12 / FP32_PEAK_TFLOPS},
        "logz_rel_err_vs_fp64": err,
        "logzv_max_abs_err_vs_fp64": site_err,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_source": f"bf16_tflops ({peak_kind})",
                     "traffic": (traffic or {}).get(tkey),
                     "algorithmic_flops_per_sweep": fps,
                     "sweep_ms": sweep_ms,
                     # the memory side of the same sweep: site tensors once (operand precision)
                     # plus z-1 message reads and one write per update (FP32)
                     "hbm": hbm_roofline(g, mode, sweep_ms, peaks),
                     "kernels": "one persistent launch for the BF16 sweeps, one for the split sweeps"
                                if mode != "native" else "one launch per sweep"},
        "cpu_baseline": cpu_baseline(g, t) if (args.cpu_baseline and world == 1) else None,
        "e2e_separate_calls": {"value": world * upd_per_step / sep_s, "unit": UNIT,
                               "calls": "set_tensors, set_messages, run, bethe_free_energy, messages"},
        "e2e_single_call": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_s * 1e3,
                            "call": "itn_bp_solve, one context, one host wait per step"},
        "e2e": {"value": pipe_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": pipe_s * 1e3,
                "call": f"itn_bp_solve_submit / itn_bp_solve_wait on {E2E_CONTEXTS} contexts (a serving loop "
                        f"with {E2E_CONTEXTS} solves in flight): every step uploads its tensors and messages "
                        f"from pinned host memory and downloads its messages and log-norm; later steps' "
                        f"uploads overlap earlier steps' solves", "steps": n_pipe},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s": wall,
    }
    if args.extra:
        # the batched workload shards across ranks (every rank takes part); the rest runs
        # on rank 0 of a one-GPU run
        batched = bench_batched(device, pg, rank, world)
        if world == 1:
            if mode == "bf16":
                line["tf32_mixed"] = bench_tf32(device, g, t, t32, args.steps)
                line["tf32x3"] = bench_tf32(device, g, t, t32, args.steps, precision="tf32x3")
            line["grad"] = bench_grad(device)
            line["bp_16x16_D4"] = bench_16x16(device)
            line["apply_layer_16x16_D4"] = bench_apply_layer(device)
        line["batched"] = batched
    print(json.dumps(line))
    eng.close()
    return 0


def bench_tf32(device, g, t, t32, steps, precision="tf32"):
    """The same 32x32 D=8 solve with TF32 tensor-core sweeps (27 TF32 + 3 split; or every
    sweep with TF32 hi/lo operands for ``tf32x3``), device-timed like the headline value,
    and its log-norm errors (total, max per site) against an FP64 GPU solve."""
    from itn_gb300 import BPEngine
    e = BPEngine(g, device=device)
    e.set_tensors(t32)
    kw = dict(maxiter=SWEEPS, precision=precision, split_sweeps=SPLIT_SWEEPS)
    for _ in range(3):
        e.init_messages()
        e.run(**kw)
    ms = []
    for _ in range(steps):
        flush_l2(device)
        e.init_messages()
        ms.append(e.run(**kw).device_ms)
    lz = e.bethe_free_energy()
    lzv = e.logscalars()["logzv"][:, 0]
    e.close()
    f = BPEngine(g, device=device)
    f.set_tensors(t)
    f.init_messages()
    f.run(maxiter=SWEEPS)
    lz64 = f.bethe_free_energy()
    lzv64 = f.logscalars()["logzv"][:, 0]
    f.close()
    best = sum(ms) / len(ms)
    what = ("every sweep with TF32 hi/lo operands (3 TF32 products each)" if precision == "tf32x3"
            else "TF32 operands, the last 3 sweeps BF16 hi/lo")
    return {"workload": f"the headline network and sweeps, {what}", "value": SWEEPS * g.nslots / (best * 1e-3),
            "unit": UNIT, "ms_per_step": best, "logz_rel_err_vs_fp64": abs(lz - lz64) / abs(lz64),
            "logzv_max_abs_err_vs_fp64": float(np.max(np.abs(lzv - lzv64)))}


def bench_grad(device):
    """12x12 open PEPS, d=2, D=6, FP32 BP to convergence + implicit (adjoint) gradient of
    the Bethe log-norm; error against central FD (step 1e-4, FP64 solves) on 32 random unit
    directions, reported as |g.d - fd| over the vector of FD derivatives.  Times: the minimum
    over three repetitions after a warm-up one."""
    from itn_gb300 import BPEngine
    from itn_gb300 import graphs as G
    g = G.square_lattice(12, 12, 6, periodic=False, phys=2)
    rng = np.random.default_rng(12)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    e = BPEngine(g, device=device)
    e.set_tensors(t.astype(np.float32))
    times, dev_ms = [], []
    for rep in range(4):  # first repetition warms up (graph capture, autotune)
        t0 = time.perf_counter()
        e.init_messages()
        r = e.run(maxiter=500, tol=1e-12)
        grad, info = e.grad(adjoint=True, tol=1e-6)
        times.append(time.perf_counter() - t0)
        dev_ms.append(info["device_ms"])
    e.close()
    f = BPEngine(g, device=device)

    def logz(x):
        f.set_tensors(x)
        f.init_messages()
        f.run(maxiter=2000, tol=1e-14)
        return f.bethe_free_energy()
    gd, fds = [], []
    h = 1e-4
    for _ in range(32):
        d = rng.standard_normal(t.size)
        d /= np.linalg.norm(d)
        fds.append((logz(t + h * d) - logz(t - h * d)) / (2 * h))
        gd.append(float(grad.astype(np.float64) @ d))
    f.close()
    gd, fds = np.array(gd), np.array(fds)
    return {"workload": "peps 12x12 open D=6 d=2, fp32 messages/gradient, fp64 log-scalars",
            "bp_sweeps": r.iterations, "adjoint_iterations": info["adjoint_iterations"],
            "grad_device_ms": min(dev_ms[1:]), "solve_plus_grad_wall_ms": 1e3 * min(times[1:]),
            "fd_rel_err": float(np.linalg.norm(gd - fds) / np.linalg.norm(fds)), "fd_directions": 32,
            "fd_step": h}


def bench_batched(device, pg=None, rank=0, world=1, steps=3):
    """256 independent random 3-regular networks, N ~ U{16..256} (even), per-edge bond
    dims from {2,3,4,6,8}, complex64 N(0,1) entries; 30 parallel sweeps, every edge of every
    network in one persistent launch per sweep, the solve captured as a CUDA graph.  With
    several ranks the networks are sharded by vertex count (no collective in the solve):
    each rank solves its share, the time is the maximum over ranks and the value all ranks'
    updates over that time; the per-network log-norms are gathered at the end."""
    from itn_gb300 import BPEngine
    from itn_gb300 import distributed as D
    from itn_gb300 import graphs as G
    rng = np.random.default_rng(256)
    nets = []
    for _ in range(256):
        n = int(rng.integers(8, 129)) * 2
        edges = G.random_regular_edges(n, 3, rng)
        bonds = rng.choice([2, 3, 4, 6, 8], size=len(edges))
        nets.append(G.from_edges(n, edges, bonds, phys=2))
    g_all = G.batched(nets)
    t_all = G.random_tensors(g_all, rng, np.complex64)
    vstart = np.concatenate([[0], np.cumsum([g.nv for g in nets])])
    lo, hi, g = D.shard_batch(nets, rank, world)
    t = t_all[g_all.toff[vstart[lo]]:g_all.toff[vstart[hi]]]
    e = BPEngine(g, device=device)
    e.set_tensors(t)
    ms = []
    for rep in range(steps + 1):
        e.init_messages()
        r = e.run(maxiter=30)
        if rep:
            ms.append(r.device_ms)
    logz = e.bethe_free_energy(None)
    e.close()
    local = {lo + i: v for i, v in enumerate(logz if isinstance(logz, list) else [logz])}
    gathered = D.gather_logz(local, len(nets), device=f"cuda:{device}" if pg is not None else "cpu")
    best = max_over_ranks(pg, min(ms), device)
    upd = 30 * g_all.nslots
    flops = 30 * sum(4 * len(g_all.legs(u)) * 2.0 * 2 * np.prod(g_all.legs(u)) * np.sum(g_all.legs(u))
                     for u in range(g_all.nv))
    return {"workload": "256 random 3-regular norm networks, N in [16,256], D_e in {2,3,4,6,8}, c64, 30 sweeps",
            "vertices": g_all.nv, "updates_per_solve": upd, "value": upd / (best * 1e-3),
            "unit": "message updates/s", "ms_per_solve": best, "ranks": world,
            "sharding": "networks split by vertex count across ranks, log-norms gathered" if world > 1 else None,
            "achieved_tflops_complex_alg": flops / (best * 1e-3) / 1e12,
            "logz_finite": bool(np.all(np.isfinite(gathered)))}


def run_case(name, device=0):
    """Small runs of one kernel family each, for ncu captures (profiles/*.md give the
    commands): d8 = FP32 32x32 D=8 sweeps (sweep_d8_kernel); mixed = the 30-sweep mixed solve
    (bp_tc_kernel, tc_image_kernel); grad = the 12x12 D=6 FP32 gradient (bp2_dual_kernel, the
    adjoint update fused into it); gate = one layer of 128 gates (gate_kernel); contract = 2048^3 float32
    contractions in the three precisions (gemm_cc_kernel, gemm_tc_kernel); batched = the
    256-network complex64 batch (sweep_z3_kernel); exact6 = the exact FP64 contraction of the
    6x6 D=3 norm network (permute_kernel, gemm_cc_kernel<double>) in the greedy and the sweep
    order; exact6_sweep = the sweep order alone, twice (permute_tensor32_kernel,
    gemm_thin_kernel<double>); padded = 30-sweep mixed solves of the 16x16 D=4 and 12x12 D=6 open
    lattices on the zero-padded tensor-core sweep (bp_tc_kernel with PAD, one launch per sweep);
    open16 = FP32 and FP64 solves of the 16x16 D=4 open lattice to tol 1e-10, twice each with
    the sweeps as one persistent launch (bp2_kernel with a grid barrier), then once with one
    launch per sweep."""
    from itn_gb300 import BPEngine
    from itn_gb300 import graphs as G
    if name in ("d8", "mixed"):
        g, t = workload()
        with BPEngine(g, device=device) as e:
            e.set_tensors(t.astype(np.float32))
            for _ in range(2):
                e.init_messages()
                r = e.run(maxiter=4) if name == "d8" else e.run(maxiter=SWEEPS, precision="bf16",
                                                                split_sweeps=SPLIT_SWEEPS)
            print(name, "device ms", r.device_ms)
    elif name == "grad":
        g = G.square_lattice(12, 12, 6, periodic=False, phys=2)
        t = G.random_tensors(g, np.random.default_rng(5), np.float64, G.peps_scale(g)).astype(np.float32)
        with BPEngine(g, device=device) as e:
            e.set_tensors(t)
            e.init_messages()
            e.run(maxiter=200, tol=1e-12)
            print("grad", e.grad(adjoint=True, tol=1e-6)[1])
    elif name == "gate":
        print("gate", bench_apply_layer(device)["device_ms"])
    elif name == "batched":
        print("batched", bench_batched(device))
    elif name == "contract":
        from itn_gb300.contract import contract_network
        rng = np.random.default_rng(3)
        A = rng.standard_normal((2048, 2048)).astype(np.float32)
        B = rng.standard_normal((2048, 2048)).astype(np.float32)
        for prec in ("native", "bf16", "tf32x3"):
            for _ in range(2):  # the first call of a precision includes one-time set-up (self-test, module load)
                _, _, ms = contract_network([A, B], [["m", "k"], ["k", "n"]], precision=prec, return_time=True)
            print("contract", prec, "device ms", ms)
    elif name == "exact6":
        from itn_gb300.contract import contract_network, norm_network_tensors
        g6 = G.square_lattice(6, 6, 3, periodic=False, phys=2)
        t6 = G.random_tensors(g6, np.random.default_rng(63), np.float64, G.peps_scale(g6))
        ts, ls = norm_network_tensors(g6, t6)
        z, _, ms = contract_network(ts, ls, return_time=True)
        print("exact6 log z", float(np.log(z[()])), "device ms", ms)
        z, _, ms = contract_network(ts, ls, alg="sweep", return_time=True)
        print("exact6 sweep order: log z", float(np.log(z[()])), "device ms", ms)
    elif name == "padded":
        # the padded tensor-core sweep on open lattices (one launch per sweep)
        for L, D in ((16, 4), (12, 6)):
            g = G.square_lattice(L, L, D, periodic=False, phys=2)
            t = G.random_tensors(g, np.random.default_rng(100 * L + D), np.float64, G.peps_scale(g))
            with BPEngine(g, device=device) as e:
                e.set_tensors(t.astype(np.float32))
                for _ in range(2):
                    e.init_messages()
                    r = e.run(maxiter=SWEEPS, precision="bf16", split_sweeps=SPLIT_SWEEPS)
                print(f"padded {L}x{L} D={D} bf16 mixed: device ms {r.device_ms:.4f}, launches {r.kernel_launches}")
    elif name == "open16":
        g = G.square_lattice(16, 16, 4, periodic=False, phys=2)
        t = G.random_tensors(g, np.random.default_rng(16), np.float64, G.peps_scale(g))
        for dt in (np.float32, np.float64):
            with BPEngine(g, device=device) as e:
                e.set_tensors(t.astype(dt))
                for mode in (0, 0, 1):
                    e.inject_fault("no_persistent_sweeps", mode)
                    e.init_messages()
                    r = e.run(maxiter=50, tol=1e-10)
                    print(f"open16 {np.dtype(dt).name} {'per-sweep' if mode else 'persistent'}: "
                          f"{r.iterations} sweeps, device ms {r.device_ms:.4f}, launches {r.kernel_launches}")
    elif name == "exact6_sweep":
        from itn_gb300.contract import contract_network, norm_network_tensors
        g6 = G.square_lattice(6, 6, 3, periodic=False, phys=2)
        t6 = G.random_tensors(g6, np.random.default_rng(63), np.float64, G.peps_scale(g6))
        ts, ls = norm_network_tensors(g6, t6)
        for _ in range(2):
            z, _, ms = contract_network(ts, ls, alg="sweep", return_time=True)
        print("exact6 sweep order: log z", float(np.log(z[()])), "device ms", ms)
    else:
        raise SystemExit(f"unknown case {name}")
    return 0


def bench_16x16(device):
    """16x16 open PEPS, d=2, D=4, N(0,1)/sqrt(d D^4): 50 parallel sweeps or tol 1e-10, FP32
    and FP64; plus the BP error of a 6x6 D=3 network against its exact contraction."""
    from itn_gb300 import BPEngine
    from itn_gb300 import graphs as G
    from itn_gb300.contract import contract_network, norm_network_tensors
    g = G.square_lattice(16, 16, 4, periodic=False, phys=2)
    rng = np.random.default_rng(16)
    t = G.random_tensors(g, rng, np.float64, G.peps_scale(g))
    out = {"workload": "peps 16x16 open D=4 d=2, maxiter 50 / tol 1e-10"}
    for name, dt in (("fp32", np.float32), ("fp64", np.float64)):
        e = BPEngine(g, device=device)
        e.set_tensors(t.astype(dt))
        best = None
        for rep in range(3):
            e.init_messages()
            r = e.run(maxiter=50, tol=1e-10)
            best = r if best is None or r.device_ms < best.device_ms else best
        out[name] = {"iterations": best.iterations, "ms": best.device_ms,
                     "updates_per_s": best.iterations * g.nslots / (best.device_ms * 1e-3)}
        e.close()
    out["tensor_cores"] = bench_padded_tc(device)
    g6 = G.square_lattice(6, 6, 3, periodic=False, phys=2)
    t6 = G.random_tensors(g6, np.random.default_rng(63), np.float64, G.peps_scale(g6))
    e = BPEngine(g6, device=device)
    e.set_tensors(t6)
    e.init_messages()
    e.run(maxiter=200, tol=1e-12)
    lz_bp = e.bethe_free_energy()
    e.close()
    ts, ls = norm_network_tensors(g6, t6)
    z, _, ms = contract_network(ts, ls, return_time=True)
    zs, _, ms_s = contract_network(ts, ls, alg="sweep", return_time=True)
    out["exact_6x6_D3"] = {"logz_exact": float(np.log(z[()])), "logz_bp": lz_bp,
                           "bp_abs_err": abs(lz_bp - float(np.log(z[()]))), "contract_ms": ms,
                           "contract_ms_sweep_order": ms_s,
                           "sweep_vs_greedy_rel_diff": abs(zs[()] - z[()]) / abs(z[()])}
    return out


def bench_padded_tc(device):
    """Tensor-core sweeps of open-boundary lattices (vertices of 2-4 legs, zero-padded to the
    8 x 8 x 8 x 8 x 2 frame, one launch per sweep) beside the FP32 CUDA-core sweeps of the same
    networks: 16x16 D=4 and 12x12 D=6, d=2, N(0,1)/sqrt(d D^4), 30 parallel sweeps from the
    normalised identity (device time of the solve, best of 3), and with the stopping rule
    maxiter 50 / tol 1e-10 for the FP32-accurate modes."""
    from itn_gb300 import BPEngine
    from itn_gb300 import graphs as G
    out = {}
    for L, D in ((16, 4), (12, 6)):
        g = G.square_lattice(L, L, D, periodic=False, phys=2)
        t = G.random_tensors(g, np.random.default_rng(100 * L + D), np.float64, G.peps_scale(g))
        e = BPEngine(g, device=device)
        e.set_tensors(t.astype(np.float32))
        res = {}
        for name, kw in (("fp32_cuda_cores", {}), ("bf16_27_split_3", dict(precision="bf16", split_sweeps=3)),
                         ("tf32x3", dict(precision="tf32x3")), ("fp32_cuda_cores_tol", dict(tol=1e-10)),
                         ("tf32x3_tol", dict(precision="tf32x3", tol=1e-10))):
            maxiter = 50 if "tol" in kw else 30
            best = None
            for rep in range(3):
                e.init_messages()
                r = e.run(maxiter=maxiter, **kw)
                best = r if best is None or r.device_ms < best.device_ms else best
            res[name] = {"iterations": best.iterations, "ms": best.device_ms,
                         "updates_per_s": best.iterations * g.nslots / (best.device_ms * 1e-3)}
        e.close()
        out[f"open{L}x{L}_D{D}"] = res
    return out


def bench_apply_layer(device):
    """BP simple-update gate application (apply_operators.jl): one layer of 128 random
    two-site gates on the horizontal bonds (even columns) of a 16x16 open PEPS, d=2, D=4,
    environments from a converged FP64 BP solve, truncation to rank 4.  The whole layer is
    one itn_apply_gates batch (one CTA per gate); the CPU leg applies the same gates with the
    numpy restatement of the algorithm, one by one, on the host."""
    from itn_gb300 import network as N
    from itn_gb300.apply import apply_gates
    L, D, d = 16, 4, 2
    rng = np.random.default_rng(1616)
    s = {(x, y): N.Index(d) for x in range(L) for y in range(L)}
    h = {(x, y): N.Index(D) for x in range(L - 1) for y in range(L)}
    v = {(x, y): N.Index(D) for x in range(L) for y in range(L - 1)}
    tensors = {}
    for x in range(L):
        for y in range(L):
            inds = [s[(x, y)]]
            if x > 0:
                inds.append(h[(x - 1, y)])
            if x < L - 1:
                inds.append(h[(x, y)])
            if y > 0:
                inds.append(v[(x, y - 1)])
            if y < L - 1:
                inds.append(v[(x, y)])
            shape = [i.dim for i in inds]
            tensors[(x, y)] = N.ITensor(rng.standard_normal(shape) / np.sqrt(d * D ** 4), inds)
    tn = N.ITensorNetwork(tensors)
    nn = N.NormNetwork(tn)
    env = N.beliefpropagation(nn, N.message_environment("one", nn), stopping_criterion=dict(maxiter=200, tol=1e-10))
    ops = []
    for x in range(0, L - 1, 2):
        for y in range(L):
            cod = [N.Index(d), N.Index(d)]
            ops.append(N.operator(rng.standard_normal((d, d, d, d)), cod, [s[(x, y)], s[(x + 1, y)]]))
    gates = [N._gate_of(op, tn, env) for op in ops]
    times = []
    for _ in range(4):
        t0 = time.perf_counter()
        res, ms = apply_gates(gates, max_rank=D, return_time=True)
        times.append((ms, time.perf_counter() - t0))
    ms = min(t[0] for t in times[1:])
    wall = min(t[1] for t in times[1:])
    out = {"workload": "16x16 open PEPS d=2 D=4, 128 two-site gates (one layer), BP environments, trunc rank 4, FP64",
           "gates": len(gates), "device_ms": ms, "gates_per_s_device": len(gates) / (ms * 1e-3),
           "e2e_ms": wall * 1e3, "gates_per_s_e2e": len(gates) / wall,
           "bond_dims": sorted(set(int(len(r[2])) for r in res))}
    try:
        sys.path.insert(0, ROOT)
        from oracle import apply_oracle as AO
        t0 = time.perf_counter()
        for g in gates:
            AO.apply_gate_2site(g.sites[0], g.sites[1], g.envs[0], g.envs[1], g.op, maxrank=D)
        cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(gates) / cpu, "unit": "gates/s", "cores": 1, "kind": "port",
                               "sample": "the same 128 gates, numpy restatement, one by one"}
    except Exception as exc:  # the CPU restatement is only a baseline: its absence leaves the GPU number
        out["cpu_baseline"] = {"unavailable": str(exc)}
    return out


def G_identity(g):
    from itn_gb300 import graphs as G
    return G.identity_messages(g, np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("ITN_BENCH_PRECISION", "bf16"),
                    choices=["native", "bf16", "tf32", "tf32x3"])
    ap.add_argument("--case", default=None, choices=["d8", "mixed", "grad", "gate", "contract", "batched", "exact6", "exact6_sweep", "open16",
                                                        "padded"],
                    help="run one small profiling case instead of the benchmark")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-extra", dest="extra", action="store_false",
                    help="skip the secondary configurations (gradient, batched, 16x16, exact 6x6)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    import __graft_entry__
    __graft_entry__.build()
    if args.case:
        return run_case(args.case)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
