"""Benchmark: 30-qubit f64 random circuit (depth 40 + qft) on one GB300, qvnt semantics.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--engine tensor64|plain|fused]

A step is one run of the workload circuit on a resident 30-qubit register: reset to |0> and
apply the 2,967-gate queue (40 layers of {h, s, t, u3} on every qubit, 15 random two-qubit gates
from {rxx, ryy, rzz, swap, i_swap, sqrt_i_swap}, 3 Toffolis, then qft over all 30 qubits).
Inputs are seeded synthetic circuits (no public suite).  The state (16 GiB) is larger than L2
(129 MB), so no flush is needed between steps.

The headline engine is TENSOR64: IEEE f64 amplitudes at the call boundary, 64-bit block floating
point between passes, gates fused into dense 5-qubit blocks and contracted on the tensor cores as
exact fp16 digit products (no FP64 instruction, one rounding per pass to 2^-54 of the largest
component).  Printed as one JSON line (rank 0):
  value        unfused gate passes per second (qvnt SingleOps), whole job, device-timed
  e2e          the same metric through the plugin call qvnt_apply_host (Applicable::apply): the
               state goes host -> device -> host from pinned memory inside the timed region
  roofline     the engine's pass kernel: algorithmic bytes (2 x 2^30 x 16 B per pass) / its
               average CUDA-event duration, against the measured HBM copy bandwidth
  plain_f64_gpu the PLAIN engine (one IEEE f64 pass per SingleOp, bit-identical to qvnt) on the
               same circuit
  cpu_baseline the CPU oracle (qvnt's algorithm restated in C: one out-of-place gather pass per
               gate, OpenMP on every host core) timed per gate on a stratified sample of the same
               circuit at 30 qubits (1-qubit gates, 2-qubit gates, Toffolis, QFT rotations)
  forms        the double-float fused engine (df64), the batching, serving and precision forms
--impl reference times only that CPU implementation (the reference is Rust; no cargo exists here),
with the circuit built by the oracle's own builders, so no engine code runs in that process.
With N > 1 (torchrun) each rank runs an independent replica on its own GPU ("replicas only").
"""
import argparse
import ctypes
import json
import os

# 32 hardware work queues for the serving form's concurrent streams; must precede CUDA initialisation
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
DEPTH = 40
SEED = 2
AMP_BYTES = 16
PROFILE_TRAFFIC = {"fused": os.path.join(ROOT, "profiles", "fused_pass_traffic.json"),
                   "tensor64": os.path.join(ROOT, "profiles", "tensor64_pass_traffic.json")}
KERNEL = {"tensor64": "tensor64_pass_kernel", "fused": "fused_df_kernel", "plain": "plain_gate_kernel"}
ARITHMETIC = {
    "tensor64": "IEEE f64 at every call boundary; between the passes of a call 64-bit block floating point "
                "(int64 components, one exponent per register, the largest renormalised to 2^53..2^54 before "
                "each pass); dense 5-qubit blocks on tcgen05, each operand split into 7 exact fp16 digits "
                "(34 digit products, FP32 accumulation of integers below 2^23, exact), one rounding per pass "
                "to 2^-54 of the largest component; no FP64 instruction",
    "plain": "IEEE f64, one pass per SingleOp in qvnt's operand order, bit-identical to the oracle",
    "fused": "double-float (pairs of FP32 with error-free transforms, 48-bit significand, FP32 exponent range) on "
             "the FP32 pipes, within 1e-12 of the IEEE f64 oracle",
}
DTYPE = {"tensor64": "f64 (int64 block floating point between passes)", "plain": "f64", "fused": "df64 (2 x f32, 48-bit significand)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=N_QUBITS)
    ap.add_argument("--depth", type=int, default=DEPTH)
    ap.add_argument("--engine", default="tensor64", choices=["tensor64", "plain", "fused"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=1, help="steps of the plain f64 GPU path (0 = skip)")
    ap.add_argument("--forms", default="plain,df64,batch,serve,precision",
                    help="extra forms to measure: plain, df64, batch, serve, precision (empty = none)")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--mma-costs", action="store_true",
                    help="print the tensor-core instruction costs that bound the TENSOR64 pass, then exit")
    ap.add_argument("--serve-engine", default="fused", choices=["tensor64", "fused"],
                    help="engine of the serving form's registers (fused: small CTAs share an SM with other "
                         "requests' tiles; a tensor64 CTA holds a whole SM)")
    ap.add_argument("--cpu-per-class", type=int, default=3, help="gates per stratum in the cpu_baseline sample")
    ap.add_argument("--precision-qubits", type=int, default=32)
    ap.add_argument("--precision-depth", type=int, default=60)
    ap.add_argument("--precision-ref-qubits", type=int, default=30, help="size of the fidelity check (0 = none)")
    ap.add_argument("--batch-fusion", default="auto", help="batch form: 'auto' (autotune) or 'K,BUDGET'")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, rank, local, backend):
        self.ws, self.rank = ws, rank
        self.pg = None
        if ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group(backend=backend, rank=rank, world_size=ws)
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if self.td.get_backend() == "nccl" else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if self.td.get_backend() == "nccl" else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_pass_bytes(n):
    return 2 * (1 << n) * AMP_BYTES


def workload_config(n, depth, gates, ws):
    """The workload's description, identical in both arms (ours and --impl reference)."""
    return {"workload": "random circuit %dq f64, depth %d + qft, %d gates" % (n, depth, gates), "n_qubits": n,
            "depth": depth, "seed": SEED, "gates": gates, "parallelism": "replicas" if ws > 1 else "single",
            "l2": "state %d GiB > L2 129 MB, no flush" % ((1 << n) * AMP_BYTES >> 30)}


class CpuSampler:
    """The oracle (qvnt's algorithm: one out-of-place gather pass per gate over every amplitude,
    src/operator/atomic/dispatch.rs:50-67, OpenMP over all host threads) timed gate by gate on a
    stratified sample of the circuit: `per_class` gates from each of its strata (1-qubit gates,
    2-qubit gates, Toffolis, QFT controlled rotations), spread over the whole circuit and different
    on every call; the circuit's time is estimated as sum over strata of (gates in the stratum) x
    (mean sampled time).  The circuit is built with the oracle's own builders.  Returns gate passes
    per second, threads and a description of the sample."""

    def __init__(self, n, depth, seed):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import numpy as np
        import oracle_ref as orc
        self.orc, self.n = orc, n
        self.gates = orc.random_circuit_gates(n, depth, seed=seed)
        self.arr = orc.arr(self.gates)
        self.strata = {}
        for i, g in enumerate(self.gates):
            self.strata.setdefault(orc.gate_class(g), []).append(i)
        self.threads = orc.max_threads()
        self.cur = orc.new_state(n, 0)
        self.nxt = np.zeros_like(self.cur)  # touched once here, outside any timed pass
        self.calls = 0

    def _pass(self, i):
        t0 = time.perf_counter()
        self.orc.lib().oracle_for_each(ctypes.byref(self.arr[i]), self.cur.ctypes.data, self.nxt.ctypes.data,
                                       self.cur.size, self.threads)
        dt = time.perf_counter() - t0
        self.cur, self.nxt = self.nxt, self.cur
        return dt

    def sample(self, per_class):
        est, timed, counts = 0.0, 0, {}
        for name in sorted(self.strata):
            idx = self.strata[name]
            picks = [idx[((self.calls * per_class + k) * 7919 + len(idx) // 2) % len(idx)] for k in range(per_class)]
            ts = [self._pass(i) for i in picks]
            est += len(idx) * sum(ts) / len(ts)
            timed += len(ts)
            counts[name] = len(idx)
        self.calls += 1
        desc = ("%d gate passes timed at %d qubits, %d per stratum of %s, circuit time = sum of stratum size x mean "
                "sampled pass time" % (timed, self.n, per_class, counts))
        return len(self.gates) / est, self.threads, desc


def bench_batch(ctx, count, steps, fusion="auto"):
    """Batching form: `count` registers (n uniform in [8, 20], depth uniform in [10, 60], random basis
    state, measure_mask of all qubits) in one persistent launch per run, tile width and pass budget
    autotuned on every 16th register.  Beside it, the plain f64 GPU path (one register at a time,
    one pass per gate) on every 64th register, extrapolated to the batch."""
    import numpy as np
    from qvnt_gb300 import ENGINE_PLAIN, QReg
    from qvnt_gb300.batch import Batch
    from qvnt_gb300.circuits import SplitMix64, batch_workload

    w = batch_workload(count=count)
    b = Batch(w.q_nums, w.states, w.gates, w.offsets, w.masks, ctx=ctx)
    if fusion == "auto":
        k, budget, tune_ms = b.autotune(stride=16)
    else:
        k, budget = (int(x) for x in fusion.split(","))
        b.set_fusion(k, budget)
        tune_ms = None
    rng = SplitMix64(17)
    u01 = np.array([rng.uniform() for _ in range(w.count)])
    b.run(u01)  # warm-up
    ms = []
    t0 = time.perf_counter()
    for _ in range(steps):
        b.run(u01)
        ms.append(b.info()["last_ms"])
    wall = time.perf_counter() - t0
    info = b.info()
    b.close()
    dev_s = sum(ms) / 1e3
    sample = list(range(0, w.count, 64))
    import torch
    t_plain = 0.0
    for i in sample:
        q = QReg.with_state(int(w.q_nums[i]), int(w.states[i]), ctx=ctx)
        q.set_engine(ENGINE_PLAIN)
        ptr, cnt = w.gates_of(i)
        q.sync()
        t1 = time.perf_counter()
        q.apply_gates(ptr, cnt)
        q.measure_mask(int(w.masks[i]), u01=float(u01[i]))
        q.sync()
        t_plain += time.perf_counter() - t1
        q.close()
    torch.cuda.synchronize()
    plain_cps = len(sample) / t_plain
    return {"workload": "%d registers, n uniform [8, 20], depth uniform [10, 60] random layers, measure_mask(all)"
                        % w.count,
            "circuits_per_s": w.count * steps / dev_s, "gate_passes_per_s": w.total_gates * steps / dev_s,
            "ms_per_run": dev_s * 1e3 / steps, "e2e_circuits_per_s": w.count * steps / wall,
            "gates": w.total_gates, "state_bytes": info["state_bytes"], "schedule_items": info["items"],
            "passes": info["passes"], "fusion_k": k, "pass_budget": budget, "autotune_best_sample_ms": tune_ms,
            "launches_per_run": 1, "dtype": "df64 (2 x f32, 48-bit significand), within 1e-12 of IEEE f64",
            "plain_f64_gpu": {"circuits_per_s": plain_cps, "sample": "every 64th register (%d), one at a time"
                              % len(sample)}}


def bench_precision(ctx, n=32, depth=60, n_ref=30):
    """Precision form: complex<f32> register of n qubits (32 GiB at 32), the random-layer generator
    at depth 60, dense 5-qubit blocks on the tensor cores with FP64 norm restoration every 10
    passes.  Fidelity defect and max-abs error against the PLAIN IEEE f64 engine (bit-identical to
    the oracle) at n_ref qubits with the same seed; the plain f64 GPU path at n qubits timed on the
    first 64 gates and extrapolated per gate."""
    import torch
    from qvnt_gb300 import ENGINE_PLAIN, ENGINE_PRECISION, QReg
    from qvnt_gb300.circuits import SplitMix64, random_layers_gates

    def gates(m):
        return random_layers_gates(m, depth, SplitMix64(3))

    arr, cnt = gates(n)
    q = QReg(n, 0, ctx=ctx, engine=ENGINE_PRECISION)
    q.apply_gates(arr, cnt)  # warm-up
    q.sync()
    q.kernel_timing(enable=1)
    s = torch.cuda.ExternalStream(q.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _, p0 = q.stats()
    e0.record(s)
    q.reset(0)
    q.apply_gates(arr, cnt)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kms, kn = q.kernel_timing(enable=0)
    _, p1 = q.stats()
    q.close()
    del q
    pass_bytes = 2 * (1 << n) * 8
    # plain f64 path at the same size, per gate on a sample
    qp = QReg(n, 0, ctx=ctx, engine=ENGINE_PLAIN)
    sp = torch.cuda.ExternalStream(qp.stream())
    sample = min(64, cnt)
    qp.apply_gates(arr, 4)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(sp)
    qp.apply_gates(arr, sample)
    f1.record(sp)
    torch.cuda.synchronize()
    plain_ms_per_gate = f0.elapsed_time(f1) / sample
    qp.close()
    del qp
    # fidelity at n_ref qubits against IEEE f64 (the plain engine, bit-identical to the oracle)
    fid, mx, cnt_r = float("nan"), float("nan"), 0
    if n_ref:
        arr_r, cnt_r = gates(n_ref)
        a = QReg(n_ref, 0, ctx=ctx, engine=ENGINE_PRECISION)
        a.apply_gates(arr_r, cnt_r)
        b = QReg(n_ref, 0, ctx=ctx, engine=ENGINE_PLAIN)
        b.apply_gates(arr_r, cnt_r)
        fid, mx = a.overlap(b)
        a.close()
        b.close()
    avg = kms / kn
    return {"workload": "%d qubits complex<f32>, random layers depth %d (%d gates), dense 5-qubit blocks on tcgen05 "
                        "(TF32 hi/lo, FP32 accumulate), FP64 norm restoration every 10 passes" % (n, depth, cnt),
            "circuits_per_s": 1e3 / ms, "ms_per_circuit": ms, "gate_passes_per_s": cnt / (ms / 1e3),
            "passes": p1 - p0, "kernel_avg_ms": avg, "kernel_gbs": pass_bytes / (avg / 1e3) / 1e9,
            "fidelity_defect_vs_f64": 1.0 - fid, "max_abs_err_vs_f64": mx, "fidelity_qubits": n_ref,
            "fidelity_reference": "PLAIN engine (IEEE f64, bit-identical to the oracle), same seed, %d gates" % cnt_r,
            "plain_f64_gpu": {"circuits_per_s": 1e3 / (plain_ms_per_gate * cnt),
                              "sample": "first %d gates at %d qubits, extrapolated per gate" % (sample, n)}}


def bench_plain_kernels(ctx, n=30, reps=8):
    """The PLAIN engine's kernels gate by gate on a 30-qubit register: per case (kind, target
    qubits, controls) the mean CUDA-event time of one launch and the HBM bandwidth of the bytes it
    must move (read + write of the 2^(n - controls) amplitudes it touches; the SWAP family touches
    only the half whose two bits differ).  Low targets (all below qubit 5) run the warp-shuffle
    kernel, the others the strided-orbit kernel."""
    from qvnt_gb300 import ENGINE_PLAIN, QReg, op
    from qvnt_gb300.operator import MultiOp
    cases = [("x", op.x(1 << 0), 0, 1.0), ("x", op.x(1 << 20), 0, 1.0), ("x", op.x(0b10110), 0, 1.0),
             ("z", op.z(1 << 3), 0, 1.0), ("s", op.s(1 << 25), 0, 1.0), ("t", op.t(1 << 2), 0, 1.0),
             ("rx", op.rx(0.3, 1 << 1), 0, 1.0), ("rx", op.rx(0.3, 1 << 22), 0, 1.0),
             ("ry", op.ry(0.7, 1 << 4), 0, 1.0), ("rz", op.rz(0.7, 1 << 28), 0, 1.0),
             ("h1", op.h(1 << 0), 0, 1.0), ("h1", op.h(1 << 29), 0, 1.0),
             ("h2", op.h(0b11), 0, 1.0), ("h2", op.h((1 << 12) | (1 << 27)), 0, 1.0),
             ("rxx", op.rxx(1.1, 0b1010), 0, 1.0), ("rxx", op.rxx(1.1, (1 << 8) | (1 << 21)), 0, 1.0),
             ("rzz", op.rzz(1.1, (1 << 5) | (1 << 20)), 0, 1.0),
             ("swap", op.swap(0b11), 0, 0.5), ("swap", op.swap((1 << 10) | (1 << 25)), 0, 0.5),
             ("toffoli", op.x(1 << 7).c((1 << 3) | (1 << 19)), 2, 1.0)]
    q = QReg(n, 0, ctx=ctx)
    q.set_engine(ENGINE_PLAIN)
    q.apply(op.h((1 << n) - 1))
    out = []
    for name, one, ctrls, frac in cases:
        ops = MultiOp(list(one.ops) * reps)
        q.apply(ops)  # warm-up
        q.sync()
        q.kernel_timing(enable=1)
        q.apply(ops)
        ms, k = q.kernel_timing(enable=0)
        per = ms / k
        moved = 2 * (1 << (n - ctrls)) * AMP_BYTES * frac
        tg = one.ops[0].g
        out.append({"gate": name, "targets": hex(tg.a_mask | tg.b_mask), "ctrl": hex(tg.ctrl),
                    "kernel": "diagonal" if name in ("z", "s", "t", "rz", "rzz") else
                    "shuffle" if ((tg.a_mask | tg.b_mask) < 32 and not (tg.ctrl & 31) and name != "swap") else "orbit",
                    "ms": per, "gbs": moved / (per / 1e3) / 1e9})
    q.close()
    return {"workload": "one gate of each case on a %d-qubit PLAIN register, %d launches each" % (n, reps),
            "cases": out}


def bench_serve(ctx, rate, seconds, engine=None):
    """Serving form: Poisson arrivals at `rate`/s for `seconds` s (n log-uniform [10, 28], depth
    uniform [5, 100] over 1-3 apply/measure rounds, 150 GB HBM budget, 32 slots, queue of 1024);
    then 5 s to drain.  Latency = completion - scheduled arrival.  The server's registers run on
    `engine` (the context's default engine when None)."""
    import numpy as np
    from qvnt_gb300.circuits import serve_requests
    from qvnt_gb300.serve import Server

    max_queue = 1024
    if engine is not None:
        ctx.set_engine(engine)
    s = Server(budget_bytes=150 * 10**9, slots=32, max_queue=max_queue, ctx=ctx)
    t0 = s.clock()
    offered = shed = 0
    for r in serve_requests(rate=rate, duration=seconds, seed=5):
        offered += 1
        lag = r.arrival - (s.clock() - t0)
        if lag > 0:
            time.sleep(lag)
        if s.stats()["queued"] >= max_queue:
            shed += 1  # shed without building the circuit
            continue
        gates, calls = r.build()
        if s.submit(r.n, r.state, gates, calls, arrival=t0 + r.arrival, detached=True) is None:
            shed += 1
    time.sleep(5.0)
    st = s.stats()
    lat = s.latencies()
    ages = s.queued_ages()
    elapsed = s.clock() - t0
    s.close()
    pct = (lambda a, p: float(np.percentile(a, p)) * 1e3 if a.size else None)
    censored = np.concatenate([lat, ages]) if ages.size else lat
    return {"workload": "Poisson %.0f req/s for %.0f s, n log-uniform [10, 28], depth uniform [5, 100], "
                        "1-3 apply/measure rounds, 150 GB budget, 32 slots, queue 1024" % (rate, seconds),
            "offered": offered, "submitted": st["submitted"], "shed": shed, "completed": st["completed"],
            "failed": st["failed"], "queued_at_end": st["queued"], "running_at_end": st["running"],
            "served_circuits_per_s": st["completed"] / elapsed, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "p99_ms_incl_queued": pct(censored, 99), "peak_running": st["peak_running"], "elapsed_s": elapsed}


def run_reference(args, ws, rank):
    """--impl reference: qvnt's CPU algorithm on the host cores (the C restatement of the oracle;
    the Rust crate cannot be built here), rank 0 only.  Each step times one stratified sample of the
    workload's gate passes (about 8 s); nothing of the engine library is loaded."""
    if rank != 0:
        return
    sampler = CpuSampler(args.qubits, args.depth, SEED)
    vals, walls, desc, threads = [], [], "", 1
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        v, threads, desc = sampler.sample(1)
        if i >= args.warmup:
            vals.append(v)
            walls.append(time.perf_counter() - t0)
    value = sum(vals) / len(vals)
    unit = "gate-passes/s"
    line = {
        "impl": "reference", "metric": "%dq gate-passes/s" % args.qubits, "value": value, "unit": unit,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(walls) / len(walls) * 1e3,
        "ms_per_circuit_estimate": len(sampler.gates) / value * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded SplitMix64 random circuit)",
        "config": workload_config(args.qubits, args.depth, len(sampler.gates), ws),
        "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port",
                         "sample": "per step: " + desc + "; value = mean over steps"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_df64(ctx, circ_arr, ngates, n, steps):
    """The double-float fused engine (48-bit significand, FP32 exponent range: narrower than IEEE
    f64) on the same circuit: gate passes/s and its per-pass HBM roofline."""
    import torch
    from qvnt_gb300 import ENGINE_FUSED, QReg
    q = QReg(n, 0, ctx=ctx)
    q.set_engine(ENGINE_FUSED)
    s = torch.cuda.ExternalStream(q.stream())
    q.reset(0)
    q.apply_gates(circ_arr, ngates)
    q.sync()
    _, p0 = q.stats()
    q.kernel_timing(enable=1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        q.reset(0)
        q.apply_gates(circ_arr, ngates)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kms, kn = q.kernel_timing(enable=0)
    _, p1 = q.stats()
    q.close()
    avg = kms / kn if kn else None
    return {"value": ngates * steps / (ms / 1e3), "unit": "gate-passes/s", "ms_per_step": ms / steps, "steps": steps,
            "dtype": DTYPE["fused"], "arithmetic": ARITHMETIC["fused"], "passes_per_step": (p1 - p0) / steps,
            "kernel": KERNEL["fused"], "avg_launch_ms": avg,
            "kernel_gbs": algorithmic_pass_bytes(n) / (avg / 1e3) / 1e9 if avg else None}


def mma_costs(device):
    """The tensor-core instruction costs that bound the TENSOR64 pass (SM cycles, all SMs issuing):
    one tcgen05.mma.kind::f16 (M = 128, K = 16) of N = 64 and of N = 256, and a pass tile's 44 MMAs."""
    import ctypes
    from qvnt_gb300 import Context
    from qvnt_gb300._abi import check, lib
    ctx = Context(device)
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(lib().qvnt_tensor64_mma_costs(ctx.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    print(json.dumps({"measurement": "tcgen05.mma.kind::f16 cost, M = 128, K = 16, A from tensor memory",
                      "cycles_per_mma_n64": a.value, "cycles_per_mma_n256": b.value,
                      "cycles_per_pass_tile_44_mmas": c.value}), flush=True)
    ctx.close()


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.mma_costs:
        mma_costs(local)
        return
    import numpy as np
    import torch
    from qvnt_gb300 import ENGINE_FUSED, ENGINE_PLAIN, ENGINE_TENSOR64, Context, QReg
    from qvnt_gb300._abi import gate_array
    from qvnt_gb300.circuits import random_circuit

    torch.cuda.set_device(local)
    dist = Dist(ws, rank, local, "nccl")
    ctx = Context(local)
    n = args.qubits
    circ = random_circuit(n, args.depth, seed=SEED)
    gates = circ.gates()
    garr = gate_array(gates)
    ngates = len(gates)
    engines = {"tensor64": ENGINE_TENSOR64, "plain": ENGINE_PLAIN, "fused": ENGINE_FUSED}
    engine = engines[args.engine]

    q = QReg(n, 0, ctx=ctx)
    q.set_engine(engine)
    stream = torch.cuda.ExternalStream(q.stream())

    def step():
        q.reset(0)
        q.apply_gates(garr, ngates)

    for _ in range(args.warmup):
        step()
    q.sync()
    launches0, passes0 = q.stats()
    q.kernel_timing(enable=1)
    clocks = ClockSampler(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)
    kern_ms, kern_n = q.kernel_timing(enable=0)
    launches1, passes1 = q.stats()
    ms_max = dist.max(dev_ms)
    gpu_launches = int(dist.sum(launches1 - launches0))
    passes_per_step = (passes1 - passes0) / args.steps

    units = ngates * args.steps * ws
    value = units / (ms_max / 1e3)
    pass_bytes = algorithmic_pass_bytes(n)
    if engine == ENGINE_PLAIN:  # one pass per gate over the 2^(n - controls) amplitudes it touches
        step_bytes = sum(2 * (1 << (n - bin(g.ctrl).count("1"))) * AMP_BYTES for g in gates if g.kind != 0)
    else:
        step_bytes = passes_per_step * pass_bytes
    hbm_gbs = step_bytes * args.steps / (dev_ms / 1e3) / 1e9

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    if not peak:
        peak = 6800.0
    avg_launch_ms = kern_ms / kern_n if kern_n else None
    if engine == ENGINE_PLAIN:
        achieved = step_bytes * args.steps / (kern_ms / 1e3) / 1e9 if kern_ms else None
    else:
        achieved = pass_bytes / (avg_launch_ms / 1e3) / 1e9 if avg_launch_ms else None
    traffic = None
    try:
        with open(PROFILE_TRAFFIC[args.engine]) as f:
            traffic = json.load(f).get("bytes_per_full_launch_%dq" % n)
    except Exception:
        pass

    # plain f64 GPU path on the same workload (one pass per SingleOp), for the comparison the metric names
    plain = None
    if args.plain_steps > 0 and engine != ENGINE_PLAIN:
        qp = QReg(n, 0, ctx=ctx)
        qp.set_engine(ENGINE_PLAIN)
        sp = torch.cuda.ExternalStream(qp.stream())
        qp.reset(0)
        qp.apply_gates(garr, ngates)  # warm-up
        qp.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(sp)
        for _ in range(args.plain_steps):
            qp.reset(0)
            qp.apply_gates(garr, ngates)
        e1.record(sp)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1)
        plain = {"value": ngates * args.plain_steps / (pms / 1e3), "unit": "gate-passes/s",
                 "ms_per_step": pms / args.plain_steps, "steps": args.plain_steps, "dtype": "f64",
                 "arithmetic": ARITHMETIC["plain"]}
        qp.close()
        del qp

    # e2e through the plugin call with host buffers (Applicable::apply semantics)
    e2e = None
    if not args.no_e2e:
        q.close()
        del q
        torch.cuda.synchronize()
        ctx.set_engine(engine)
        length = max(1 << n, 8)
        hin = torch.zeros(length * 2, dtype=torch.float64, pin_memory=True)
        hout = torch.empty(length * 2, dtype=torch.float64, pin_memory=True)
        hin[0] = 1.0
        nin = hin.numpy().view(np.complex128)
        nout = hout.numpy().view(np.complex128)

        def e2e_step():
            ctx.apply_host(circ, nin, nout)

        for _ in range(max(1, args.warmup)):  # warm-up: the plugin register, the pinned buffers' first copies
            e2e_step()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        dist.barrier()
        e2e_s = dist.max(time.perf_counter() - t0)
        e2e = {"value": ngates * args.steps * ws / e2e_s, "unit": "gate-passes/s",
               "h2d_bytes_per_step": length * AMP_BYTES + ngates * ctypes.sizeof(gates[0]),
               "d2h_bytes_per_step": length * AMP_BYTES, "engine": args.engine}

    forms = {}
    ctx.set_engine(ENGINE_FUSED)  # the forms choose their engines themselves
    if args.no_e2e:  # the e2e leg has already released the 30-qubit register
        q.close()
        del q
    if rank == 0:
        torch.cuda.synchronize()
        for form in [f for f in args.forms.split(",") if f]:
            try:
                if form == "plain":
                    forms["plain_kernels"] = bench_plain_kernels(ctx, n)
                elif form == "df64":
                    if engine != ENGINE_FUSED:
                        forms["df64"] = bench_df64(ctx, garr, ngates, n, max(1, min(args.steps, 3)))
                elif form == "batch":
                    forms["batch"] = bench_batch(ctx, args.batch_count, max(1, min(args.steps, 5)), args.batch_fusion)
                elif form == "serve":
                    # server registers launch one CTA per tile, so that small requests' tiles
                    # interleave with large requests' passes
                    se = {"tensor64": ENGINE_TENSOR64, "fused": ENGINE_FUSED}[args.serve_engine]
                    forms["serve"] = bench_serve(ctx, args.serve_rate, args.serve_seconds, se)
                    forms["serve"]["engine"] = {"tensor64": "tensor64 (f64)", "fused": "fused (double-float)"}[args.serve_engine]
                    # the same request mix at a rate one GPU sustains (the configured rate is about
                    # two orders of magnitude above its capacity for this mix)
                    forms["serve"]["at_sustainable_rate"] = bench_serve(ctx, 4.0, min(args.serve_seconds, 20.0), se)
                    # the plain f64 GPU path serving the same mix (20 s of the same Poisson stream)
                    pl = bench_serve(ctx, args.serve_rate, min(args.serve_seconds, 20.0), ENGINE_PLAIN)
                    forms["serve"]["plain_f64_gpu"] = {
                        "served_circuits_per_s": pl["served_circuits_per_s"], "p50_ms": pl["p50_ms"],
                        "p99_ms": pl["p99_ms"], "completed": pl["completed"],
                        "sample": "the same Poisson mix for %.0f s on the PLAIN engine" % min(args.serve_seconds, 20.0)}
                    ctx.set_engine(ENGINE_FUSED)
                elif form == "precision":
                    forms["precision"] = bench_precision(ctx, args.precision_qubits, args.precision_depth,
                                                         args.precision_ref_qubits)
            except Exception as exc:  # a form's failure is reported, not hidden
                forms[form] = {"error": "%s: %s" % (type(exc).__name__, exc)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        sampler = CpuSampler(n, args.depth, SEED)
        v, threads, desc = sampler.sample(args.cpu_per_class)
        cpu = {"value": v, "unit": "gate-passes/s", "cores": threads, "kind": "port", "sample": desc}
        del sampler

    if rank == 0:
        regime = {
            "tensor64": "one pass per dense 5-qubit block: TMA tile loads/stores overlap the digit products on "
                        "the tensor cores and the integer slicing/reconstruction on the CUDA cores",
            "fused": "compute-bound: double-float arithmetic on the FP32/ALU pipes",
            "plain": "one pass per gate; rotations bound by the FP64 pipe (about 1.6 FP64 ops/clk/SM), "
                     "permutations by HBM; achieved = all gates' algorithmic bytes over their kernel time",
        }[args.engine]
        line = {
            "metric": "%dq gate-passes/s" % n,
            "value": value,
            "unit": "gate-passes/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": DTYPE[args.engine],
            "data": "synthetic (seeded SplitMix64 random circuit)",
            "config": workload_config(n, args.depth, ngates, ws),
            "engine": args.engine,
            "arithmetic": ARITHMETIC[args.engine],
            "passes_per_step": passes_per_step,
            "hbm_gbs": hbm_gbs,
            "circuits_per_s": ws * args.steps / (ms_max / 1e3),
            "wall_s": wall,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "peak_source": peak_src, "kernel": KERNEL[args.engine],
                         "launches_timed": kern_n, "avg_launch_ms": avg_launch_ms, "regime": regime},
            "plain_f64_gpu": plain,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": gpu_launches,
            "clocks": clk,
            "forms": forms,
        }
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
