"""Benchmark of the noisy-circuit hot path on GB300: gate applications per second
on the large state-vector workload (33-qubit complex64 random brickwork, depth
30, from |0...0>), with achieved HBM bandwidth against the measured peak.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Default mode "plan": the circuit is compiled once into fused tile passes
(kernels specialised per pass structure) and a step runs the whole depth-30
circuit (1470 logical gates).  Modes "fused2"/"unfused" run one brickwork layer
per step as dense gate sweeps (the per-gate form).  The state (64 GiB) is far
larger than L2, so no flush is needed between steps.
Multi-GPU runs are independent replicas (one state per GPU, no collective on
the data path; weak scaling).  `--impl reference` times the CPU restatement of
the reference's path (the reference is Julia, not runnable here) on the host
cores for the same metric.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bluetangle.jl_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

METRIC = "gate-apps/s"
# ncu-measured DRAM bytes per amplitude of one pass (read + write) of the dominant
# kernel, from single-launch captures at 28 qubits (traffic grows in proportion to
# the state, so it is scaled to the workload's 2^n amplitudes): the specialised
# fused tile pass (plan mode) moved 2.173 GB read + 2.087 GB written per 2^28
# amplitudes, the dense k_gate sweep (layer modes) 2.148 + 2.087 GB.
TRAFFIC_BYTES_PER_AMP = {"plan": (2.173e9 + 2.087e9) / 2 ** 28,
                         "sweep": (2.147591e9 + 2.087163e9) / 2 ** 28}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=33)
    ap.add_argument("--depth", type=int, default=30)
    ap.add_argument("--prec", default="c64", choices=["c64", "c128"])
    ap.add_argument("--mode", default="plan", choices=["unfused", "fused2", "plan"])
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-n", type=int, default=24, help="qubits of the CPU baseline sample")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fidelity", dest="fidelity", action="store_false",
                    help="plan mode, complex64: skip the precision statement (by default the circuit also runs "
                         "in complex128 and the line reports the infidelity and the <Z_i> deviation)")
    ap.add_argument("--autotune", action="store_true",
                    help="plan mode: time the fusion configurations on the state and keep the fastest")
    ap.add_argument("--workload", default="brickwork", choices=["brickwork", "serve", "c1", "c2", "c3", "vqa", "tc"],
                    help="brickwork: 33q c64 depth-30 (default); serve: the serving stream; c1: 12q c128 "
                         "brickwork + <Z> + shots; c2: 10q noisy density matrix; c3: 20q trajectories; tc: "
                         "tensor-core plans against scalar plans on the brickwork and an SU(4) brickwork")
    ap.add_argument("--c3-n", type=int, default=20)
    ap.add_argument("--c3-members", type=int, default=4096)
    ap.add_argument("--c3-twirl", type=int, default=64, help="twirl instances (x3 ZNE scales)")
    ap.add_argument("--c3-engine", default="program", choices=["program", "slots"])
    ap.add_argument("--rate", type=float, default=2000.0, help="serving: Poisson arrival rate (req/s)")
    ap.add_argument("--lanes", type=int, default=8, help="serving: concurrent lanes (contexts/streams)")
    ap.add_argument("--python-server", action="store_true",
                    help="serving: the Python scheduler instead of the library's bt_serve engine")
    ap.add_argument("--traj-max-n", type=int, default=14,
                    help="serving: largest qubit count of the trajectory clients (the configuration's 26 runs "
                         "their batches on the grouped executor)")
    ap.add_argument("--sustained", action="store_true",
                    help="serving: also run at 0.8x the served rate and report that latency")
    ap.add_argument("--no-serve", dest="serve", action="store_false",
                    help="headline: skip the serving measurement added to the default line")
    ap.add_argument("--serve-requests", type=int, default=10000,
                    help="headline: requests of the serving measurement added to the default line")
    return ap.parse_args()


# ------------------------------------------------------------------ workload
def layers_of(n, depth, seed):
    """Brickwork layers: list of (ones, cnots) with ones[q] = 2x2 matrix, cnots = [(q, q+1)].
    The generator is host-only Python: importing it maps no native library, so the
    reference arm loads nothing of the engine."""
    import bluetangle_gpu.circuits as C
    ops = C.brickwork(n, depth, np.random.default_rng(seed))
    out, i = [], 0
    for layer in range(depth):
        ones = {}
        for _ in range(n):
            ones[ops[i].qubit] = ops[i].mat
            i += 1
        ncx = len(range(1 if layer % 2 == 0 else 2, n, 2))
        cx = [(ops[i + j].qubit, ops[i + j].target_qubit) for j in range(ncx)]
        i += ncx
        out.append((ones, cx))
    return out


CNOT = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=complex)


def layer_program(layer, mode):
    """List of (matrix, qubits) passes for one layer and its logical gate count."""
    ones, cx = layer
    logical = len(ones) + len(cx)
    if mode == "unfused":
        prog = [(m, [q]) for q, m in sorted(ones.items())] + [(CNOT, [a, b]) for a, b in cx]
        return prog, logical
    prog, used = [], set()
    for a, b in cx:  # the layer's one-qubit gates precede its CNOTs
        prog.append((CNOT @ np.kron(ones[a], ones[b]), [a, b]))
        used |= {a, b}
    prog += [(m, [q]) for q, m in sorted(ones.items()) if q not in used]
    return prog, logical


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU baseline
def cpu_baseline(args, seconds):
    """The oracle (CPU restatement of the reference's path, complex128) on the host
    cores: brickwork layers on a cpu_n-qubit state until `seconds` elapse; the
    rate is scaled by 2^(cpu_n - n) to the workload's qubit count (work per gate
    is proportional to 2^n)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    n = args.cpu_n
    layers = layers_of(n, args.depth, args.seed)
    psi = np.zeros(2 ** n, dtype=np.complex128)
    psi[0] = 1
    gates = 0
    t0 = time.perf_counter()
    li = 0
    while time.perf_counter() - t0 < seconds:
        prog, logical = layer_program(layers[li % len(layers)], "unfused")
        O.run_gates(psi, prog)
        gates += logical
        li += 1
    dt = time.perf_counter() - t0
    rate = gates / dt / 2 ** (args.n - n)
    return {"value": rate, "unit": METRIC, "cores": O.num_threads(), "kind": "port",
            "sample": f"{li} brickwork layers ({gates} gates) on a {n}-qubit complex128 state in {dt:.1f} s "
                      f"through the oracle (the dense C restatement of the reference's gate semantics, not the "
                      f"reference's own sparse-kron path, which cannot run here), OpenMP {O.num_threads()} "
                      f"threads; the {args.n}-qubit rate is EXTRAPOLATED from it by 2^-{args.n - n} (work per "
                      f"gate is proportional to 2^n; a {args.n}-qubit complex128 state does not fit host RAM)"}


def run_reference(args):
    ws, rank, _, dist = dist_setup(args)
    if rank != 0:
        return
    per_step = max(2.0, args.cpu_seconds / 2)
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(args, per_step)
        if i >= args.warmup:
            vals.append(r["value"])
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": f"brickwork-{args.n}q-depth{args.depth}", "global_batch": 1, "seq_len": None,
                       "parallelism": "replicas", "l2": "state larger than L2", "precision": "complex128"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def run_ours(args):
    ws, rank, local, dist = dist_setup(args)
    import bluetangle_gpu as bt
    import torch

    torch.cuda.set_device(local)
    ctx = bt.Context(local, seed=args.seed + rank)
    bt.Context._default = ctx
    layers = layers_of(args.n, args.depth, args.seed)
    progs = [layer_program(l, args.mode) for l in layers]
    st = bt.zero_state(args.n, args.prec, 1, ctx)
    lib = bt.lib()
    plan = None
    tuned = None
    if args.mode == "plan":
        # the whole circuit compiled once into fused tile passes; a step runs all of it
        plan = bt.Plan(args.n, "sv", args.prec, ctx)
        for prog, _ in [layer_program(l, "unfused") for l in layers]:
            for m, qs in prog:
                plan.add_matrix(m, qs)
        t_c = time.perf_counter()
        plan.compile(True)
        compile_s = time.perf_counter() - t_c
        if args.autotune:  # fusion width / register bits / packed code chosen by timing them here
            tuned = plan.autotune(st, reps=1)
        pstats = plan.stats()
    # pre-packed column-major matrices and qubit arrays (the circuit is resident on the host)
    packed = []
    for prog, logical in progs:
        pk = []
        for m, qs in prog:
            M = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).T)
            Q = np.ascontiguousarray(qs, dtype=np.int32)
            pk.append((M, Q))
        packed.append((pk, logical))
    import ctypes
    P = ctypes.c_void_p

    def step(i):
        if plan is not None:
            plan.run(st)
            return sum(lg for _, lg in packed), pstats["passes"]
        pk, logical = packed[i % len(packed)]
        for M, Q in pk:
            rc = lib.bt_apply_matrix(st.h, len(Q), Q.ctypes.data_as(P), M.ctypes.data_as(P), 0, None, -1)
            if rc:
                ctx.check(rc)
        return logical, len(pk)

    stream = torch.cuda.ExternalStream(ctx.stream)
    for i in range(args.warmup):
        step(i)
    ctx.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    ctx.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)
    l0 = ctx.launch_count
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    t_host = time.perf_counter()
    logical_total = passes = 0
    for i in range(args.warmup, args.warmup + args.steps):
        lg, ps = step(i)
        logical_total += lg
        passes += ps
    ev1.record(stream)
    ev1.synchronize()
    ctx.synchronize()
    host_dt = time.perf_counter() - t_host
    launches = ctx.launch_count - l0
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    barrier(dist)
    ms_max = max_over_ranks(dist, ms)
    value = logical_total * ws / (ms_max / 1e3)

    # roofline of the dominant kernel (the gate sweep: every launch in the region)
    esize = 8 if args.prec == "c64" else 16
    bytes_per_launch = 2 * (2 ** args.n) * esize
    achieved = bytes_per_launch / ((ms / 1e3) / launches) / 1e9
    peak, peak_kind = measured_peak()
    traffic = None
    if args.prec == "c64":
        traffic = TRAFFIC_BYTES_PER_AMP["plan" if plan is not None else "sweep"] * 2 ** args.n
    # the arithmetic side: the plan's algorithmic flops (an FMA counts two) against
    # the CUDA-core peak at the sampled SM clock (FP32: 128 lanes x 2 flops per SM
    # per cycle; FP64: the nominal 1.25 TFLOP/s of this part)
    compute = None
    if plan is not None:
        cost = plan.cost()
        flops = cost["flops_per_amp"] * 2 ** args.n * args.steps
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        if args.prec == "c64" and clk.get("sm_mhz"):
            fpeak, fkind = sms * 128 * 2 * clk["sm_mhz"] * 1e6, "FP32 CUDA cores at the sampled SM clock"
        else:
            fpeak, fkind = 1.25e12, "nominal FP64"
        fach = flops / (ms / 1e3)
        hbm_floor = cost["bytes_per_amp"] * 2 ** args.n / (peak * 1e9)
        compute = {"achieved": fach / 1e12, "peak": fpeak / 1e12, "unit": "TFLOP/s", "frac": fach / fpeak,
                   "peak_kind": fkind, "flops_per_amp": cost["flops_per_amp"],
                   "bytes_per_amp": cost["bytes_per_amp"],
                   "floors_ms_per_step": {"hbm": hbm_floor * 1e3, "arith": flops / args.steps / fpeak * 1e3}}

    # end to end through the public API: per step the layer's matrices go from host
    # memory into the launches, and <Z_i> for every qubit comes back to the host
    zout = np.empty(args.n, dtype=np.float64)
    e2e_steps = max(3, args.steps // 2) if plan is None else max(2, args.steps // 3)
    h2d = 0
    # a plan holds its matrix entries on the host and passes each pass's entries as
    # kernel parameters: those are the bytes that go host -> device per run
    param_bytes = 24 + (4 if args.prec == "c64" else 8) * (4096 if args.prec == "c64" else 2048) + 8
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        if plan is not None:
            ctx.check(lib.bt_plan_run(plan.h, st.h, -1))
            h2d += pstats["passes"] * param_bytes
        else:
            pk, _ = packed[i % len(packed)]
            for M, Q in pk:
                rc = lib.bt_apply_matrix(st.h, len(Q), Q.ctypes.data_as(P), M.ctypes.data_as(P), 0, None, -1)
                if rc:
                    ctx.check(rc)
                h2d += M.nbytes + Q.nbytes
        ctx.check(lib.bt_expect_z_all(st.h, 0, zout.ctypes.data_as(P)))
    e2e_dt = time.perf_counter() - t0
    e2e_dt = max_over_ranks(dist, e2e_dt)
    if plan is not None:
        e2e_logical = e2e_steps * sum(lg for _, lg in packed)
    else:
        e2e_logical = sum(packed[i % len(packed)][1] for i in range(e2e_steps))
    e2e = {"value": e2e_logical * ws / e2e_dt, "unit": METRIC, "h2d_bytes_per_step": h2d // e2e_steps,
           "d2h_bytes_per_step": zout.nbytes, "readout": "<Z_i> for all qubits each step",
           "inputs": ("compiled plan resident; per step each pass's matrix entries go to the device as kernel "
                      "parameters (the h2d bytes)") if plan is not None else
                     "each gate's matrix and qubits from host memory through bt_apply_matrix"}
    assert np.all(np.isfinite(zout))

    precision = None
    if args.fidelity and plan is not None and args.prec == "c64":
        # the same circuit in complex128 from |0...0>: infidelity of the complex64
        # state (renormalised in FP64) and the largest <Z_i> deviation
        ref = bt.Plan(args.n, "sv", "c128", ctx)
        for prog, _ in [layer_program(l, "unfused") for l in layers]:
            for m, qs in prog:
                ref.add_matrix(m, qs)
        ref.compile(True)
        s128 = bt.zero_state(args.n, "c128", 1, ctx)
        ref.run(s128)
        st.set_zero()
        plan.run(st)
        # both norms in FP64: the reference's T gates are rounded to 10 digits, so
        # even the complex128 state drifts from norm 1 (~2e-9 at this depth)
        nrm, nrm128 = np.empty(1), np.empty(1)
        ctx.check(lib.bt_norm2(st.h, 0, nrm.ctypes.data_as(P)))
        ctx.check(lib.bt_norm2(s128.h, 0, nrm128.ctypes.data_as(P)))
        z64, z128 = np.empty(args.n), np.empty(args.n)
        ctx.check(lib.bt_expect_z_all(st.h, 0, z64.ctypes.data_as(P)))
        ctx.check(lib.bt_expect_z_all(s128.h, 0, z128.ctypes.data_as(P)))
        precision = {"infidelity_vs_c128": 1 - bt.fidelity(st, s128) / (nrm[0] * nrm128[0]),
                     "max_abs_z_dev_vs_c128": float(np.abs(z64 / nrm[0] - z128 / nrm128[0]).max()),
                     "reference": "the same circuit as a complex128 fused plan from |0...0>; "
                                  "infidelity = 1 - |<psi64|psi128>|^2 / (|psi64|^2 |psi128|^2)"}
        s128.free()
        del ref

    st.free()
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(args, args.cpu_seconds)
    # the metric's serving clause on the same GPU: the configuration's stream at
    # its offered rate (>= 10^4 requests), then at 0.8x the rate it served
    serve = None
    if rank == 0 and ws == 1 and args.serve and plan is not None:
        try:
            ctx.synchronize()
            over = serve_measure(args.seed, args.rate, args.serve_requests, args.lanes)
            sus = serve_measure(args.seed + 2, 0.8 * over["circuits_per_s"], max(2000, args.serve_requests // 5),
                                args.lanes, plain=False)
            serve = {"circuits_per_s": over["circuits_per_s"], "offered_req_per_s": over["offered_req_per_s"],
                     "requests": over["requests"], "p50_ms": over["p50_ms"], "p99_ms": over["p99_ms"],
                     "plain_c128_circuits_per_s": over["plain_c128_circuits_per_s"], "vs_plain": over["vs_plain"],
                     "max_infidelity_c64": over["max_infidelity_c64"],
                     "max_rel_dev_vs_c128": over["max_rel_dev_vs_c128"],
                     "sustained": {"offered_req_per_s": sus["offered_req_per_s"],
                                   "circuits_per_s": sus["circuits_per_s"], "p50_ms": sus["p50_ms"],
                                   "p99_ms": sus["p99_ms"], "requests": sus["requests"]},
                     "traj_n_max": over["traj_n_max"], "engine": over["engine"]}
        except Exception as e:  # the headline stands without it
            serve = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.prec, "data": "synthetic",
                "config": {"workload": f"brickwork-{args.n}q-depth{args.depth}", "mode": args.mode,
                           "precision": {"c64": "complex64 (FP32 arithmetic; precision statement vs complex128 "
                                                 "in 'precision')", "c128": "complex128"}[args.prec],
                           "step": ("the whole depth-%d circuit (%d logical gates) as fused tile passes"
                                    % (args.depth, sum(lg for _, lg in packed))) if plan is not None else
                                   "one brickwork layer (logical gates: n one-qubit + CNOTs)",
                           "plan": pstats if plan is not None else None,
                           "plan_compile_s": compile_s if plan is not None else None,
                           "tuning": {k: os.environ.get(k) for k in ("BTGPU_JIT_MINB", "BTGPU_PLAN_MAX_OPS",
                                                                      "BTGPU_TILE_RB", "BTGPU_JIT_PACKED",
                                                                      "BTGPU_JIT_DIRECT", "BTGPU_JIT_PREFETCH",
                                                                      "BTGPU_PLAN_FACTOR")
                                      if os.environ.get(k)},
                           "autotune": ([{"max_ops": c[0], "tile_rb": c[1], "packed": c[2], "tile_bits": c[3],
                                          "s_per_circuit": t} for c, t in tuned] if tuned else None),
                           "passes_per_step": passes / args.steps, "global_batch": 1, "seq_len": None,
                           "parallelism": f"replicas x{ws}", "l2": "state larger than L2, no flush needed",
                           "state_bytes": (2 ** args.n) * esize},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                             "kernel": "k_fused (tile pass)" if plan is not None else "k_gate (dense sweep)",
                             "bytes_per_launch": bytes_per_launch,
                             "launches": launches, "compute": compute},
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "host_s": host_dt}
        if precision is not None:
            line["precision"] = precision
        if serve is not None:
            line["serve"] = serve
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------------ serving workload
def serve_specs(seed, clients=32, traj_max_n=14):
    """The serving mix: 70% state-vector jobs (n ~ U{8..26}), 20% trajectory
    batches of 64 (n ~ U{8..traj_max_n}; up to 14 each member fits one CTA's
    shared memory and the whole batch is one launch, above that the batch runs on
    the grouped executor), 10% density-matrix jobs (n ~ U{8..12});
    hardware-efficient ansatz of depth U{4..12}; <H> of 4n random 2-local Pauli
    terms."""
    import bluetangle_gpu.serving as S
    rng = np.random.default_rng(seed)
    out = []
    for cid in range(clients):
        kind = rng.choice(["sv", "traj", "dm"], p=[0.7, 0.2, 0.1])
        n = int(rng.integers(8, 27) if kind == "sv" else
                (rng.integers(8, traj_max_n + 1) if kind == "traj" else rng.integers(8, 13)))
        out.append(S.make_client(rng, cid, str(kind), n, int(rng.integers(4, 13))))
    return out


def serve_measure(seed, rate, total, lanes=8, native=True, traj_max_n=14, plain=True, checks=True):
    """One serving run: `total` requests with Poisson arrivals at `rate` req/s from
    the 32 clients of serve_specs; returns circuits/s, latency percentiles over all
    requests, service and queueing, and (plain=True) the plain per-call complex128
    rate on one request per client with the deviation of the served values."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.serving as S
    specs = serve_specs(seed, traj_max_n=traj_max_n)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1 / rate, total))
    owners = rng.integers(0, len(specs), total)
    reqs = [S.Request(i, int(owners[i]), rng.normal(0, 0.3, specs[owners[i]].nparams), seed=7000 + i)
            for i in range(total)]
    srv = (S.NativeServer if native else S.Server)(specs, lanes=lanes, prec="c64")

    def wait(r):
        if native:
            srv.wait(r)
        else:
            r.done.wait(600)

    try:
        # warm-up: every client admitted once, then wait for the specialised kernels
        warm = [S.Request(-1 - c.cid, c.cid, rng.normal(0, 0.3, c.nparams), seed=c.cid) for c in specs]
        for w in warm:
            srv.submit(w)
        for w in warm:
            wait(w)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 600:
            plans = ([p for p in srv.keep if isinstance(p, bt.Plan)] if native else
                     [r.plan for r, _ in srv.resident.values() if r is not None and r.plan is not None])
            if all(p.stats()["jit_passes"] == p.stats()["fused_passes"] for p in plans):
                break
            time.sleep(0.2)
        srv.completed.clear()
        start = time.perf_counter()
        for r, at in zip(reqs, arrivals):
            dt = start + at - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            srv.submit(r)
        for r in reqs:
            wait(r)
        makespan = max(r.t_done for r in reqs) - start
    finally:
        srv.close()
    errs = [r.error for r in reqs if r.error is not None]
    if errs:
        raise errs[0]
    lat = np.array([r.t_done - r.t_submit for r in reqs]) * 1e3
    svc = np.array([r.t_done - r.t_start for r in reqs]) * 1e3
    out = {"offered_req_per_s": rate, "requests": total, "circuits_per_s": total / makespan,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "mean_service_ms": float(svc.mean()),
           "mean_queue_ms": float(lat.mean() - svc.mean()),
           "mean_service_ms_by_kind": {k: float(np.mean([v for r, v in zip(reqs, svc) if specs[r.cid].kind == k]
                                                       or [0])) for k in ("sv", "traj", "dm")},
           "lane_busy_frac": float(svc.sum() / 1e3 / (lanes * makespan)),
           "mix": {k: sum(1 for c in specs if c.kind == k) for k in ("sv", "traj", "dm")},
           "traj_n_max": max([c.n for c in specs if c.kind == "traj"] or [0]),
           "engine": "bt_serve (native lanes)" if native else "python Server"}
    if not plain:
        return out
    # plain per-call complex128 path on a sample: one request per client, serially
    pctx = bt.Context(0, seed=5)
    sample = [next(r for r in reqs if r.cid == c.cid) for c in specs if any(r.cid == c.cid for r in reqs)]
    t = time.perf_counter()
    plain_vals = [S.plain_request(specs[r.cid], r.theta, r.seed, pctx, prec="c128") for r in sample]
    out["plain_c128_circuits_per_s"] = len(sample) / (time.perf_counter() - t)
    out["vs_plain"] = out["circuits_per_s"] / out["plain_c128_circuits_per_s"]

    def rel(r, v):
        return abs(r.value - v) / max(1e-12, sum(abs(x[0]) for x in specs[r.cid].terms))

    if checks:
        if native:
            # trajectory clients drew on the device (Philox keyed by the request seed):
            # check them against complex128 runs with the same draws
            dev = max([rel(r, v) for r, v in zip(sample, plain_vals) if specs[r.cid].kind != "traj"] or [0.0])
            dctx = bt.Context(0, seed=1234)  # the engine's key (NativeServer's seed)
            dev = max([dev] + [rel(r, S.program_request(specs[r.cid], r.theta, r.seed, dctx))
                               for r in sample if specs[r.cid].kind == "traj"])
            dctx.close()
        else:
            dev = max(rel(r, v) for r, v in zip(sample, plain_vals))
        out["max_rel_dev_vs_c128"] = dev
        # state infidelity of the served precision (c64 fused plan) against c128
        infid = 0.0
        for c in [c for c in specs if c.kind == "sv"][:6]:
            th = rng.normal(0, 0.3, c.nparams)
            a = bt.zero_state(c.n, "c64", ctx=pctx)
            p = bt.Plan(c.n, "sv", "c64", pctx)
            for op in S.hea_ops(c.n, c.depth, th):
                p.add(op)
            p.compile(True).run(a)
            b = bt.apply(S.hea_ops(c.n, c.depth, th), bt.zero_state(c.n, "c128", ctx=pctx))
            # 1 - |<psi64|psi128>|^2 with both states' norms in FP64
            na, nb = np.empty(1), np.empty(1)
            a.ctx.check(bt.lib().bt_norm2(a.h, 0, na.ctypes.data_as(ctypes.c_void_p)))
            b.ctx.check(bt.lib().bt_norm2(b.h, 0, nb.ctypes.data_as(ctypes.c_void_p)))
            infid = max(infid, 1 - bt.fidelity(a, b) / (na[0] * nb[0]))
            a.free()
            b.free()
        out["max_infidelity_c64"] = infid
    pctx.close()
    return out


def run_serve(args):
    """The serving stream alone: args.rate offered, max(2, steps) requests per
    client, and (--sustained) a second run at 0.8x the served rate for the latency
    of a load the engine sustains."""
    per = max(2, args.steps)
    res = serve_measure(args.seed, args.rate, per * 32, args.lanes, not args.python_server, args.traj_max_n)
    line = {"metric": "served circuits/s", "value": res["circuits_per_s"], "unit": "circuits/s", "n_gpus": 1,
            "steps": per, "warmup": 1, "ms_per_step": 1e3 / res["circuits_per_s"] * 32, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": f"serving-32clients-poisson{args.rate:g}", "requests": per * 32,
                       "lanes": args.lanes, "traj_n_max": res["traj_n_max"]},
            "serve": res, "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None}
    if args.sustained:
        line["serve_sustained"] = serve_measure(args.seed + 2, 0.8 * res["circuits_per_s"], per * 32, args.lanes,
                                                not args.python_server, args.traj_max_n, plain=False)
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ the other configurations
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return O


def _op_qubits(op):
    return [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]


def _op_ctrls(op):
    return [op.control] if op.control != -2 else []


def _events(ctx):
    import torch
    s = torch.cuda.ExternalStream(ctx.stream)
    return s, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _timed(ctx, fn, steps, warmup):
    """Runs fn(i) warmup + steps times; CUDA-event ms and host seconds of the timed steps."""
    for i in range(warmup):
        fn(i)
    ctx.synchronize()
    stream, e0, e1 = _events(ctx)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    l0 = ctx.launch_count
    e0.record(stream)
    t0 = time.perf_counter()
    for i in range(warmup, warmup + steps):
        fn(i)
    e1.record(stream)
    e1.synchronize()
    host = time.perf_counter() - t0
    return e0.elapsed_time(e1), host, ctx.launch_count - l0, clocks.stop()


def run_c1(args):
    """12-qubit complex128 brickwork of depth 20 from |0...0>, outputs the state,
    <Z_i> for every qubit and 10^4 shots (the configuration the reference runs as
    is on CPU).  A step is one circuit: reset, the circuit as a compiled plan,
    <Z_i> and the shots returned to the host; e2e adds the state download."""
    import bluetangle_gpu as bt
    from bluetangle_gpu.circuits import brickwork
    n, depth, shots = 12, 20, 10_000
    ctx = bt.Context(0, seed=args.seed)
    bt.Context._default = ctx
    ops = brickwork(n, depth, np.random.default_rng(args.seed))
    plan = bt.Plan(n, "sv", "c128", ctx)
    for op in ops:
        plan.add(op)
    plan.compile(True)
    st = bt.zero_state(n, "c128", ctx=ctx)
    # a 12-qubit state fits one tile: the autotuner weighs smaller tiles (more CTAs
    # per pass) against more passes
    tuned = plan.autotune(st, reps=5)
    out = {}

    def circuit(i, download=False):
        st.set_zero()
        plan.run(st)
        out["z"] = bt.expect(st, "Z")
        out["s"] = bt.sample(st, shots, seed=i)
        if download:
            out["psi"] = st.to_numpy()

    ms, host, launches, clk = _timed(ctx, circuit, args.steps, args.warmup)
    t0 = time.perf_counter()
    for i in range(args.steps):
        circuit(i, True)
    e2e_s = time.perf_counter() - t0
    # parity against the oracle on the same circuit
    O = _oracle()
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    for op in ops:
        psi = O.apply_k(psi, op.mat, _op_qubits(op), _op_ctrls(op))
    circuit(0, True)
    dev = float(np.abs(out["psi"] - psi).max())
    p = np.abs(psi) ** 2
    bits = (np.arange(2 ** n)[:, None] >> (n - np.arange(1, n + 1))[None, :]) & 1
    zref = (p[:, None] * (1 - 2 * bits)).sum(0)
    zdev = float(np.abs(np.asarray(out["z"]) - zref).max())
    # CPU: the oracle runs the same circuit with the same outputs, single thread
    cpu_n = 0
    t0 = time.perf_counter()
    urng = np.random.default_rng(1)
    while time.perf_counter() - t0 < min(args.cpu_seconds, 10.0) or cpu_n < 3:
        q = np.zeros(2 ** n, complex)
        q[0] = 1
        for op in ops:
            q = O.apply_k(q, op.mat, _op_qubits(op), _op_ctrls(op))
        pq = np.abs(q) ** 2
        _ = (pq[:, None] * (1 - 2 * bits)).sum(0)
        _ = O.sample(q, urng.random(shots))
        cpu_n += 1
    cpu_rate = cpu_n / (time.perf_counter() - t0)
    value = args.steps / (ms / 1e3)
    line = {"metric": "circuits/s", "value": value, "unit": "circuits/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "brickwork-12q-c128-depth20+Z+1e4shots", "gates": len(ops),
                       "plan": plan.stats(), "l2": "state (64 KiB) is L2/shared-memory resident",
                       "autotune": [{"config": list(c), "ms_per_circuit_plan_only": t * 1e3} for c, t in tuned]},
            "parity": {"max_abs_state_vs_oracle": dev, "max_abs_z_vs_oracle": zdev},
            "cpu_baseline": {"value": cpu_rate, "unit": "circuits/s", "cores": 1, "kind": "port",
                             "sample": f"{cpu_n} circuits through the oracle (same outputs), 1 thread"},
            "e2e": {"value": args.steps / e2e_s, "unit": "circuits/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": (2 ** n) * 16 + n * 8 + shots * 8},
            "gpu_launches": launches, "launches_per_circuit": launches / args.steps, "clocks": clk,
            "host_s": host}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_c2(args):
    """10-qubit density matrix, brickwork of depth 16 with depolarizing and
    amplitude-damping channels after every gate and a final 2% bit flip per qubit;
    outputs rho, <Z_i> and <Z_i Z_i+1>.  value: the chosen form (complex64, the
    circuit compiled into fused passes with every Kraus sum inside the passes);
    beside it the plain complex128 op-by-op path and the complex128 plan."""
    import bluetangle_gpu as bt
    from bluetangle_gpu.circuits import noisy_brickwork_dm
    n, depth = 10, 16
    ctx = bt.Context(0, seed=args.seed)
    bt.Context._default = ctx
    ops = noisy_brickwork_dm(n, depth, np.random.default_rng(args.seed))
    ops += [bt.OpQC("bit_flip", 0.02, q) for q in range(1, n + 1)]
    ngate = sum(1 for op in ops if not isinstance(op, bt.OpQC))
    plans = {}
    for prec in ("c64", "c128"):
        p = bt.Plan(n, "dm", prec, ctx)
        for op in ops:
            p.add(op)
        plans[prec] = p.compile(True)
    rhos = {prec: bt.zero_rho(n, prec, ctx=ctx) for prec in ("c64", "c128")}
    res = {}

    def outputs(r):
        z = bt.expect(r, "Z")
        zz = [bt.correlation(r, "Z,Z", [q, q + 1]) for q in range(1, n)]
        return np.asarray(z), np.asarray(zz)

    def chosen(i, prec="c64"):
        r = rhos[prec]
        r.set_zero()
        plans[prec].run(r)
        res[prec] = outputs(r)

    ms64, host64, launches, clk = _timed(ctx, chosen, args.steps, args.warmup)
    ms128, _, _, _ = _timed(ctx, lambda i: chosen(i, "c128"), args.steps, args.warmup)
    # the plain per-call complex128 path: one call per gate and per channel
    plain = bt.zero_rho(n, "c128", ctx=ctx)

    def plain_run(i):
        plain.set_zero()
        bt.apply(ops, plain)
        res["plain"] = outputs(plain)

    k_plain = max(2, args.steps // 3)
    msp, _, _, _ = _timed(ctx, plain_run, k_plain, 1)
    r64, r128, rp = rhos["c64"].to_numpy(), rhos["c128"].to_numpy(), plain.to_numpy()
    # parity: the oracle's Kraus-sum restatement on the same circuit (complex128)
    O = _oracle()
    rho = np.zeros((2 ** n, 2 ** n), complex)
    rho[0, 0] = 1
    t0 = time.perf_counter()
    for op in ops:
        if isinstance(op, bt.OpQC):
            qs = _op_qubits(op)
            rho = O.dm_channel(rho, op.kraus, qs[0], qs[1] if len(qs) == 2 else -1)
        else:
            rho = O.dm_gate(rho, op.mat, _op_qubits(op), _op_ctrls(op))
    cpu_s = time.perf_counter() - t0
    line = {"metric": "circuits/s", "value": args.steps / (ms64 / 1e3), "unit": "circuits/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms64 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": "noisy-brickwork-dm-10q-depth16", "gates": ngate,
                       "channels": len(ops) - ngate, "plan_c64": plans["c64"].stats(),
                       "l2": "rho (8 MiB c64 / 16 MiB c128) is L2-resident"},
            "c128_plan_circuits_per_s": args.steps / (ms128 / 1e3),
            "plain_c128_circuits_per_s": k_plain / (msp / 1e3),
            "vs_plain": (args.steps / (ms64 / 1e3)) / (k_plain / (msp / 1e3)),
            "errors": {"c64_vs_c128_max_abs_rho": float(np.abs(r64 - r128).max()),
                       "c64_vs_c128_max_abs_z": float(np.abs(res["c64"][0] - res["c128"][0]).max()),
                       "c64_vs_c128_max_abs_zz": float(np.abs(res["c64"][1] - res["c128"][1]).max()),
                       "c128_plan_vs_oracle_max_abs_rho": float(np.abs(r128 - rho).max()),
                       "plain_c128_vs_oracle_max_abs_rho": float(np.abs(rp - rho).max())},
            "cpu_baseline": {"value": 1 / cpu_s, "unit": "circuits/s", "cores": O.num_threads(), "kind": "port",
                             "sample": f"one circuit through the oracle (complex128 Kraus sums) in {cpu_s:.1f} s"},
            "gpu_launches": launches, "clocks": clk}
    print(json.dumps(line), flush=True)
    ctx.close()


def _c3_noise_after(op, p1=1e-3, p2=1e-2, gamma=5e-3):
    from bluetangle_gpu.ops import OpQC
    if op.q == 1:
        return [OpQC("depolarizing", p1, op.qubit), OpQC("amplitude_damping", gamma, op.qubit)]
    return [OpQC("depolarizing", p2, op.qubit, op.target_qubit), OpQC("amplitude_damping", gamma, op.qubit),
            OpQC("amplitude_damping", gamma, op.target_qubit)]


def run_c3(args):
    """4096 Monte-Carlo trajectories of a 20-qubit open-chain TFIM (J=1, h_i ~
    U[0.5,1.5], dt=0.05; RZZ on ascending pairs then RX), depolarizing and
    amplitude damping after every gate sampled per trajectory, a Z measurement of
    each qubit with probability 0.1 per step; beside them 64 Pauli-twirled
    instances at ZNE scales 1, 3, 5 (CNOT.RZ.CNOT form, uneven depth, 192 members
    with depolarizing noise after every gate including the repetitions).  A step is
    one Trotter step of every member (40 make the circuit); complex64, on-device
    Philox draws."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    from bluetangle_gpu.noise import NoiseModel
    n, B, dt = args.c3_n, args.c3_members, 0.05
    ctx = bt.Context(0, seed=args.seed)
    bt.Context._default = ctx
    h = np.random.default_rng(args.seed).uniform(0.5, 1.5, n)
    step_ops = []
    for q in range(1, n):
        op = bt.Op(f"RZZ({2 * dt!r})", q, q + 1)
        step_ops += [op] + _c3_noise_after(op)
    for q in range(1, n + 1):
        op = bt.Op(f"RX({float(2 * h[q - 1] * dt)!r})", q)
        step_ops += [op] + _c3_noise_after(op)
    # the shared-payload slots of one step (every member the same ops), then the
    # measurement slots with this step's per-member masks
    base = []
    for op in step_ops:
        (kind, payload), = T._op_slots(op, False)
        base.append(T.Slot(kind, [payload] * B))
    mrng = np.random.default_rng(args.seed + 7)
    meas_payload = [("MZ", q) for q in range(1, n + 1)]

    def step_slots():
        sl = list(base)
        for q in range(1, n + 1):
            mask = mrng.random(B) < 0.1
            sl.append(T.Slot("measure", [meas_payload[q - 1] if m else None for m in mask]))
        return sl

    # twirl / ZNE copies: CNOT.RZ.CNOT form, NoiseModel depolarizing after every gate
    ncopy = args.c3_twirl * 3
    copy_step = []
    for q in range(1, n):
        copy_step += [bt.Op("CNOT", q, q + 1), bt.Op(f"RZ({2 * dt!r})", q + 1), bt.Op("CNOT", q, q + 1)]
    copy_step += [bt.Op(f"RX({float(2 * h[q - 1] * dt)!r})", q) for q in range(1, n + 1)]
    noise = NoiseModel(bt.Noise1("depolarizing", 1e-3), bt.Noise2("depolarizing", 1e-2))
    frame_rng = np.random.default_rng(args.seed + 11)
    zne = [k % 3 for k in range(ncopy)]

    # trajectories and copies are one batch of B + ncopy members: each step's
    # slots hold the trajectories' ops (members [0, B)) and then the copies' ops
    # (members [B, B + ncopy)), the other group idle there
    tot = B + ncopy
    groups = []
    for _ in range(args.warmup + args.steps):
        g = [(step_slots(), B)]
        if ncopy:
            mo = T.member_programs([copy_step], n, ncopy, zne_ids=zne, twirl=True, frame_rng=frame_rng,
                                   measure_prob=0.1, measure_rng=mrng)
            g.append((T.build_slots(mo, noise), ncopy))
        groups.append(g)
    pre = [T.concat_slots(*g) for g in groups]

    def member_ops(slots):
        return sum(sum(1 for it in s.items if it is not None) for s in slots)

    progs = None
    if args.c3_engine == "program":
        # each step's slots compiled into one program over the whole batch (grouped
        # executor: the members exceed shared memory), built before the timed region
        st = bt.zero_state(n, "c64", tot, ctx)
        progs = [T.compile_program(sl, n, tot, "c64", ctx)[0].prepare() for sl in pre]
    else:
        # the lock-step engine launches over a whole batch per op: the trajectories
        # and the copies keep a batch each
        sts = [bt.zero_state(n, "c64", b, ctx) for _, b in groups[0]]
        st = sts[0]

    def step(i):
        if progs is not None:
            progs[i].run(st, seed=1000 + i, records=False)
        else:
            for (sl, _), s_ in zip(groups[i], sts):
                T.run_slots(s_, sl, records=False)

    ms, host, launches, clk = _timed(ctx, step, args.steps, args.warmup)
    timed = range(args.warmup, args.warmup + args.steps)
    timed_ops = sum(member_ops(pre[i]) for i in timed)
    # algorithmic HBM bytes per step: per op pass (slots engine) a gate reads and
    # writes every member it acts on, a channel adds a reduction read unless it is
    # a unitary mixture, a measurement reads once and rewrites (collapse); the
    # grouped executor moves, per group of ops within two qubits, a reduction read
    # (when a decision needs one) and one read and write of each acting member
    if progs is not None:
        bytes_step = float(np.mean([T.grouped_bytes(pre[i], n, tot, "c64") for i in timed]))
    else:
        S1 = (2 ** n) * 8

        def slot_bytes(sl):
            k = sum(1 for it in sl.items if it is not None) * S1
            if sl.kind == "gate":
                return 2 * k
            live = next(it for it in sl.items if it is not None)
            if sl.kind == "channel":
                return 2 * k + (0 if T._unitary_mix(live[0]) else k)
            return 3 * k
        bytes_step = float(np.mean([sum(slot_bytes(sl) for sl in pre[i]) for i in timed]))
    zs = bt.expect(st, "Z", member=-1)
    assert np.all(np.isfinite(zs))
    # complex128 check: 256 trajectories through five Trotter steps as the same
    # programs in complex64 and complex128 with the same explicit draws (host
    # uniforms): how many members took the same branches and outcomes, and how far
    # their final states and <Z_i> are apart
    prec_check = None
    if progs is not None:
        st.free()
        K2, S2 = min(256, B), 5
        sub = []
        for i in range(S2):  # the step's gate and channel slots, then its measurement slots
            sl = [T.Slot(b.kind, [b.items[0]] * K2) for b in base]
            mr = np.random.default_rng(900 + i)
            for q in range(1, n + 1):
                mask = mr.random(K2) < 0.1
                sl.append(T.Slot("measure", [meas_payload[q - 1] if x else None for x in mask]))
            sub.append(sl)
        finals, recs = {}, {}
        for prec in ("c64", "c128"):
            s2 = bt.zero_state(n, prec, K2, ctx)
            rr = []
            for i in range(S2):
                pr, _ = T.compile_program(sub[i], n, K2, prec, ctx, unitary_mix=False)
                rr.append(pr.run(s2, rng=np.random.default_rng(4000 + i)))
            finals[prec] = s2
            recs[prec] = rr
        same = np.array([all(recs["c64"][i][m] == recs["c128"][i][m] for i in range(S2)) for m in range(K2)])
        dz = np.abs(bt.expect(finals["c64"], "Z", member=-1)[same] - bt.expect(finals["c128"], "Z", member=-1)[same])
        dmax = 0.0
        for m in np.nonzero(same)[0][:16]:
            dmax = max(dmax, float(np.abs(finals["c64"].to_numpy(int(m)) - finals["c128"].to_numpy(int(m))).max()))
        prec_check = {"trajectories": K2, "steps": S2, "same_decisions": int(sum(same)),
                      "max_abs_z_dev": float(dz.max()) if dz.size else None,
                      "max_abs_amp_dev_16_members": dmax,
                      "draws": "explicit host uniforms shared by both precisions"}
        for v in finals.values():
            v.free()
    cpu = None
    if not args.no_cpu:
        # CPU: the oracle on a sample of trajectories (one step each, complex128)
        O = _oracle()
        cpu_ops = 0
        t0 = time.perf_counter()
        urng = np.random.default_rng(3)
        traj = 0
        while time.perf_counter() - t0 < min(args.cpu_seconds, 15.0) or traj < 1:
            psi = np.zeros(2 ** n, complex)
            psi[0] = 1
            for op in step_ops:
                if isinstance(op, bt.OpQC):
                    qs = _op_qubits(op)
                    psi, _, _ = O.channel_traj(psi, op.kraus, qs[0], qs[1] if len(qs) == 2 else -1,
                                               u=urng.random())
                else:
                    psi = O.apply_k(psi, op.mat, _op_qubits(op), [])
                cpu_ops += 1
            for q in range(1, n + 1):
                if urng.random() < 0.1:
                    psi, _, _ = O.born_measure_z(psi, q, u=urng.random())
                    cpu_ops += 1
            traj += 1
        cpu = {"value": cpu_ops / (time.perf_counter() - t0), "unit": "member-ops/s", "cores": 1, "kind": "port",
               "sample": f"{traj} trajectory-steps ({cpu_ops} ops) of the oracle at {n} qubits, 1 thread"}
    value = timed_ops / (ms / 1e3)
    achieved = bytes_step * args.steps / (ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    line = {"metric": "trajectory op-apps/s", "value": value, "unit": "member-ops/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": f"tfim-{n}q-{B}traj+{ncopy}twirl/zne-copies", "members": tot,
                       "launch": ("trajectories and copies in one program per step (member ranges)"
                                  if progs is not None else "trajectories and copies as two batches"),
                       "step": "one Trotter step of every member (40 make the circuit)",
                       "ops_per_member_step": len(step_ops), "l2": f"states ({(B + ncopy) * 2 ** n * 8 / 2**30:.1f} GiB) larger than L2",
                       "engine": ("programs, grouped executor (ops within two qubits decided from one reduced "
                                  "matrix and applied in one pass)") if progs is not None else
                                 "lock-step slots (one launch sequence per op over the batch)"},
            "trajectory_steps_per_s": (B + ncopy) * args.steps / (ms / 1e3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "bytes_per_step": bytes_step,
                         "note": "algorithmic bytes of the whole batch (trajectories and copies)"},
            "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk, "host_s": host,
            "precision_vs_c128": prec_check}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_vqa(args):
    """Parameter-shift gradients of a hardware-efficient ansatz (parametrised RY, RZ
    on every qubit, CNOT ladder) for <H> of 3n random 2-local Pauli terms: the
    2P + 1 shifted evaluations of loss_and_grad_paramshift as one batch.  A step is
    one gradient; 12 qubits depth 6 (P = 144: one CTA per evaluation) and 20 qubits
    depth 4 (P = 160: fused plan, angles rewritten per evaluation)."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.vqa as V
    from bluetangle_gpu.serving import random_terms

    def ry(t):
        c, s = math.cos(t / 2), math.sin(t / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)

    def rz(t):
        return np.array([[np.exp(-0.5j * t), 0], [0, np.exp(0.5j * t)]], dtype=np.complex128)

    def hea(n, depth):
        ops = []
        for _ in range(depth):
            for q in range(1, n + 1):
                ops += [bt.Op("RY", ry, q), bt.Op("RZ", rz, q)]
            ops += [bt.Op("CNOT", q, q + 1) for q in range(1, n)]
        return ops

    ctx = bt.Context(0, seed=args.seed)
    bt.Context._default = ctx
    out = {}
    for n, depth in ((12, 6), (20, 4)):
        ops = hea(n, depth)
        P = sum(V.arg_counts(ops))
        terms = random_terms(np.random.default_rng(args.seed + n), n, 3 * n)
        rng = np.random.default_rng(args.seed)
        ps = [rng.uniform(0, 2 * np.pi, P) for _ in range(args.warmup + args.steps)]
        res = {}

        def grad(i):
            res[i] = V.loss_and_grad_paramshift(ps[i], ops, n, terms, prec=args.prec)

        ms, host, launches, clk = _timed(ctx, grad, args.steps, args.warmup)
        # plain per-call path: every evaluation gate by gate (engine.apply) + <H>, a sample
        k = 8
        t0 = time.perf_counter()
        for j in range(k):
            st = V.variational_apply(ps[0], ops, n, prec="c128", ctx=ctx)
            V._expect_members(st, terms)
            st.free()
        plain_eval = k / (time.perf_counter() - t0)
        out[f"{n}q_depth{depth}"] = {"params": P, "evaluations_per_gradient": 2 * P + 1,
                                     "gradients_per_s": args.steps / (ms / 1e3),
                                     "evaluations_per_s": args.steps * (2 * P + 1) / (ms / 1e3),
                                     "executor": "program (one CTA per evaluation)" if n <= 14 else
                                                 "fused plan (angles rewritten per evaluation)",
                                     "plain_c128_evaluations_per_s": plain_eval, "gpu_launches": launches,
                                     "clocks": clk}
        if not args.no_cpu:
            O = _oracle()
            t0 = time.perf_counter()
            cnt = 0
            counts = V.arg_counts(ops)
            while time.perf_counter() - t0 < min(args.cpu_seconds, 8.0) or cnt < 2:
                psi = np.zeros(2 ** n, complex)
                psi[0] = 1
                for op, mat in V._bound(ops, counts, ps[0]):
                    qs, cs = V._qubits(op)
                    psi = O.apply_k(psi, op.mat if mat is None else mat, qs, cs)
                _ = sum(c * O.expect_pauli_sv(psi, x, z) for c, x, z in terms)
                cnt += 1
            rate = cnt / (time.perf_counter() - t0)
            out[f"{n}q_depth{depth}"]["cpu_baseline"] = {
                "value": rate / (2 * P + 1), "unit": "gradients/s", "cores": 1, "kind": "port",
                "sample": f"{cnt} sequential evaluations through the oracle (the reference's loop), 1 thread"}
    head = out["12q_depth6"]
    line = {"metric": "parameter-shift gradients/s", "value": head["gradients_per_s"], "unit": "gradients/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.prec, "data": "synthetic",
            "config": {"workload": "paramshift-hea-12q-depth6 (+20q-depth4)", "cases": out}}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_tc(args):
    """Tensor-core fused passes (every register phase a dense 32 x 32 block on
    tcgen05, three TF32 products) against the scalar fused passes, complex64, on
    the random brickwork and on a brickwork of Haar-random two-qubit unitaries,
    both depth 30 at args.n qubits (default 30 here).  A step is one circuit.
    Reports gate-apps/s of both forms, the tensor work per circuit against the
    TF32 throughput measured on this GPU (bt_tc_tf32_peak), and the HBM fraction."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    n = args.n if args.n != 33 else 30
    ctx = bt.Context(0, seed=args.seed)
    bt.Context._default = ctx
    P = ctypes.c_void_p
    peak_tf = ctypes.c_double(0)
    ctx.check(bt.lib().bt_tc_tf32_peak(ctx.h, 4000, ctypes.byref(peak_tf)))
    st = bt.zero_state(n, "c64", 1, ctx)
    hbm, hkind = measured_peak()
    cases = {}
    for kind in ("brickwork", "su4"):
        rng = np.random.default_rng(args.seed)
        ops = C.brickwork(n, args.depth, rng) if kind == "brickwork" else C.su4_brickwork(n, args.depth, rng)
        for tc in (False, True):
            plan = bt.Plan(n, "sv", "c64", ctx)
            for op in ops:
                plan.add(op)
            plan.compile(tensor_cores=tc)
            ms, host, launches, clk = _timed(ctx, lambda i: plan.run(st), args.steps, args.warmup)
            stt = plan.stats()
            per = ms / args.steps
            case = {"ms_per_circuit": per, "gate_apps_per_s": len(ops) / (per / 1e3), "gates": len(ops),
                    "passes": stt["passes"], "phases": stt["phases"],
                    "hbm_frac": stt["passes"] * 2 * (2 ** n) * 8 / (per / 1e3) / (hbm * 1e9), "clocks": clk,
                    "gpu_launches": launches}
            if tc:
                # 48 MMAs of 128 x 64 x 8 per phase of a 2^13-amplitude tile
                tiles = 2 ** (n - 13)
                flops = stt["phases"] * tiles * 48 * 2 * 128 * 64 * 8
                case["tensor_tflops"] = flops / (per / 1e3) / 1e12
                case["tensor_frac_of_tf32_peak"] = case["tensor_tflops"] / peak_tf.value
            cases[f"{kind}_{'tc' if tc else 'scalar'}"] = case
    for kind in ("brickwork", "su4"):
        cases[f"{kind}_tc_speedup"] = cases[f"{kind}_scalar"]["ms_per_circuit"] / cases[f"{kind}_tc"]["ms_per_circuit"]
    head = cases["su4_tc"]
    line = {"metric": "gate-apps/s", "value": head["gate_apps_per_s"], "unit": "gate-apps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_circuit"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64 (3xTF32 tensor cores)",
            "data": "synthetic",
            "config": {"workload": f"su4-brickwork-{n}q-depth{args.depth} (tensor-core plan; + brickwork)",
                       "l2": "state larger than L2, no flush needed", "cases": cases},
            "tf32_peak_tflops_measured": peak_tf.value, "hbm_peak_gbs": hbm, "hbm_peak_kind": hkind,
            "gpu_launches": head["gpu_launches"], "clocks": head["clocks"]}
    print(json.dumps(line), flush=True)
    st.free()
    ctx.close()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "serve":
        run_serve(a)
    elif a.workload in ("c1", "c2", "c3", "vqa", "tc"):
        {"c1": run_c1, "c2": run_c2, "c3": run_c3, "vqa": run_vqa, "tc": run_tc}[a.workload](a)
    else:
        run_ours(a)
