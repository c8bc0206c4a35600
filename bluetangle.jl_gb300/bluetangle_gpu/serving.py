"""Serving loop: continuous batching of variational circuit jobs on one GPU.

A client is a VQE/Trotter-style loop of the reference (variational_apply +
expect(state, H), BlueTangle.jl src/vqa.jl:420-456, src/func.jl:100): a fixed
circuit structure (a hardware-efficient ansatz, src/vqa.jl:302-314) evaluated
again and again at new parameters, each time returning <H> of a Pauli-sum
Hamiltonian.  The server

  * admits clients by HBM footprint: a client's state (and plan) stay resident
    between its requests; when the budget is exhausted, idle clients are evicted
    oldest-first and admission waits until memory frees up;
  * compiles each client's circuit once into a fused plan (kernels specialised
    per pass structure); a request only rewrites the angles in place;
  * runs requests on `lanes` worker threads, each with its own context and CUDA
    stream, so requests that arrive while others are on the GPU start as soon as
    a lane is free and their kernels overlap on the device (a small circuit is a
    single fused launch);
  * serves each client's requests in arrival order (they share its state) and
    records per-request latency (submit to result) for p50/p99.

Job kinds: "sv" (state vector, one fused plan), "traj" (a batch of Monte-Carlo
trajectories with depolarizing and amplitude-damping noise after every gate,
<H> averaged over members), "dm" (density matrix with the same noise as Kraus
sums, one fused plan).
"""
import ctypes
import heapq
import math
import threading
import time
from collections import deque

import numpy as np

from . import _lib as L
from .engine import Context, GPUDensity, GPUState, Plan, _cm, _ptr
from .gates import gates
from .noise import noise_model
from .ops import Op, OpQC

__all__ = ["ClientSpec", "make_client", "Server", "NativeServer", "plain_request", "hea_ops"]


def _ry(t):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def _rz(t):
    return np.array([[np.exp(-0.5j * t), 0], [0, np.exp(0.5j * t)]], dtype=np.complex128)


CNOT = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)


def _hea_mats(theta):
    """RY(theta[0]), RZ(theta[1]), RY(theta[2]), ... as column-major 2x2 complex128
    matrices back to back (the ABI's layout), built in one vectorised step."""
    th = np.asarray(theta, dtype=np.float64)
    out = np.zeros((len(th), 4), dtype=np.complex128)
    ev, od = th[0::2], th[1::2]
    c, s = np.cos(ev / 2), np.sin(ev / 2)
    out[0::2, 0], out[0::2, 1], out[0::2, 2], out[0::2, 3] = c, s, -s, c
    out[1::2, 0], out[1::2, 3] = np.exp(-0.5j * od), np.exp(0.5j * od)
    return out.ravel()


class ClientSpec:
    """kind, n, depth, Hamiltonian terms (coef, xmask, zmask) and trajectory count."""

    def __init__(self, cid, kind, n, depth, terms, ntraj=64, p1=1e-3, p2=1e-2, gamma=5e-3):
        self.cid, self.kind, self.n, self.depth, self.terms = cid, kind, n, depth, terms
        self.ntraj, self.p1, self.p2, self.gamma = ntraj, p1, p2, gamma

    @property
    def nparams(self):
        return 2 * self.n * self.depth

    def footprint(self, prec, pack=1):
        """HBM bytes of the client's resident state; pack: members of a packed
        state-vector client (NativeServer, n small enough for one CTA)."""
        es = 8 if prec == "c64" else 16
        if self.kind == "dm":
            return (4 ** self.n) * es
        if self.kind == "traj":
            return self.ntraj * (2 ** self.n) * es
        from .trajectories import SHARED_MAX_N
        return (pack if pack > 1 and self.n <= SHARED_MAX_N[prec] else 1) * (2 ** self.n) * es


def random_terms(rng, n, count):
    """count random 2-local Pauli terms on any pair of qubits with N(0,1) coefficients."""
    terms = []
    for _ in range(count):
        a, b = rng.choice(np.arange(1, n + 1), size=2, replace=False)
        x = z = 0
        for q in (a, b):
            p = "XYZ"[rng.integers(0, 3)]
            bit = 1 << (n - int(q))
            if p in "XY":
                x |= bit
            if p in "ZY":
                z |= bit
        terms.append((float(rng.normal()), x, z))
    return terms


def make_client(rng, cid, kind, n, depth):
    return ClientSpec(cid, kind, n, depth, random_terms(rng, n, 4 * n))


def hea_ops(n, depth, theta):
    """The ansatz as reference ops: per layer RY, RZ on every qubit, then a CNOT ladder."""
    ops, i = [], 0
    for _ in range(depth):
        for q in range(1, n + 1):
            ops.append(Op("RY", _ry(theta[i]), q))
            ops.append(Op("RZ", _rz(theta[i + 1]), q))
            i += 2
        for q in range(1, n):
            ops.append(Op("CNOT", q, q + 1))
    return ops


def _noisy(spec, ops):
    """config-2 style noise after every gate: depolarizing (p1 / p2, the two-qubit
    one a 16-term kron channel) and amplitude damping on each touched qubit."""
    out = []
    for op in ops:
        out.append(op)
        if op.q == 1:
            out += [OpQC("depolarizing", spec.p1, op.qubit), OpQC("amplitude_damping", spec.gamma, op.qubit)]
        else:
            out += [OpQC("depolarizing", spec.p2, op.qubit, op.target_qubit),
                    OpQC("amplitude_damping", spec.gamma, op.qubit),
                    OpQC("amplitude_damping", spec.gamma, op.target_qubit)]
    return out


def _expect_h(st, terms, member=-1):
    """<H> per member divided by the member's norm (trace), accumulated in FP64:
    removes the complex64 norm drift of long circuits; averaged over members."""
    lib = L.lib()
    xs = np.ascontiguousarray([t[1] for t in terms], dtype=np.uint64)
    zs = np.ascontiguousarray([t[2] for t in terms], dtype=np.uint64)
    cs = np.ascontiguousarray([t[0] for t in terms], dtype=np.float64)
    rows = st.batch if member == -1 else 1
    out = np.empty(rows * len(terms), dtype=np.float64)
    st.ctx.check(lib.bt_expect_pauli(st.h, len(terms), _ptr(xs), _ptr(zs), _ptr(cs), member, _ptr(out)))
    nrm = np.empty(rows, dtype=np.float64)
    st.ctx.check(lib.bt_norm2(st.h, member, _ptr(nrm)))
    return float((out.reshape(rows, len(terms)).sum(axis=1) / nrm).mean())


class _Resident:
    """A client's resident GPU objects (on one lane's context)."""

    def __init__(self, spec, ctx, prec, tiered=True):
        self.spec, self.ctx, self.prec = spec, ctx, prec
        n = spec.n
        theta0 = np.full(spec.nparams, 0.1)
        self.pidx = []  # add indices of the parametrised gates, in theta order
        self.plan = None
        if spec.kind in ("sv", "dm"):
            dm = spec.kind == "dm"
            self.state = (GPUDensity if dm else GPUState)(n, prec, 1, ctx)
            self.plan = Plan(n, spec.kind, prec, ctx)
            ops = hea_ops(n, spec.depth, theta0)
            for i, op in enumerate(_noisy(spec, ops) if dm else ops):
                self.plan.add(op)
                if op.name in ("RY", "RZ"):
                    self.pidx.append(i)
            self.plan.set_variable(self.pidx).compile(True, tiered=tiered)
        else:
            self.state = GPUState(n, prec, spec.ntraj, ctx)
            self.program = None
            from . import trajectories as T
            ops = _noisy(spec, hea_ops(n, spec.depth, theta0))
            slots = T.build_slots(T.member_programs([ops], n, spec.ntraj))
            if T.program_supported(slots, n, prec):
                # one slot per op (no ZNE, no twirl): slot i is op i
                self.program, gate_ops = T.compile_program(slots, n, spec.ntraj, prec, ctx)
                self.pidx = [gate_ops[i] for i, op in enumerate(ops) if op.name in ("RY", "RZ")]
        self.last_used = time.perf_counter()

    def free(self):
        self.state.free()
        self.plan = None
        self.program = None

    def run(self, theta, seed):
        spec = self.spec
        self.state.set_zero()
        if spec.kind in ("sv", "dm"):
            ups = []
            for j, ai in enumerate(self.pidx):
                ups.append((ai, _ry(theta[j]) if j % 2 == 0 else _rz(theta[j])))
            self.plan.set_matrices(ups).run(self.state)
            return _expect_h(self.state, spec.terms)
        if self.program is not None:
            for j, oi in enumerate(self.pidx):
                self.program.set_gate(oi, _ry(theta[j]) if j % 2 == 0 else _rz(theta[j]))
            # draws from the request's seed, in the order the plain path consumes them
            self.program.run(self.state, rng=np.random.default_rng(seed), records=False)
            return _expect_h(self.state, spec.terms, -1)
        from .trajectories import run_trajectories
        steps = [_noisy(spec, hea_ops(spec.n, spec.depth, theta))]
        run_trajectories(steps, spec.n, spec.ntraj, prec=self.prec, rng=np.random.default_rng(seed),
                         state=self.state)
        return _expect_h(self.state, spec.terms, -1)


class Request:
    def __init__(self, rid, cid, theta, seed):
        self.rid, self.cid, self.theta, self.seed = rid, cid, theta, seed
        self.t_submit = None
        self.t_start = None
        self.t_done = None
        self.value = None
        self.error = None
        self.done = threading.Event()


class Server:
    def __init__(self, specs, lanes=8, prec="c64", hbm_budget=None, device=0, seed=1234, tiered=True):
        self.specs = {s.cid: s for s in specs}
        self.prec = prec
        self.tiered = tiered
        self.lanes = [Context(device, seed=seed + i) for i in range(lanes)]
        self.budget = hbm_budget if hbm_budget is not None else 200 * 2 ** 30
        self.used = 0
        self.resident = {}  # cid -> (_Resident, lane index)
        self.queues = {s.cid: deque() for s in specs}
        self.busy = set()
        self.cv = threading.Condition()
        self.stop = False
        self.completed = []
        self.threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(lanes)]
        for t in self.threads:
            t.start()

    # ---------------------------------------------------------------- API
    def submit(self, req):
        with self.cv:
            req.t_submit = time.perf_counter()
            self.queues[req.cid].append(req)
            self.cv.notify_all()
        return req

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        for r, _ in list(self.resident.values()):
            r.free()
        self.resident.clear()
        for c in self.lanes:
            c.close()

    def latencies(self):
        return np.array([r.t_done - r.t_submit for r in self.completed])

    # ---------------------------------------------------------------- scheduling
    def _pick(self, lane):
        """Oldest pending request of a client that is idle and admissible."""
        best = None
        for cid, q in self.queues.items():
            if not q or cid in self.busy:
                continue
            if cid in self.resident and self.resident[cid][1] != lane:
                continue  # resident on another lane's context
            if best is None or q[0].t_submit < self.queues[best][0].t_submit:
                best = cid
        return best

    def _admit(self, cid, lane):
        spec = self.specs[cid]
        need = spec.footprint(self.prec)
        if need > self.budget:
            raise MemoryError(f"client {cid} needs {need} bytes, more than the HBM budget")
        while self.used + need > self.budget:
            idle = [(r.last_used, c) for c, (r, _) in self.resident.items() if c not in self.busy]
            if not idle:
                return False
            _, victim = min(idle)
            r, _ = self.resident.pop(victim)
            self.used -= r.spec.footprint(self.prec)
            r.free()
        self.used += need
        self.resident[cid] = (None, lane)  # reserved; built outside the lock
        return True

    def _worker(self, lane):
        ctx = self.lanes[lane]
        while True:
            with self.cv:
                while True:
                    if self.stop:
                        return
                    cid = self._pick(lane)
                    if cid is not None and (cid in self.resident or self._admit(cid, lane)):
                        break
                    self.cv.wait(0.01)
                self.busy.add(cid)
                req = self.queues[cid].popleft()
            try:
                res = self.resident[cid][0]
                if res is None:
                    res = _Resident(self.specs[cid], ctx, self.prec, self.tiered)
                    self.resident[cid] = (res, lane)
                req.t_start = time.perf_counter()
                req.value = res.run(req.theta, req.seed)
                res.last_used = time.perf_counter()
            except Exception as e:  # reported on the request; the server keeps serving
                req.error = e
            req.t_done = time.perf_counter()
            with self.cv:
                self.busy.discard(cid)
                self.completed.append(req)
                self.cv.notify_all()
            req.done.set()


class NativeServer:
    """The library's serving engine (bt_serve_*: C++ lanes, admission and
    scheduling inside libbtgpu) over the same clients and requests as Server.
    State-vector and density-matrix clients are compiled plans; trajectory
    clients are programs (n <= 14 complex64 / 13 complex128), their draws keyed
    by the request's seed on the device.  State-vector clients small enough for
    one CTA are packed: a program of `pack` members, one request per member, so
    up to `pack` queued requests of the client run as one launch (pack=1: plans
    for every state-vector client)."""

    def __init__(self, specs, lanes=8, prec="c64", hbm_budget=None, device=0, seed=1234, tiered=True, pack=8):
        from . import trajectories as T
        lib = L.lib()
        h = ctypes.c_void_p()
        L.check(lib.bt_serve_create(int(device), int(lanes), int(seed), int(hbm_budget or 0), ctypes.byref(h)))
        self.h = h
        self.ctx = Context(device, seed=seed + 7919)  # owns the programs' device tables
        self.specs = {s.cid: s for s in specs}
        self.prec = prec
        self.native = {}  # cid -> (client id, gate indices in theta order)
        self.keep = []    # plans / programs / term arrays the server borrows
        self.pending = {}
        self.completed = []
        for spec in specs:
            n = spec.n
            theta0 = np.full(spec.nparams, 0.1)
            xs = np.ascontiguousarray([t[1] for t in spec.terms], dtype=np.uint64)
            zs = np.ascontiguousarray([t[2] for t in spec.terms], dtype=np.uint64)
            cs = np.ascontiguousarray([t[0] for t in spec.terms], dtype=np.float64)
            cid = ctypes.c_int64()
            if spec.kind == "sv" and pack > 1 and n <= T.SHARED_MAX_N[prec]:
                prog = T.Program(n, pack, prec, self.ctx)
                pidx = []
                for op in hea_ops(n, spec.depth, theta0):
                    qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
                    if op.name in ("RY", "RZ"):  # per-member matrices: one request per member
                        pidx.append(prog.add_gate([op.mat] * pack, qs))
                    else:
                        prog.add_gate(op.mat, qs)
                L.check(lib.bt_serve_add_packed_client(h, prog.h, len(cs), _ptr(xs), _ptr(zs), _ptr(cs),
                                                        ctypes.byref(cid)))
                self.keep.append(prog)
            elif spec.kind in ("sv", "dm"):
                dm = spec.kind == "dm"
                plan = Plan(n, spec.kind, prec, self.ctx)
                ops = hea_ops(n, spec.depth, theta0)
                pidx = []
                for i, op in enumerate(_noisy(spec, ops) if dm else ops):
                    plan.add(op)
                    if op.name in ("RY", "RZ"):
                        pidx.append(i)
                plan.set_variable(pidx).compile(True, tiered=tiered)
                L.check(lib.bt_serve_add_plan_client(h, plan.h, len(cs), _ptr(xs), _ptr(zs), _ptr(cs),
                                                      ctypes.byref(cid)))
                self.keep.append(plan)
            else:
                ops = _noisy(spec, hea_ops(n, spec.depth, theta0))
                slots = T.build_slots(T.member_programs([ops], n, spec.ntraj))
                if not T.program_supported(slots, n, prec):
                    raise ValueError(f"trajectory client {spec.cid} (n={n}) does not fit a program")
                prog, gate_ops = T.compile_program(slots, n, spec.ntraj, prec, self.ctx)
                pidx = [gate_ops[i] for i, op in enumerate(ops) if op.name in ("RY", "RZ")]
                L.check(lib.bt_serve_add_program_client(h, prog.h, len(cs), _ptr(xs), _ptr(zs), _ptr(cs),
                                                         ctypes.byref(cid)))
                self.keep.append(prog)
            self.keep.append((xs, zs, cs))
            self.native[spec.cid] = (cid.value, np.ascontiguousarray(pidx, dtype=np.int64))

    def submit(self, req):
        cid, pidx = self.native[req.cid]
        mats = _hea_mats(req.theta)
        t = ctypes.c_int64()
        req.t_submit = time.perf_counter()
        L.check(L.lib().bt_serve_submit(self.h, cid, len(pidx), _ptr(pidx), _ptr(mats), int(req.seed),
                                        ctypes.byref(t)))
        self.pending[t.value] = req
        return req

    def wait(self, req, timeout=600.0):
        ticket = next(k for k, v in self.pending.items() if v is req)
        val, lat, svc = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        rc = L.lib().bt_serve_poll(self.h, ticket, int(timeout * 1e3), ctypes.byref(val), ctypes.byref(lat),
                                   ctypes.byref(svc))
        if rc == L.BT_ERR_TIMEOUT:
            raise TimeoutError(f"request {req.rid} still pending")
        del self.pending[ticket]
        if rc:
            req.error = L.BTError(rc, L.lib().bt_last_error(None).decode())
        req.value = val.value
        req.t_done = req.t_submit + lat.value
        req.t_start = req.t_done - svc.value
        req.done.set()
        self.completed.append(req)
        return req

    def stats(self):
        v = [ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64(), ctypes.c_uint64(),
             ctypes.c_int64()]
        L.check(L.lib().bt_serve_stats(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("completed", "p50_s", "p99_s", "resident", "hbm_used", "runs"), (x.value for x in v)))

    def close(self):
        if getattr(self, "h", None):
            L.lib().bt_serve_destroy(self.h)
            self.h = None
        self.keep = []
        self.ctx.close()


def program_request(spec, theta, seed, ctx, prec="c128"):
    """A trajectory client's request as one program run with the on-device draws
    of `seed` under ctx's seed: the same draws as the serving engine makes when
    its seed equals ctx's (for checking a served complex64 value in complex128)."""
    from . import trajectories as T
    ops = _noisy(spec, hea_ops(spec.n, spec.depth, theta))
    slots = T.build_slots(T.member_programs([ops], spec.n, spec.ntraj))
    prog, _ = T.compile_program(slots, spec.n, spec.ntraj, prec, ctx)
    st = GPUState(spec.n, prec, spec.ntraj, ctx)
    prog.run(st, seed=seed, records=False)
    v = _expect_h(st, spec.terms, -1)
    st.free()
    return v


def plain_request(spec, theta, seed, ctx, prec="c128"):
    """The plain per-call path: fresh state, one sweep per gate (and one call per
    channel), <H> at the end; the comparison point of the serving engine."""
    from .engine import apply
    n = spec.n
    if spec.kind == "traj":
        from .trajectories import run_trajectories
        st, _ = run_trajectories([_noisy(spec, hea_ops(n, spec.depth, theta))], n, spec.ntraj, prec=prec,
                                 rng=np.random.default_rng(seed), ctx=ctx, engine="slots")
        v = _expect_h(st, spec.terms, -1)
        st.free()
        return v
    ops = hea_ops(n, spec.depth, theta)
    if spec.kind == "dm":
        st = GPUDensity(n, prec, 1, ctx)
        apply(_noisy(spec, ops), st)
    else:
        st = GPUState(n, prec, 1, ctx)
        apply(ops, st)
    v = _expect_h(st, spec.terms)
    st.free()
    return v
