"""GPU-resident states and the reference's hot-path API on top of libbtgpu.

GPUState / GPUDensity stand where the reference passes a SparseVector /
SparseMatrixCSC (BlueTangle.jl src/hilbert.jl:469, :639).  Every function below
keeps the reference's name, argument meaning and error behaviour and runs its
arithmetic in libbtgpu; nothing here computes on the CPU beyond 2^k x 2^k
host tables (gate matrices, Kraus sets, reduced matrices of k <= 3 qubits).

Randomness: where the reference calls rand(), these functions take `rng` (a
numpy Generator whose draws are passed to the GPU) or use the engine's
on-device Philox stream when rng is None; `forced` pins outcomes/branches.
GPU states are updated in place; the functions also return the state, so the
reference's `state = apply(state, op)` pattern works unchanged.
"""
import ctypes
import math
import random as _random

import numpy as np

from . import _lib as L
from .gates import gate, gates
from .noise import NoiseModel, QuantumChannel, apply_twirl
from .ops import Op, OpQC, QuantumOps, ifOp

__all__ = ["Context", "GPUState", "GPUDensity", "zero_state", "zero_rho", "state_from", "rho_from", "apply",
           "apply_noise", "apply_matrix", "apply_channel", "channel_probs", "born_measure_Z", "sample",
           "sample_exact", "expect", "correlation", "partial_trace", "fidelity", "to_state", "to_rho", "run",
           "measure", "Measurement", "pauli_masks"]

_P = ctypes.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _cm(m):
    """numpy matrix -> column-major complex128 buffer (the ABI's Julia layout)."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128).T)


def _i32(xs):
    return np.ascontiguousarray(np.asarray(xs, dtype=np.int32))


class Context:
    """One CUDA device and stream (bt_ctx)."""

    _default = None

    def __init__(self, device=0, seed=0x5EED):
        h = _P()
        L.check(L.lib().bt_ctx_create(int(device), int(seed) & (2 ** 64 - 1), ctypes.byref(h)))
        self.h = h
        self.device = device

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context()
        return cls._default

    def check(self, rc):
        L.check(rc, self.h)

    def synchronize(self):
        self.check(L.lib().bt_ctx_synchronize(self.h))

    @property
    def launch_count(self):
        v = ctypes.c_int64(0)
        self.check(L.lib().bt_ctx_launch_count(self.h, ctypes.byref(v)))
        return v.value

    @property
    def stream(self):
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        v = _P()
        self.check(L.lib().bt_ctx_stream(self.h, ctypes.byref(v)))
        return v.value or 0

    def close(self):
        if getattr(self, "h", None):
            L.lib().bt_ctx_destroy(self.h)
            self.h = None
        if Context._default is self:
            Context._default = None


_PREC = {"c128": L.BT_PREC_C128, "c64": L.BT_PREC_C64, "complex128": L.BT_PREC_C128, "complex64": L.BT_PREC_C64}


class _Handle:
    repr_code = None

    def __init__(self, n, prec="c128", batch=1, ctx=None):
        self.ctx = ctx or Context.default()
        self.n = int(n)
        self.prec = prec
        self.batch = int(batch)
        h = _P()
        self.ctx.check(L.lib().bt_state_alloc(self.ctx.h, self.n, self.repr_code, _PREC[prec], self.batch,
                                              ctypes.byref(h)))
        self.h = h

    def free(self):
        if getattr(self, "h", None) and self.ctx.h:
            L.lib().bt_state_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def entries(self):
        return 1 << (self.n if self.repr_code == L.BT_REPR_SV else 2 * self.n)

    def set_zero(self, member=-1):
        self.ctx.check(L.lib().bt_state_set_zero(self.h, member))
        return self

    def set_basis(self, index, member=-1):
        self.ctx.check(L.lib().bt_state_set_basis(self.h, member, int(index)))
        return self

    def _upload_flat(self, flat, member):
        flat = np.ascontiguousarray(flat, dtype=np.complex128)
        if flat.size != self.entries:
            raise ValueError("array size does not match the state")
        self.ctx.check(L.lib().bt_state_upload(self.h, member, 0, flat.size, _ptr(flat)))

    def _download_flat(self, member):
        out = np.empty(self.entries, dtype=np.complex128)
        self.ctx.check(L.lib().bt_state_download(self.h, member, 0, out.size, _ptr(out)))
        return out

    def copy_from(self, other, dst_member=-1, src_member=0):
        self.ctx.check(L.lib().bt_state_copy(self.h, dst_member, other.h, src_member))
        return self

    def clone(self):
        c = type(self)(self.n, self.prec, self.batch, self.ctx)
        for m in range(self.batch):
            c.copy_from(self, m, m)
        return c

    @property
    def N(self):
        return self.n


class GPUState(_Handle):
    """2^n state vector(s) on the GPU (`batch` members: trajectories, copies, slots)."""

    repr_code = L.BT_REPR_SV

    def upload(self, psi, member=0):
        self._upload_flat(np.asarray(psi).ravel(), member)
        return self

    def to_numpy(self, member=0):
        return self._download_flat(member)


class GPUDensity(_Handle):
    """4^n density matrix (matrices) on the GPU; rho[i, j] lives at i + j*2^n."""

    repr_code = L.BT_REPR_DM

    def upload(self, rho, member=0):
        rho = np.asarray(rho, dtype=np.complex128)
        self._upload_flat(rho.T.ravel(), member)  # column-major
        return self

    def to_numpy(self, member=0):
        d = 1 << self.n
        return self._download_flat(member).reshape(d, d).T.copy()


def zero_state(n, prec="c128", batch=1, ctx=None):
    """zero_state(N) (src/hilbert.jl:866) on the GPU."""
    return GPUState(n, prec, batch, ctx)


def zero_rho(n, prec="c128", batch=1, ctx=None):
    """zero_state(N)*zero_state(N)' as a GPU density matrix."""
    return GPUDensity(n, prec, batch, ctx)


def state_from(psi, prec="c128", ctx=None):
    psi = np.asarray(psi, dtype=np.complex128).ravel()
    n = int(psi.size).bit_length() - 1
    return GPUState(n, prec, 1, ctx).upload(psi)


def rho_from(rho, prec="c128", ctx=None):
    rho = np.asarray(rho, dtype=np.complex128)
    n = int(rho.shape[0]).bit_length() - 1
    return GPUDensity(n, prec, 1, ctx).upload(rho)


# ------------------------------------------------------------------ low level
def apply_matrix(state, mat, qubits, controls=(), member=-1):
    """op.expand(N)*state (or e_op*rho*e_op') for a dense matrix on `qubits`."""
    qubits = list(qubits)
    q = _i32(qubits)
    c = _i32(list(controls) or [0])
    M = _cm(mat)
    state.ctx.check(L.lib().bt_apply_matrix(state.h, len(qubits), _ptr(q), _ptr(M), len(controls),
                                            _ptr(c) if controls else None, member))
    return state


def _draws(rng, n):
    if rng is None:
        return None
    return np.ascontiguousarray(rng.random(n), dtype=np.float64)


def apply_channel(state, kraus, qubit, target=None, rng=None, forced=None, probs_out=False):
    """QuantumChannel.apply / OpQC.apply (src/struct.jl:31-76): Monte-Carlo branch on a
    state vector (every member draws its own branch), Kraus sum on a density matrix."""
    kraus = [np.asarray(K, dtype=np.complex128) for K in kraus]
    k = int(round(math.log2(kraus[0].shape[0])))
    if k == 3:
        qubits = [qubit, qubit + 1, qubit + 2]
    elif k == 2:
        if target is None or target < 0:
            raise ValueError("for 2-qubit quantum channel, you must select the target_qubit")
        qubits = [qubit, target]
    else:
        qubits = [qubit]
    q = _i32(qubits)
    K = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for m in kraus]))
    if isinstance(state, GPUDensity):
        state.ctx.check(L.lib().bt_apply_kraus(state.h, k, _ptr(q), len(kraus), _ptr(K), L.BT_KRAUS_SUM,
                                               None, None, None, None))
        return state
    B = state.batch
    u = _draws(rng, B)
    f = None
    if forced is not None:
        f = _i32(np.broadcast_to(np.asarray(forced), (B,)))
    br = np.empty(B, dtype=np.int32)
    pr = np.empty(B * len(kraus), dtype=np.float64)
    state.ctx.check(L.lib().bt_apply_kraus(state.h, k, _ptr(q), len(kraus), _ptr(K),
                                           L.BT_KRAUS_TRAJ | L.BT_KRAUS_REF_ORDER, _ptr(u), _ptr(f), _ptr(br),
                                           _ptr(pr)))
    if probs_out:
        return state, br, pr.reshape(B, len(kraus))
    return state


def partial_trace(state, keep, member=0):
    """partial_trace(psi, keep) (src/linalg.jl:83-192) for <= 3 kept qubits, in the listed order."""
    keep = [keep] if isinstance(keep, int) else list(keep)
    d = 1 << len(keep)
    out = np.empty(d * d, dtype=np.complex128)
    q = _i32(keep)
    state.ctx.check(L.lib().bt_reduced_dm(state.h, len(keep), _ptr(q), member, _ptr(out)))
    return out.reshape(d, d).T.copy()


def channel_probs(state, kraus, qubit, target=None, member=0):
    """__calc_prob (src/struct.jl:9-29): p_k = Re tr(K rho_A K^dagger) with rho_A the
    reduced state of (qubit) or of the pair in ascending order."""
    if target is None or target < 0:
        rho = partial_trace(state, [qubit], member)
    else:
        rho = partial_trace(state, sorted([qubit, target]), member)
    return np.array([np.real(np.trace(K @ rho @ K.conj().T)) for K in kraus])


def born_measure_Z(state, qubit, qubit2=None, rng=None, forced=None):
    """born_measure_Z(N, psi, q) (src/hilbert.jl:682-696): returns (state, outcome, p0);
    outcome and p0 are arrays of length batch for a batched state, scalars otherwise.
    On a density matrix: sum_b P_b rho P_b (src/hilbert.jl:784-796).

    born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721) with qubit2 given:
    returns (state, outcome, probs) with outcome in 1..4 (the reference's index
    into [P0 P0, P1 P0, P0 P1, P1 P1] on (q1, q2)) and probs the four weights."""
    if qubit2 is not None:
        return _born_measure_Z2(state, qubit, qubit2, rng, forced)
    B = state.batch
    u = _draws(rng, B)
    f = _i32(np.broadcast_to(np.asarray(forced), (B,))) if forced is not None else None
    out = np.empty(B, dtype=np.int32)
    p0 = np.empty(B, dtype=np.float64)
    state.ctx.check(L.lib().bt_measure_z(state.h, int(qubit), _ptr(u), _ptr(f), _ptr(out), _ptr(p0)))
    if B == 1:
        return state, int(out[0]), float(p0[0])
    return state, out, p0


def _born_measure_Z2(state, q1, q2, rng, forced):
    if not isinstance(state, GPUState):
        raise ValueError("the two-qubit Born measurement acts on state vectors")
    B = state.batch
    u = _draws(rng, B)
    f = _i32(np.broadcast_to(np.asarray(forced), (B,))) if forced is not None else None
    out = np.empty(B, dtype=np.int32)
    probs = np.empty((B, 4), dtype=np.float64)
    state.ctx.check(L.lib().bt_measure_z2(state.h, int(q1), int(q2), _ptr(u), _ptr(f), _ptr(out), _ptr(probs)))
    if B == 1:
        return state, int(out[0]), probs[0]
    return state, out, probs


# ------------------------------------------------------------------ apply
def _op_matrix(op, pars=None):
    if op.type == "f":
        if pars is None:
            raise ValueError("parametrised op needs pars")
        return np.asarray(op.mat(*pars), dtype=np.complex128)
    return op.mat


def _apply_gate(state, op, pars=None):
    mat = _op_matrix(op, pars)
    ctrls = [op.control] if op.control != -2 else []
    if op.q == 1:
        return apply_matrix(state, mat, [op.qubit], ctrls)
    if op.control != -2 and abs(op.qubit - op.target_qubit) != 1:
        # controlled non-adjacent pairs exist only as CCX/CCZ (src/hilbert.jl:56-64)
        if not (np.array_equal(mat, gate["CX"]) or np.array_equal(mat, gate["CZ"])):
            raise ValueError("Unsupported operation. Use 'CCZ' or 'CCX'.")
    return apply_matrix(state, mat, [op.qubit, op.target_qubit], ctrls)


def _measurement_basis(name, rng):
    up = name.upper()
    if up in ("MR", "M(R)"):
        r = rng if rng is not None else _random
        up = ["MX", "MY", "MZ"][int(r.integers(0, 3)) if hasattr(r, "integers") else r.randrange(3)]
    if up in ("MZ", "M(Z)"):
        return None
    if up in ("MX", "M(X)"):
        return gate["H"]
    return gate["HSP"]


def _born_measure(state, name, qubit, rng=None, forced=None):
    """_born_measure (src/hilbert.jl:669-679): rotate, measure Z, rotate back."""
    rot = _measurement_basis(name, rng)
    if rot is not None:
        apply_matrix(state, rot, [qubit])
    state, ind, _ = born_measure_Z(state, qubit, rng=rng, forced=forced)
    if rot is not None:
        apply_matrix(state, rot.conj().T, [qubit])
    return state, ind


def _reset_Z(state, qubit, rng=None, forced=None):
    """_reset_Z (src/hilbert.jl:752-759)."""
    state, ind, _ = born_measure_Z(state, qubit, rng=rng, forced=forced)
    if state.batch == 1:
        if ind == 1:
            apply_matrix(state, gate["X"], [qubit])
    else:
        for m in np.nonzero(np.asarray(ind) == 1)[0]:
            apply_matrix(state, gate["X"], [qubit], member=int(m))
    return state, ind


def apply_noise(state, op, noise, rng=None):
    """apply_noise (src/hilbert.jl:322-364)."""
    if not getattr(op, "noisy", False) or not isinstance(noise, NoiseModel):
        return state
    if op.q == 1:
        ch = noise.q1 if op.control == -2 else noise.q2
        if not isinstance(ch, QuantumChannel):
            return state
        if op.control == -2:
            return apply_channel(state, ch.kraus, op.qubit, rng=rng)
        return apply_channel(state, ch.kraus, op.control, op.qubit, rng=rng)
    if op.q == 2 and isinstance(noise.q2, QuantumChannel):
        return apply_channel(state, noise.q2.kraus, op.qubit, op.target_qubit, rng=rng)
    return state


def apply(a, b, noise=False, track_measurements=False, rng=None, pars=None, forced=None):
    """apply(state, op; noise, track_measurements) and apply(ops, state; ...)
    (src/hilbert.jl:469-557, :639-666).  `forced` (iterable) pins the outcomes
    of successive mid-circuit measurements, in order."""
    if isinstance(a, (list, tuple)):
        ops, state = a, b
    elif isinstance(b, (list, tuple)):
        state, ops = a, b
    else:
        ops, state = None, a
    if ops is None:
        ops = [b]
    forced_iter = iter(forced) if forced is not None else None
    mids = []
    for op in ops:
        if isinstance(op, tuple):
            op = Op(*op)
        state, m = _apply_one(state, op, noise, rng, pars, forced_iter)
        mids.extend(m)
    return (state, mids) if track_measurements else state


def _apply_one(state, op, noise, rng, pars, forced_iter):
    mids = []
    dm = isinstance(state, GPUDensity)
    if isinstance(op, OpQC):
        if op.name.upper() in ("RES", "RESET") and not dm:
            f = next(forced_iter) if forced_iter is not None else None
            state, _ = _reset_Z(state, op.qubit, rng=rng, forced=f)
        else:
            apply_channel(state, op.kraus, op.qubit, op.target_qubit if op.q == 2 else None, rng=rng)
    elif op.type == "🔬":
        if dm:
            raise RuntimeError("error: fix this!" if isinstance(op, ifOp) else "fix this:")
        f = next(forced_iter) if forced_iter is not None else None
        state, ind = _born_measure(state, op.name, op.qubit, rng=rng, forced=f)
        if isinstance(op, ifOp):
            for sub in (op.if01[0] if ind == 0 else op.if01[1]):
                state, _ = _apply_one(state, sub, noise, rng, pars, forced_iter)
                state = state
        mids.append(ind)
    else:
        _apply_gate(state, op, pars)
    if isinstance(noise, NoiseModel) and not isinstance(op, ifOp):
        apply_noise(state, op, noise, rng=rng)
    return state, mids


# ------------------------------------------------------------------ plans (fused circuits)
class Plan:
    """A compiled circuit (bt_plan): gates (and, for density matrices, Kraus sums)
    fused into tile passes; running it equals applying the ops one by one."""

    def __init__(self, n, repr="sv", prec="c128", ctx=None):
        self.ctx = ctx or Context.default()
        self.n = n
        self.repr_code = L.BT_REPR_DM if repr in ("dm", "density", L.BT_REPR_DM) else L.BT_REPR_SV
        self.prec = prec
        h = _P()
        self.ctx.check(L.lib().bt_plan_create(self.ctx.h, n, self.repr_code, _PREC[prec], ctypes.byref(h)))
        self.h = h

    def __del__(self):
        try:
            if getattr(self, "h", None):
                L.lib().bt_plan_free(self.h)
                self.h = None
        except Exception:
            pass

    def add_matrix(self, mat, qubits, controls=()):
        q = _i32(list(qubits))
        c = _i32(list(controls) or [0])
        M = _cm(mat)
        self.ctx.check(L.lib().bt_plan_add_matrix(self.h, len(q), _ptr(q), _ptr(M), len(controls),
                                                  _ptr(c) if controls else None))
        return self

    def add_kraus_sum(self, kraus, qubits):
        q = _i32(list(qubits))
        K = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for m in kraus]))
        self.ctx.check(L.lib().bt_plan_add_kraus_sum(self.h, len(q), _ptr(q), len(kraus), _ptr(K)))
        return self

    def add(self, op, pars=None):
        """Appends a gate Op (any density/state plan) or an OpQC (density plans)."""
        if isinstance(op, OpQC):
            if self.repr_code != L.BT_REPR_DM:
                raise ValueError("channels in a state-vector plan need trajectories; apply them with apply()")
            qs = [op.qubit] if op.q == 1 else ([op.qubit, op.target_qubit] if op.q == 2 else None)
            if qs is None:
                raise ValueError("3-qubit OpQC has no density-matrix method in the reference")
            return self.add_kraus_sum(op.kraus, qs)
        if op.type == "🔬":
            raise ValueError("measurements end a plan")
        mat = _op_matrix(op, pars)
        qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
        ctrls = [op.control] if op.control != -2 else []
        return self.add_matrix(mat, qs, ctrls)

    def compile(self, fused=True, tiered=False, tensor_cores=False):
        """fused: tile passes (else one sweep per gate); tiered: run the generic
        kernel at once and switch to specialised kernels when their background
        compile finishes; tensor_cores (complex64 state vectors): every register
        phase of a pass as one dense 32 x 32 block on the tensor cores."""
        mode = 3 if tensor_cores else ((2 if tiered else 0) if fused else 1)
        self.ctx.check(L.lib().bt_plan_compile(self.h, mode))
        return self

    def set_matrices(self, updates):
        """updates: list of (add_index, matrix) — new matrices for gates already added
        (add_index counts add_* calls from 0)."""
        if not updates:
            return self
        idx = np.ascontiguousarray([u[0] for u in updates], dtype=np.int64)
        mats = np.ascontiguousarray(np.concatenate([_cm(u[1]).ravel() for u in updates]))
        self.ctx.check(L.lib().bt_plan_set_matrices(self.h, len(updates), _ptr(idx), _ptr(mats)))
        return self

    def set_variable(self, indices):
        """Marks the gates of these add indices as variable (updated in place by
        set_matrices): compiled in entry-independent forms, so updates never
        recompile.  Call before compile."""
        idx = np.ascontiguousarray(list(indices), dtype=np.int64)
        self.ctx.check(L.lib().bt_plan_set_variable(self.h, len(idx), _ptr(idx)))
        return self

    def set_tuning(self, max_ops=0, tile_rb=0, packed=-1, tile_bits=0):
        """Fusion width (gates per pass), register bits per thread (4 or 5),
        two-lane arithmetic and tile bits of the fused passes; 0 / -1 keep the
        defaults.  Takes effect at the next compile."""
        self.ctx.check(L.lib().bt_plan_set_tuning(self.h, int(max_ops), int(tile_rb), int(packed), int(tile_bits)))
        return self

    def autotune(self, state, configs=None, reps=2):
        """Times each tuning configuration (max_ops, tile_rb, packed, tile_bits) on
        `state` (the timing runs overwrite it), keeps the fastest compiled and
        returns [(config, seconds per run)] in the order tried.  Smaller tiles are
        tried too: more CTAs per pass for small states, more CTAs per SM (whose
        loads and arithmetic overlap) for large ones."""
        import time
        c64 = self.prec in ("c64", "complex64")
        if configs is None:
            configs = ([(0, 5, 1, 0), (0, 5, 0, 0), (64, 5, 1, 0), (128, 5, 1, 0), (0, 4, 1, 0)] if c64
                       else [(0, 0, -1, 0), (64, 0, -1, 0), (128, 0, -1, 0)])
            nbits = self.n * (2 if self.repr_code == L.BT_REPR_DM else 1)
            mdef, mmin = (13, 10) if c64 else (12, 9)
            for m in range(min(mdef, nbits) - 1, mmin - 1, -1)[:3]:
                configs.append((0, 0, -1, m))
        configs = [tuple(c) + (0,) * (4 - len(c)) for c in configs]
        results = []
        for cfg in configs:
            self.set_tuning(*cfg).compile(True)
            self.run(state)  # loads the specialised kernels
            self.ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                self.run(state)
            self.ctx.synchronize()
            results.append((tuple(cfg), (time.perf_counter() - t0) / reps))
        best = min(results, key=lambda r: r[1])[0]
        self.set_tuning(*best).compile(True)
        return results

    def stats(self):
        v = [ctypes.c_int64(0) for _ in range(5)]
        self.ctx.check(L.lib().bt_plan_stats(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("gates", "passes", "fused_passes", "phases", "jit_passes"), (x.value for x in v)))

    def cost(self):
        """Per amplitude of a member and run: real flops of the compiled passes'
        arithmetic (an FMA counts two) and HBM bytes moved."""
        f, b = ctypes.c_double(0), ctypes.c_double(0)
        self.ctx.check(L.lib().bt_plan_cost(self.h, ctypes.byref(f), ctypes.byref(b)))
        return {"flops_per_amp": f.value, "bytes_per_amp": b.value}

    def run(self, state, member=-1):
        self.ctx.check(L.lib().bt_plan_run(self.h, state.h, member))
        return state

    def run_members(self, state, indices, member_mats):
        """Runs the plan on every member of state, member m with member_mats[m]
        (one matrix per add index in `indices`) for those gates: one launch per
        pass for the whole batch (bt_plan_run_members)."""
        idx = np.ascontiguousarray(list(indices), dtype=np.int64)
        if len(member_mats) != state.batch:
            raise ValueError("one list of matrices per member")
        buf = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for mm in member_mats for m in mm]))
        self.ctx.check(L.lib().bt_plan_run_members(self.h, state.h, len(idx), _ptr(idx), _ptr(buf)))
        return state


def plan_from_ops(ops, n, repr="sv", prec="c128", fused=True, ctx=None):
    p = Plan(n, repr, prec, ctx)
    for op in ops:
        p.add(op)
    return p.compile(fused)


# ------------------------------------------------------------------ sampling / observables
def sample(state, shots, rng=None, seed=0, member=0):
    """sample(psi, shots) (src/ops.jl:46-62): basis indices 0..2^N-1."""
    u = _draws(rng, shots)
    out = np.empty(int(shots), dtype=np.int64)
    state.ctx.check(L.lib().bt_sample(state.h, member, int(shots), _ptr(u), int(seed) & (2 ** 64 - 1), _ptr(out)))
    return out


def sample_exact(state, member=0):
    """sample_exact (src/ops.jl:98-101, :129-132): indices with non-zero weight and weights."""
    out = np.empty(1 << state.n, dtype=np.float64)
    state.ctx.check(L.lib().bt_probabilities(state.h, member, _ptr(out)))
    nz = np.nonzero(out)[0]
    return nz, out[nz]


def pauli_masks(names, qubits, n):
    """Masks of a Pauli string with names[i] on qubits[i] (qubit q -> bit n-q)."""
    x = z = 0
    for s, q in zip(names, qubits):
        b = 1 << (n - q)
        s = s.upper()
        if s == "X":
            x |= b
        elif s == "Z":
            z |= b
        elif s == "Y":
            x |= b
            z |= b
        elif s != "I":
            raise ValueError(f"{s} is not a Pauli name")
    return x, z


_PAULI = {"I": gate["I"], "X": gate["X"], "Y": gate["Y"], "Z": gate["Z"]}


def _pauli_terms(mats, qubits, n):
    """Expands a product of one-qubit matrices into Pauli strings: list of (coef, x, z)."""
    terms = [(1.0 + 0j, 0, 0)]
    for M, q in zip(mats, qubits):
        b = 1 << (n - q)
        new = []
        for name, P in _PAULI.items():
            c = np.trace(P @ M) / 2
            if c == 0:
                continue
            x = b if name in ("X", "Y") else 0
            z = b if name in ("Z", "Y") else 0
            new.extend((tc * c, tx | x, tz | z) for tc, tx, tz in terms)
        terms = new
    return terms


def _expect_terms(state, terms, member=0):
    if not terms:
        return 0.0
    xs = np.ascontiguousarray([t[1] for t in terms], dtype=np.uint64)
    zs = np.ascontiguousarray([t[2] for t in terms], dtype=np.uint64)
    out = np.empty(len(terms), dtype=np.float64)
    state.ctx.check(L.lib().bt_expect_pauli(state.h, len(terms), _ptr(xs), _ptr(zs), None, member, _ptr(out)))
    # Hermitian strings have real expectations: Re(c <P>) = Re(c) <P>
    return float(sum(np.real(t[0]) * v for t, v in zip(terms, out)))


def expect(state, what, qubit=None, member=0):
    """expect(state, op) / expect(state, "Z") / expect(rho, ...) (src/func.jl:91-101)."""
    n = state.n
    if isinstance(what, str):
        if what.upper() == "Z" and qubit is None:
            rows = state.batch if member == -1 else 1
            out = np.empty(rows * n, dtype=np.float64)
            state.ctx.check(L.lib().bt_expect_z_all(state.h, member, _ptr(out)))
            return out.reshape(rows, n) if member == -1 else list(out)
        M = gates(what)
        qs = range(1, n + 1) if qubit is None else [qubit]
        vals = [_expect_terms(state, _pauli_terms([M], [q], n), member) for q in qs]
        return vals if qubit is None else vals[0]
    op = what
    if isinstance(state, GPUState) and op.q <= 2 and op.type != "f":
        mat = op.mat
        qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
        ctrls = [op.control] if op.control != -2 else []
        q = _i32(qs)
        c = _i32(ctrls or [0])
        M = _cm(mat)
        out = np.empty(1, dtype=np.float64)
        state.ctx.check(L.lib().bt_expect_matrix(state.h, len(qs), _ptr(q), _ptr(M), len(ctrls),
                                                 _ptr(c) if ctrls else None, member, _ptr(out)))
        return float(out[0])
    # density matrix: Re tr(rho E) through the Pauli expansion of E
    if op.q == 1 and op.control == -2:
        return _expect_terms(state, _pauli_terms([op.mat], [op.qubit], n), member)
    raise NotImplementedError("expect(rho, op) supports uncontrolled one-qubit ops; use correlation for strings")


def correlation(state, list_of_operators, qubits_applied, member=0):
    """correlation(state/rho, "Z,Z", [i, j]) (src/func.jl:139-147)."""
    names = [s.strip() for s in list_of_operators.split(",")]
    if len(names) != len(qubits_applied):
        raise ValueError("qubit number does not match with operators")
    mats = [gates(s) for s in names]
    return _expect_terms(state, _pauli_terms(mats, list(qubits_applied), state.n), member)


def fidelity(a, b, amember=0, bmember=0):
    """fidelity(psi, phi) = |<psi|phi>|^2 (src/tensor.jl:219); for two density
    matrices fidelity(rho, sigma) = tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2
    (src/tensor.jl:222-229, bt_fidelity_dm)."""
    out = ctypes.c_double(0)
    if isinstance(a, GPUDensity) or isinstance(b, GPUDensity):
        a.ctx.check(L.lib().bt_fidelity_dm(a.h, amember, b.h, bmember, ctypes.byref(out)))
    else:
        a.ctx.check(L.lib().bt_fidelity(a.h, amember, b.h, bmember, ctypes.byref(out)))
    return out.value


# ------------------------------------------------------------------ drivers
def _num_qubits(ops):
    m = 0
    for op in ops:
        m = max(m, op.qubit, getattr(op, "target_qubit", -1), getattr(op, "control", -2))
    return m


def _expanded_ops(ops, id=0, twirl=False, rng=None):
    """_expanded_ops_for_shot (src/ops.jl:555-573)."""
    out = []
    for op in ops:
        cnot = op.q == 2 and op.name.upper() in ("CNOT", "CX")
        if id > 0 and cnot:
            for _ in range(2 * id + 1):
                out.extend(apply_twirl(op, rng) if twirl else [op])
        elif twirl and cnot:
            out.extend(apply_twirl(op, rng))
        else:
            out.append(op)
    return out


def to_state(ops, n=None, noise=False, twirl=False, id=0, rng=None, prec="c128", batch=1, ctx=None):
    """to_state(circuit, id) (src/ops.jl:790-795)."""
    n = n or _num_qubits(ops)
    st = zero_state(n, prec, batch, ctx)
    return apply(_expanded_ops(ops, id, twirl, rng), st, noise=noise, rng=rng)


def to_rho(ops, n=None, noise=False, twirl=False, id=0, rng=None, prec="c128", ctx=None):
    """to_rho(circuit; id) (src/ops.jl:806-844)."""
    n = n or _num_qubits(ops)
    rho = zero_rho(n, prec, 1, ctx)
    for op in ops:
        if op.q == 2 and op.name in ("CNOT", "CX") and id > 0:
            for _ in range(2 * id + 1):
                for t in (apply_twirl(op, rng) if twirl else [op]):
                    apply(rho, t, noise=noise)
        elif op.q == 2 and twirl:
            for t in apply_twirl(op, rng):
                apply(rho, t, noise=noise)
        else:
            apply(rho, op, noise=noise)
    return rho


def run(ops, shots=1, noise=False, id=0, twirl=False, rng=None, prec="c128", ctx=None):
    """run(ops, shots; backend=:statevector) (src/ops.jl:659-692): mid-circuit records per shot."""
    if shots <= 0:
        raise ValueError("`number_of_experiment` must be positive.")
    n = _num_qubits(ops)
    res = []
    for _ in range(shots):
        st = zero_state(n, prec, 1, ctx)
        _, mids = apply(_expanded_ops(ops, id, twirl, rng), st, noise=noise, track_measurements=True, rng=rng)
        res.append(mids)
        st.free()
    return res


class Measurement:
    """Measurement record (src/struct.jl:907-917): bitstr, probabilities (sample),
    <Z_i> (expect), 12 magnetisation moments, basis, shots, circuit name, qubits
    and the accumulated density matrix (a GPUDensity when the circuit asked for
    one, else None: the reference's empty placeholder)."""

    def __init__(self, bitstr, probs, n, shots, measurement_basis="0", circuit_name="state to measurement",
                 density_matrix=None):
        self.measurement_basis = measurement_basis
        self.circuit_name = circuit_name
        self.density_matrix = density_matrix
        self.bitstr = np.asarray(bitstr)
        self.sample = np.asarray(probs)
        self.number_of_qubits = n
        self.number_of_experiment = shots
        fock = ((self.bitstr[:, None] >> (n - 1 - np.arange(n))[None, :]) & 1) if len(self.bitstr) else np.zeros((0, n))
        self.expect = [float(np.sum(np.where(fock[:, i] == 0, self.sample, -self.sample))) for i in range(n)]
        mag = np.sum(1 - 2 * fock, axis=1) if len(self.bitstr) else np.zeros(0)
        self.mag_moments = [float(np.sum(mag.astype(float) ** k * self.sample)) for k in range(1, 13)]


def measure(state, shots=-1, rng=None, seed=0):
    """measure(state, number_of_experiment) (src/ops.jl:496-513)."""
    if shots == -1:
        bit, prob = sample_exact(state)
        return Measurement(bit, prob, state.n, shots)
    s = sample(state, shots, rng=rng, seed=seed)
    vals, counts = np.unique(s, return_counts=True)
    return Measurement(vals, counts / len(s), state.n, shots)
