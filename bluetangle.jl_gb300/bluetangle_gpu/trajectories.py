"""Batched Monte-Carlo trajectories: many noisy shots of one circuit in lock-step.

The reference re-simulates the whole circuit once per shot
(`measure(circuit, shots)`, BlueTangle.jl src/ops.jl:619-630), each shot drawing
its own Kraus branches (src/struct.jl:31-41), mid-circuit outcomes
(src/hilbert.jl:682-696), Pauli-twirl frames (src/noise.jl:230-255) and, for
zero-noise extrapolation, repeating every CNOT 2*id+1 times (src/ops.jl:555-573).
Here all shots are members of one batched GPU state and every op is one launch
over the whole batch: a gate is one pass (one matrix for all members, or a
matrix per member for twirl frames), a channel is one reduction + one device-side
branch decision per member + one pass, and a measurement likewise.  Members whose
expanded op sequence is shorter (fewer ZNE repetitions, no measurement at that
point) are masked: they keep an identity matrix and skip channels and
measurements (forced = -2), so uneven depths run in the same launches.
"""
import ctypes

import numpy as np

from . import _lib as L
from .engine import GPUState, _cm, _i32, _ptr, apply_matrix
from .gates import gate
from .noise import NoiseModel, QuantumChannel, twirl_set
from .ops import Op, OpQC, ifOp

__all__ = ["Slot", "expand_member", "build_slots", "run_slots", "run_trajectories", "Program", "compile_program",
           "program_supported"]

_ID2 = np.eye(2, dtype=np.complex128)


class Slot:
    """One lock-step position: kind in {"gate", "channel", "measure"}; per member a
    payload or None (masked).  Gates carry (matrix, qubits, controls); channels
    (kraus, qubits); measurements (name, qubit)."""

    def __init__(self, kind, items):
        self.kind = kind
        self.items = items


def expand_member(op, zne_id=0, twirl=False, rng=None):
    """The reference's per-shot expansion of one circuit op (src/ops.jl:555-573 with
    apply_twirl, src/noise.jl:230-255), as a list of ops."""
    cnot = op.q == 2 and op.name.upper() in ("CNOT", "CX")
    reps = 2 * zne_id + 1 if (zne_id > 0 and cnot) else 1
    out = []
    for _ in range(reps):
        if twirl and op.q == 2 and op.name.upper() in ("CNOT", "CX", "ECR"):
            least = min(op.qubit, op.target_qubit)
            frame = twirl_set(op.name, op.qubit, op.target_qubit, rng)
            for i, p in enumerate(frame, start=1):
                if i == 3:
                    out.append(op)
                out.append(Op(p, least if i % 2 == 1 else least + 1))
        else:
            out.append(op)
    return out


def _noise_ops(op, noise):
    """Channel ops a NoiseModel adds after `op` (src/hilbert.jl:322-340)."""
    if not isinstance(noise, NoiseModel) or not getattr(op, "noisy", False):
        return []
    if op.q == 1:
        ch = noise.q1 if op.control == -2 else noise.q2
        if not isinstance(ch, QuantumChannel):
            return []
        return [(ch.kraus, [op.qubit] if op.control == -2 else [op.control, op.qubit])]
    if isinstance(noise.q2, QuantumChannel):
        return [(noise.q2.kraus, [op.qubit, op.target_qubit])]
    return []


def _op_slots(op, noise):
    """Slots of one op for one member (gate followed by its NoiseModel channels)."""
    if isinstance(op, OpQC):
        qs = [op.qubit] if op.q == 1 else ([op.qubit, op.target_qubit] if op.q == 2 else [op.qubit, op.qubit + 1, op.qubit + 2])
        return [("channel", (op.kraus, qs))]
    if op.type == "🔬":
        return [("measure", (op.name, op.qubit))]
    ctrls = [op.control] if op.control != -2 else []
    qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
    return [("gate", (op.mat, qs, ctrls))] + [("channel", c) for c in _noise_ops(op, noise)]


def explicit_noise(member_ops, noise):
    """member_ops with the channels a NoiseModel adds after each noisy op written
    out as OpQC ops (src/hilbert.jl:322-340), so that members built under
    different noise settings can share one batch (build_slots(..., noise=False))."""
    out = []
    for segs in member_ops:
        row = []
        for seg in segs:
            s2 = []
            for op in seg:
                s2.append(op)
                if not isinstance(op, OpQC) and op.type != "🔬":  # as _op_slots: none after measurements
                    for kraus, qs in _noise_ops(op, noise):
                        s2.append(OpQC("noise", kraus, qs[0], qs[1] if len(qs) == 2 else -1))
            row.append(s2)
        out.append(row)
    return out


def concat_members(*groups):
    """One batch from groups of members with different op sequences: each group's
    segments stay in order and every other group gets empty segments there, so
    at every slot the members of the other groups are idle (identity gates,
    skipped channels and measurements) and the whole batch runs as one program."""
    nseg = [len(g[0]) if g else 0 for g in groups]
    out = []
    for gi, g in enumerate(groups):
        before, after = sum(nseg[:gi]), sum(nseg[gi + 1:])
        for segs in g:
            out.append([[] for _ in range(before)] + list(segs) + [[] for _ in range(after)])
    return out


def concat_slots(*groups):
    """One slot list over the members of several groups, given as (slots, batch)
    pairs: each group's slots in order, the other groups' members idle (None) in
    them, so that compile_program gives each slot its group's member range."""
    out = []
    total = sum(b for _, b in groups)
    lo = 0
    for slots, b in groups:
        for sl in slots:
            out.append(Slot(sl.kind, [None] * lo + list(sl.items) + [None] * (total - lo - b)))
        lo += b
    return out


def build_slots(member_ops, noise=False):
    """Aligns per-member op sequences into lock-step slots.  member_ops[m] is a list
    of segments (one per circuit position), each a list of ops for that member;
    segments are padded to the longest member at that position."""
    B = len(member_ops)
    nseg = len(member_ops[0])
    slots = []
    for s in range(nseg):
        seqs = []
        for m in range(B):
            seq = []
            for op in member_ops[m][s]:
                seq.extend(_op_slots(op, noise))
            seqs.append(seq)
        L_ = max(len(x) for x in seqs)
        for i in range(L_):
            kinds = {x[i][0] for x in seqs if i < len(x)}
            if len(kinds) != 1:
                raise ValueError("members disagree on the kind of op at one position")
            kind = kinds.pop()
            slots.append(Slot(kind, [x[i][1] if i < len(x) else None for x in seqs]))
    return slots


def _same_gate(items):
    first = items[0] if items else None
    if first is not None and all(it is first for it in items):  # one shared payload
        return True
    first = None
    for it in items:
        if it is None:
            return False
        if first is None:
            first = it
        elif not (np.array_equal(it[0], first[0]) and it[1] == first[1] and it[2] == first[2]):
            return False
    return True


def _unitary_mix(kraus):
    for K in kraus:
        P = K.conj().T @ K
        if not np.allclose(P, P[0, 0] * np.eye(K.shape[0]), atol=1e-12):
            return False
    return True


def run_slots(state, slots, rng=None, records=True):
    """Runs lock-step slots on a batched state.  rng: numpy Generator whose draws
    decide branches/outcomes (one per member per channel or measurement), or None
    for the engine's on-device Philox stream.  Returns the per-member measurement
    records (-1 where a member was not measured)."""
    lib = L.lib()
    B = state.batch
    recs = [[] for _ in range(B)] if records else None
    for sl in slots:
        items = sl.items
        if sl.kind == "gate":
            live = [it for it in items if it is not None]
            if _same_gate(items):
                mat, qs, ctrls = items[0]
                apply_matrix(state, mat, qs, ctrls)
                continue
            qs, ctrls = live[0][1], live[0][2]
            if any(it[1] != qs or it[2] != ctrls for it in live):
                raise ValueError("members disagree on the qubits of a gate position")
            d = 2 ** len(qs)
            mats = np.concatenate([_cm(it[0] if it is not None else np.eye(d)).ravel() for it in items])
            q = _i32(qs)
            c = _i32(ctrls or [0])
            state.ctx.check(lib.bt_apply_matrix_members(state.h, len(qs), _ptr(q), _ptr(np.ascontiguousarray(mats)),
                                                         len(ctrls), _ptr(c) if ctrls else None))
        elif sl.kind == "channel":
            live = [it for it in items if it is not None]
            kraus, qs = live[0]
            if any(it[1] != qs or (it[0] is not kraus and not all(np.array_equal(a, b) for a, b in zip(it[0], kraus)))
                   for it in live):
                raise ValueError("members disagree on the channel at one position")
            forced = None if len(live) == B else _i32([-1 if it is not None else -2 for it in items])
            K = np.ascontiguousarray(np.concatenate([_cm(k).ravel() for k in kraus]))
            q = _i32(qs)
            u = None if rng is None else np.ascontiguousarray(rng.random(B))
            mode = L.BT_KRAUS_TRAJ | L.BT_KRAUS_REF_ORDER
            if rng is None and _unitary_mix(kraus):
                mode |= L.BT_KRAUS_UNITARY_MIX
            state.ctx.check(lib.bt_apply_kraus(state.h, len(qs), _ptr(q), len(kraus), _ptr(K), mode, _ptr(u),
                                               _ptr(forced), None, None))
        else:  # measure
            live = [it for it in items if it is not None]
            name, qubit = live[0]
            forced = None if len(live) == B else _i32([-1 if it is not None else -2 for it in items])
            up = name.upper()
            rot = None if up in ("MZ", "M(Z)") else (gate["H"] if up in ("MX", "M(X)") else gate["HSP"])
            if rot is not None:
                apply_matrix(state, rot, [qubit])
            u = None if rng is None else np.ascontiguousarray(rng.random(B))
            out = np.empty(B, dtype=np.int32)
            state.ctx.check(lib.bt_measure_z(state.h, int(qubit), _ptr(u), _ptr(forced), _ptr(out), None))
            if rot is not None:
                apply_matrix(state, rot.conj().T, [qubit])
            if records:
                for m in range(B):
                    if items[m] is not None:
                        recs[m].append(int(out[m]))
    return recs


PROGRAM_MAX_N = 34          # any state the GPU holds
SHARED_MAX_N = {"c64": 14, "c128": 13, "complex64": 14, "complex128": 13}  # one member per CTA
EXECUTORS = {"auto": 0, "shared": 1, "grouped": 2}


class Program:
    """A noisy circuit run on every member of a batched state (bt_program): for
    members of n <= 14 (complex64) / 13 (complex128) qubits one CTA per member in
    shared memory runs every gate, Kraus branch and measurement in one launch;
    larger members run group by group (ops within two qubits decided together
    from one reduced matrix, applied in one pass).  Built from lock-step slots by
    compile_program; run() fills the records of the measurements."""

    def __init__(self, n, batch, prec="c64", ctx=None):
        from .engine import Context, _PREC
        self.ctx = ctx or Context.default()
        self.n, self.batch, self.prec = n, batch, prec
        h = ctypes.c_void_p()
        self.ctx.check(L.lib().bt_program_create(self.ctx.h, n, _PREC[prec], batch, ctypes.byref(h)))
        self.h = h
        self.nops = 0
        self.rec_masks = []  # per record slot: bool per member, True where the member is measured
        self._range = (0, batch)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                L.lib().bt_program_free(self.h)
                self.h = None
        except Exception:
            pass

    def set_range(self, lo=0, hi=-1):
        """Ops added next act on members [lo, hi) only (bt_program_set_range)."""
        self.ctx.check(L.lib().bt_program_set_range(self.h, int(lo), int(hi)))
        self._range = (lo, self.batch if hi < 0 else hi)
        return self

    def add_gate(self, mats, qubits):
        """mats: one matrix, or batch matrices (per member) as a list or a
        (batch, d, d) array."""
        if isinstance(mats, np.ndarray) and mats.ndim == 3:  # column-major per matrix in one step
            per = True
            buf = np.ascontiguousarray(np.transpose(mats.astype(np.complex128, copy=False), (0, 2, 1))).ravel()
        else:
            per = isinstance(mats, (list, tuple))
            buf = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for m in mats]) if per else _cm(mats).ravel())
        q = _i32(qubits)
        self.ctx.check(L.lib().bt_program_add_gate(self.h, len(q), _ptr(q), _ptr(buf), int(per)))
        self.nops += 1
        return self.nops - 1

    def prepare(self):
        """Moves the program's tables to the device now (else the first run does)."""
        self.ctx.check(L.lib().bt_program_prepare(self.h, self.ctx.h))
        return self

    def set_executor(self, name):
        """"auto", "shared" (one CTA per member) or "grouped"."""
        self.ctx.check(L.lib().bt_program_set_executor(self.h, EXECUTORS[name]))
        return self

    def set_gate(self, index, mats):
        per = isinstance(mats, (list, tuple))
        buf = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for m in mats]) if per else _cm(mats).ravel())
        self.ctx.check(L.lib().bt_program_set_gate(self.h, int(index), _ptr(buf)))

    def add_channel(self, kraus, qubits, skip=None, unitary_mix=False):
        K = np.ascontiguousarray(np.concatenate([_cm(k).ravel() for k in kraus]))
        q = _i32(qubits)
        flags = L.BT_KRAUS_TRAJ | L.BT_KRAUS_REF_ORDER | (L.BT_KRAUS_UNITARY_MIX if unitary_mix else 0)
        sk = None if skip is None else _i32(skip)
        self.ctx.check(L.lib().bt_program_add_channel(self.h, len(q), _ptr(q), len(kraus), _ptr(K), flags, _ptr(sk)))
        self.nops += 1
        return self.nops - 1

    def add_measure(self, qubit, skip=None):
        sk = None if skip is None else _i32(skip)
        self.ctx.check(L.lib().bt_program_add_measure(self.h, int(qubit), _ptr(sk)))
        mask = np.ones(self.batch, bool) if skip is None else ~np.asarray(skip, bool)
        mask[:self._range[0]] = False
        mask[self._range[1]:] = False
        self.rec_masks.append(mask)
        self.nops += 1
        return self.nops - 1

    @property
    def ndraws(self):
        v = ctypes.c_int64(0)
        self.ctx.check(L.lib().bt_program_info(self.h, None, ctypes.byref(v), None))
        return v.value

    def run(self, state, rng=None, seed=0, records=True):
        """Runs every member of `state` through the program.  rng: numpy Generator
        whose draws (ndraws x batch, in op order, as run_slots consumes them) decide
        branches and outcomes, or None for on-device Philox keyed by `seed`.
        Returns per-member measurement records (lists), or None."""
        u = None
        if rng is not None:
            nd = self.ndraws
            if nd:
                u = np.ascontiguousarray(rng.random((nd, self.batch)))
        nrec = len(self.rec_masks)
        out = np.empty((self.batch, max(nrec, 1)), dtype=np.int32) if (records and nrec) else None
        state.ctx.check(L.lib().bt_program_run(self.h, state.h, _ptr(u), int(seed) & (2 ** 64 - 1), _ptr(out)))
        if not records:
            return None
        recs = [[] for _ in range(self.batch)]
        for r, mask in enumerate(self.rec_masks):
            for m in np.nonzero(mask)[0]:
                recs[m].append(int(out[m, r]))
        return recs


def _ctrl_matrix(mat):
    """|0><0| (x) I + |1><1| (x) U on (control, target), control the matrix MSB."""
    d = mat.shape[0]
    M = np.eye(2 * d, dtype=np.complex128)
    M[d:, d:] = mat
    return M


def grouped_bytes(slots, n, batch, prec="c64"):
    """HBM bytes the grouped executor moves for these slots: it groups consecutive
    ops within two qubits as bt_program does; per group every member that acts in
    it is read once for the reduced matrix (when a decision needs it) and read and
    written once by the apply pass.  (Measurement rotations of MX/MY are not
    counted.)"""
    member = (2 ** n) * (8 if prec in ("c64", "complex64") else 16)
    total = 0.0
    q, need, act = [], False, np.zeros(batch, dtype=bool)

    def close():
        nonlocal total
        if q:
            total += act.sum() * member * (3 if need else 2)

    for sl in slots:
        live = [it for it in sl.items if it is not None]
        if not live:
            continue
        if sl.kind == "gate":
            qs = list(live[0][1]) + list(live[0][2])
        elif sl.kind == "channel":
            qs = list(live[0][1])
        else:
            qs = [live[0][1]]
        if len(set(q) | set(qs)) > 2:
            close()
            q, need, act = [], False, np.zeros(batch, dtype=bool)
        q = sorted(set(q) | set(qs))
        if sl.kind == "gate":
            on = [i for i, it in enumerate(sl.items) if it is not None]
            sub = sl.items[on[0]:on[-1] + 1]
            if _same_gate(sub):  # one matrix for the range: every member in it acts
                act[on[0]:on[-1] + 1] = True
            else:  # per-member matrices: idle members and exact identities are passed over
                for i in on:
                    mat = np.asarray(sl.items[i][0])
                    if not np.array_equal(mat, np.eye(mat.shape[0])):
                        act[i] = True
        else:
            act |= np.array([it is not None for it in sl.items])
            if sl.kind == "measure" or not _unitary_mix(live[0][0]):
                need = True
    close()
    return total


def program_supported(slots, n, prec):
    if n < 2 or n > PROGRAM_MAX_N:
        return False
    for sl in slots:
        live = [it for it in sl.items if it is not None]
        if not live:
            continue
        if sl.kind == "gate":
            if any(len(it[1]) + len(it[2]) > 2 or (len(it[1]) == 2 and it[2]) for it in live):
                return False
        elif sl.kind == "channel":
            if len(live[0][1]) > 2:
                return False
    return True


def compile_program(slots, n, batch, prec="c64", ctx=None, unitary_mix=True):
    """Lock-step slots -> Program.  unitary_mix: channels whose Kraus operators are
    multiples of unitaries draw their branch from |c_i|^2 without reducing the
    state (exact for normalised members; set False for draw-for-draw agreement with
    run_slots under explicit draws).  Returns (program, gate_ops) with gate_ops[i]
    the program op index of slot i (gates only, else None)."""
    prog = Program(n, batch, prec, ctx)
    gate_ops = []
    cur = (0, batch)
    for sl in slots:
        items = sl.items
        on = [i for i, it in enumerate(items) if it is not None]
        if not on:
            gate_ops.append(None)
            continue
        # the slot's ops act on the members between its first and last live one;
        # members outside idle there (groups of members concatenated into one batch)
        rng_ = (on[0], on[-1] + 1)
        if rng_ != cur:
            prog.set_range(rng_[0], rng_[1] if rng_[1] < batch else -1)
            cur = rng_
        items = items[rng_[0]:rng_[1]]
        live = [it for it in items if it is not None]
        full_range = len(live) == len(items)

        def skip_of():  # skip table over the whole batch (the range bounds it already)
            return None if full_range else [0] * rng_[0] + [0 if it is not None else 1 for it in items] + \
                [0] * (batch - rng_[1])

        if sl.kind == "gate":
            def full(it):
                mat, qs, ctrls = it
                return (_ctrl_matrix(np.asarray(mat, np.complex128)), [ctrls[0], qs[0]]) if ctrls else (mat, list(qs))
            fl = [full(it) if it is not None else None for it in items]
            qs = fl[items.index(live[0])][1]
            if any(f is not None and f[1] != qs for f in fl):
                raise ValueError("members disagree on the qubits of a gate position")
            if _same_gate(items):
                gate_ops.append(prog.add_gate(fl[0][0], qs))
            else:
                d = 2 ** len(qs)
                gate_ops.append(prog.add_gate([f[0] if f is not None else np.eye(d) for f in fl], qs))
        elif sl.kind == "channel":
            kraus, qs = live[0]
            if any(it[1] != qs or (it[0] is not kraus and not all(np.array_equal(a, b) for a, b in zip(it[0], kraus)))
                   for it in live):
                raise ValueError("members disagree on the channel at one position")
            prog.add_channel(kraus, list(qs), skip_of(), unitary_mix and _unitary_mix(kraus))
            gate_ops.append(None)
        else:
            name, qubit = live[0]
            up = name.upper()
            rot = None if up in ("MZ", "M(Z)") else (gate["H"] if up in ("MX", "M(X)") else gate["HSP"])
            skip = skip_of()
            if rot is not None:
                rd = rot.conj().T
                prog.add_gate(rot if full_range else [rot if it is not None else _ID2 for it in items], [qubit])
            prog.add_measure(qubit, skip)
            if rot is not None:
                prog.add_gate(rd if full_range else [rd if it is not None else _ID2 for it in items], [qubit])
            gate_ops.append(None)
    return prog, gate_ops


def member_programs(steps, n, batch, zne_ids=None, twirl=False, frame_rng=None, measure_prob=0.0,
                    measure_rng=None):
    """Per-member segment lists: each circuit op expanded for the member (ZNE,
    twirl), and after every step a Z measurement of each qubit with probability
    measure_prob, drawn independently per member."""
    zne_ids = list(zne_ids) if zne_ids is not None else [0] * batch
    frame_rng = frame_rng if frame_rng is not None else np.random.default_rng(0)
    measure_rng = measure_rng if measure_rng is not None else np.random.default_rng(1)
    member_ops = [[] for _ in range(batch)]
    for step in steps:
        for op in step:
            for m in range(batch):
                member_ops[m].append(expand_member(op, zne_ids[m], twirl, frame_rng))
        if measure_prob > 0:
            for q in range(1, n + 1):
                mask = measure_rng.random(batch) < measure_prob
                for m in range(batch):
                    member_ops[m].append([Op("MZ", q)] if mask[m] else [])
    return member_ops


def run_trajectories(steps, n, batch, noise=False, zne_ids=None, twirl=False, prec="c64", rng=None, frame_rng=None,
                     measure_prob=0.0, measure_rng=None, ctx=None, state=None, engine="auto", seed=0):
    """`batch` trajectories of a circuit given as a list of steps (lists of ops)
    from |0...0> (or the given batched `state`) in one batched state.

    zne_ids: per-member ZNE id (None: all 0).  twirl: Pauli-twirl CNOTs per member
    (frames drawn from frame_rng).  measure_prob: after each step every qubit of
    every member is measured in Z with this probability (masks from measure_rng).
    engine: "program" (the whole batch in one launch, members in shared memory;
    n <= 14 complex64 / 13 complex128, ops on <= 2 qubits), "slots" (one launch
    sequence per op over the batch) or "auto" (program when it applies).  rng
    gives the draws in the same order on both engines; without it the draws come
    from on-device Philox (`seed` for the program engine).
    Returns (state, records)."""
    if steps and not isinstance(steps[0], (list, tuple)):
        steps = [steps]
    member_ops = member_programs(steps, n, batch, zne_ids, twirl, frame_rng, measure_prob, measure_rng)
    slots = build_slots(member_ops, noise)
    st = state if state is not None else GPUState(n, prec, batch, ctx)
    use_prog = engine == "program" or (engine == "auto" and program_supported(slots, n, prec))
    if use_prog:
        prog, _ = compile_program(slots, n, batch, prec, st.ctx, unitary_mix=rng is None)
        recs = prog.run(st, rng=rng, seed=seed)
    else:
        recs = run_slots(st, slots, rng=rng)
    return st, recs
