"""Circuits with options, the circuit-level measure driver, and state preparation.

Mirrors of the reference's Options (src/struct.jl:835-854), compile
(src/ops.jl:421-445, here without layout routing: every op is kept as given),
measure(circuit, shots, id) (src/ops.jl:599-646) with its final-basis rotation
and readout channel (_final_measurement, src/ops.jl:856-914), the density_matrix
accumulation rho_construct (src/ops.jl:612, :626) and readout mitigation
(src/ops.jl:635-638), plus product_state and its Neel/Z3 wrappers, one/plus/minus
states, random_product_state and random_state (src/hilbert.jl:835-890) and
fidelity(rho, sigma) (src/tensor.jl:222-229).

The noiseless branch of measure runs the circuit once and samples every shot from
that state.  The noisy branch re-simulates the circuit once per shot in the
reference; here the shots are the members of one batched state run by the
trajectory engine (every member its own Kraus branches, mid-circuit outcomes,
twirl frames and random measurement bases), and one shot is drawn from each
member on the device (bt_sample_members).
"""
import ctypes

import numpy as np

from . import _lib as L
from .engine import (GPUDensity, GPUState, Measurement, _draws, _expanded_ops, _num_qubits, _ptr, apply,
                     measure as _measure_state, sample, zero_state)
from .gates import gate
from .noise import QuantumChannel
from .ops import Op, OpQC, ifOp

__all__ = ["Options", "Circuit", "compile", "measure", "product_state", "neel_state01", "neel_state10", "Z3", "Z3_s",
           "neel_state_s", "one_state", "plus_state", "minus_state", "random_product_state", "random_state",
           "fidelity_dm", "get_stats"]


class Options:
    """Options(; circuit_name, measurement_basis, noise, twirl, readout_noise,
    measurement_mitigate, density_matrix) (src/struct.jl:835-854); the basis is
    kept upper case, as the reference's constructor does."""

    def __init__(self, circuit_name="circuit", measurement_basis="Z", noise=False, twirl=False, readout_noise=False,
                 measurement_mitigate=False, density_matrix=False):
        self.circuit_name = circuit_name
        self.measurement_basis = measurement_basis.upper()
        self.noise = noise
        self.twirl = twirl
        self.readout_noise = readout_noise
        self.measurement_mitigate = measurement_mitigate
        self.density_matrix = density_matrix


def get_stats(ops):
    """get_stats (src/ops.jl:191-235): N, length, CNOT / two-qubit / mid-circuit
    measurement counts."""
    n = _num_qubits(ops)
    cx = sum(1 for op in ops if op.name.upper() in ("CX", "CNOT"))
    two = sum(1 for op in ops if op.q == 2)
    mid = sum(1 for op in ops if getattr(op, "type", "") == "🔬")
    return {"N": n, "len": len(ops), "cx_count": cx, "two_qubit_count": two, "mid_measurement_count": mid}


class Circuit:
    """A compiled circuit: its ops in order, statistics and options."""

    def __init__(self, ops, options=None):
        self.ops = list(ops)
        self.options = options if options is not None else Options()
        self.stats = get_stats(self.ops)

    @property
    def noise(self):
        return self.options.noise

    @property
    def n(self):
        return self.stats["N"]


def compile(ops, options=None):
    """compile(ops, options) (src/ops.jl:421-445) without layout routing."""
    return Circuit(ops, options)


# ------------------------------------------------------------------ final measurement
_BASIS = {"X": "H", "Y": "HSP", "Z": None}


def _final_ops(n, basis, rng):
    """The rotation (gate name or None) of every qubit for one shot
    (_final_measurement, src/ops.jl:856-914): H for X, HSP for Y, I for Z, and for
    R one of [H, HSP, I] drawn per qubit (rand(1:3))."""
    if basis in _BASIS:
        return [_BASIS[basis]] * n
    if basis == "R":
        return [["H", "HSP", None][int(rng.integers(0, 3))] for _ in range(n)]
    raise ValueError("measurement_basis error!")


def _final_measurement(state, options, rng):
    """Rotation of every qubit into the measured basis; the readout channel
    (apply_noise with a QuantumChannel) after each qubit's rotation."""
    ch = options.readout_noise
    for q, g in enumerate(_final_ops(state.n, options.measurement_basis, rng), start=1):
        if g is not None:
            apply(state, Op(g, q))
        if isinstance(ch, QuantumChannel):
            ch.apply(state, q, rng=rng)
    return state


def _probs_from_sample(samples):
    """get_probs_from_sample (src/ops.jl:76-91): distinct outcomes sorted, frequencies."""
    vals, counts = np.unique(np.asarray(samples, dtype=np.int64), return_counts=True)
    return vals, counts / len(samples)


def _mitigate(probs, bitstr, n, channel, ctx):
    """measure's mitigation line (src/ops.jl:635-638): normalize(abs.(inv(A) *
    avg_prob), 1).  The reference multiplies the 2^N x 2^N inverse by the vector of
    observed outcomes only, which has matching size only when every outcome was
    observed; anything else raises there (DimensionMismatch), and here."""
    from .mitigation import measurement_mitigate
    if len(bitstr) != 2 ** n:
        raise ValueError(f"DimensionMismatch: mitigation needs all 2^{n} outcomes observed, got {len(bitstr)}")
    return measurement_mitigate(probs, n, channel, ctx=ctx)


def _noisy_members(circ, shots, id, rng, frame_rng):
    """Per-member op sequences of the noisy branch: the shot's expanded circuit
    (ZNE repetitions, twirl frames), then the final rotation and readout channel
    of every qubit.  The rotations are not noisy (the reference multiplies the
    state by o.expand(N) without apply_noise's model); with basis R every qubit
    gets a rotation slot, I where the member drew it, so the members align."""
    from . import trajectories as T
    o = circ.options
    n = circ.n
    member_ops = [[] for _ in range(shots)]
    for op in circ.ops:
        for m in range(shots):
            member_ops[m].append(T.expand_member(op, id, o.twirl, frame_rng))
    ch = o.readout_noise
    for m in range(shots):
        tail = []
        for q, g in enumerate(_final_ops(n, o.measurement_basis, rng), start=1):
            if g is not None or o.measurement_basis == "R":
                tail.append(Op(g or "I", q, noisy=False))
            if isinstance(ch, QuantumChannel):
                tail.append(OpQC("readout", ch.kraus, q))
        member_ops[m].append(tail)
    return member_ops


def measure(what, shots=-1, id=0, rng=None, seed=0, prec="c128", ctx=None, engine="auto"):
    """measure(state, shots) (src/ops.jl:496-513) for a state, or
    measure(circuit, shots, id) (src/ops.jl:599-646) for a Circuit.

    rng (numpy Generator): the draws of Kraus branches, outcomes, random bases and
    shots, so that a run can be replayed; None draws on the device from `seed`."""
    if not isinstance(what, Circuit):
        return _measure_state(what, shots, rng=rng, seed=seed)
    circ, o = what, what.options
    if shots < 1:
        raise ValueError("number_of_experiment must be positive")
    n = circ.n
    rng_h = rng if rng is not None else np.random.default_rng(seed)
    rho = None
    noiseless = o.noise is False and circ.stats["mid_measurement_count"] == 0 and o.readout_noise is False
    if noiseless:
        st = zero_state(n, prec, 1, ctx)
        apply(_expanded_ops(circ.ops, 0, o.twirl, rng_h), st)
        _final_measurement(st, o, rng_h)
        shots_out = sample(st, shots, rng=rng, seed=seed)
        if o.density_matrix:
            rho = GPUDensity(n, "c128", 1, st.ctx)
            st.ctx.check(L.lib().bt_state_clear(rho.h, -1))
            st.ctx.check(L.lib().bt_rho_accumulate(rho.h, 0, st.h, ctypes.c_double(1.0)))
        c = st.ctx
        st.free()
    else:
        from . import trajectories as T
        st = GPUState(n, prec, shots, ctx)
        c = st.ctx
        if any(isinstance(op, ifOp) for op in circ.ops):
            # classically controlled ops follow each shot's own outcomes: one
            # re-simulation per member, as the reference does for every shot
            for m in range(shots):
                one = zero_state(n, prec, 1, c)
                apply(_expanded_ops(circ.ops, id, o.twirl, rng_h), one, noise=o.noise, rng=rng_h)
                _final_measurement(one, o, rng_h)
                st.copy_from(one, m, 0)
                one.free()
        else:
            member_ops = _noisy_members(circ, shots, id, rng_h, rng_h)
            slots = T.build_slots(member_ops, o.noise)
            use_prog = engine == "program" or (engine == "auto" and T.program_supported(slots, n, prec))
            if use_prog:
                prog, _ = T.compile_program(slots, n, shots, prec, c, unitary_mix=rng is None)
                prog.run(st, rng=rng, seed=seed, records=False)
            else:
                T.run_slots(st, slots, rng=rng, records=False)
        u = _draws(rng, shots)
        shots_out = np.empty(shots, dtype=np.int64)
        c.check(L.lib().bt_sample_members(st.h, _ptr(u), int(seed) & (2 ** 64 - 1), _ptr(shots_out)))
        if o.density_matrix:
            rho = GPUDensity(n, "c128", 1, c)
            c.check(L.lib().bt_state_clear(rho.h, -1))
            c.check(L.lib().bt_rho_accumulate(rho.h, 0, st.h, ctypes.c_double(1.0 / shots)))
        st.free()
    bitstr, probs = _probs_from_sample(shots_out)
    if o.measurement_mitigate and isinstance(o.readout_noise, QuantumChannel):
        probs = _mitigate(probs, bitstr, n, o.readout_noise, c)
    m = Measurement(bitstr, probs, n, shots)
    m.measurement_basis = o.measurement_basis
    m.circuit_name = o.circuit_name
    m.density_matrix = rho
    m.samples = shots_out
    return m


# ------------------------------------------------------------------ state preparation
def product_state(bits, prec="c128", ctx=None):
    """product_state(list) (src/hilbert.jl:835): qubit i in |1> where bits[i] is
    non-zero (sign(x) != 0), |0> otherwise; qubit 1 the most significant bit."""
    n = len(bits)
    idx = 0
    for b in bits:
        idx = (idx << 1) | (1 if int(np.sign(b)) != 0 else 0)
    st = GPUState(n, prec, 1, ctx)
    st.set_basis(idx)
    return st


def neel_state01(n, prec="c128", ctx=None):
    """neel_state01(N) (src/hilbert.jl:837): qubits 1, 3, ... in |0>."""
    return product_state([0 if i % 2 == 1 else 1 for i in range(1, n + 1)], prec, ctx)


def neel_state10(n, prec="c128", ctx=None):
    """neel_state10(N) (src/hilbert.jl:838): qubits 1, 3, ... in |1>."""
    return product_state([1 if i % 2 == 1 else 0 for i in range(1, n + 1)], prec, ctx)


def _z3_bits(n, j):
    return [1 if (i + 2 - j + 1) % 3 == 0 else 0 for i in range(1, n + 1)]


def Z3(n, j=1, prec="c128", ctx=None):
    """Z3(N, j) (src/hilbert.jl:844)."""
    return product_state(_z3_bits(n, j), prec, ctx)


def _index(bits):
    idx = 0
    for b in bits:
        idx = (idx << 1) | (1 if b else 0)
    return idx


def _superpose(n, indices, prec, ctx):
    """normalize(sum of basis states) written into a device state: zero, then the
    distinct indices with amplitude count / norm each."""
    st = GPUState(n, prec, 1, ctx)
    st.ctx.check(L.lib().bt_state_clear(st.h, 0))
    vals = {}
    for i in indices:
        vals[i] = vals.get(i, 0) + 1.0
    nrm = np.sqrt(sum(v * v for v in vals.values()))
    for i, v in vals.items():
        a = np.array([v / nrm + 0j])
        st.ctx.check(L.lib().bt_state_upload(st.h, 0, int(i), 1, _ptr(a)))
    return st


def Z3_s(n, prec="c128", ctx=None):
    """Z3_s(N) = normalize(Z3(N,1) + Z3(N,2) + Z3(N,3)) (src/hilbert.jl:849)."""
    return _superpose(n, [_index(_z3_bits(n, j)) for j in (1, 2, 3)], prec, ctx)


def neel_state_s(n, prec="c128", ctx=None):
    """neel_state_s(N) = (neel_state01(N) + neel_state10(N)) / sqrt(2) (src/hilbert.jl:854)."""
    a = _index([0 if i % 2 == 1 else 1 for i in range(1, n + 1)])
    b = _index([1 if i % 2 == 1 else 0 for i in range(1, n + 1)])
    return _superpose(n, [a, b], prec, ctx)


def one_state(n, prec="c128", ctx=None):
    """one_state(N) (src/hilbert.jl:867): |1...1>."""
    st = GPUState(n, prec, 1, ctx)
    st.set_basis((1 << n) - 1)
    return st


def _all_h(st):
    from .engine import Plan
    p = Plan(st.n, "sv", st.prec, st.ctx)
    for q in range(1, st.n + 1):
        p.add_matrix(gate["H"], [q])
    p.compile(True).run(st)
    return st


def plus_state(n, prec="c128", ctx=None):
    """plus_state(N) (src/hilbert.jl:869): every amplitude 1/sqrt(2^N)
    (H on every qubit of |0...0>, as one fused plan)."""
    return _all_h(zero_state(n, prec, 1, ctx))


def minus_state(n, prec="c128", ctx=None):
    """minus_state(N) (src/hilbert.jl:871-877): H on every qubit of |1...1>."""
    return _all_h(one_state(n, prec, ctx))


def random_product_state(n, rng=None, prec="c128", ctx=None):
    """random_product_state(N) = product_state(rand([0, 1], N)) (src/hilbert.jl:859)."""
    r = rng if rng is not None else np.random.default_rng()
    return product_state([int(b) for b in r.integers(0, 2, n)], prec, ctx)


def random_state(n, seed=0, prec="c128", ctx=None):
    """random_state(N) = normalize(rand(ComplexF64, 2^N)) (src/hilbert.jl:882),
    drawn on the device (bt_state_random)."""
    st = GPUState(n, prec, 1, ctx)
    st.ctx.check(L.lib().bt_state_random(st.h, 0, int(seed) & (2 ** 64 - 1)))
    return st


def fidelity_dm(rho, sigma, rmember=0, smember=0):
    """fidelity(rho, sigma) = tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2 (src/tensor.jl:222-229)."""
    out = ctypes.c_double(0)
    rho.ctx.check(L.lib().bt_fidelity_dm(rho.h, rmember, sigma.h, smember, ctypes.byref(out)))
    return out.value
