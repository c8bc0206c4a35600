"""Noise channels: Kraus sets, QuantumChannel, NoiseModel and Pauli twirling.

Host-side tables with the reference's values and quirks:
  - noise_model (BlueTangle.jl src/noise.jl:52-131), including `phase_flip`
    yielding Y (the reference compares a String with a Symbol, :78-81) and
    two-qubit channels as all kron(K_i, K_j) pairs (:126);
  - QuantumChannel / NoiseModel / Noise1 / Noise2 (src/struct.jl:90-173,
    :335-347) with the CPTP validation of is_valid_quantum_channel
    (src/struct.jl:291-309);
  - the Pauli-twirl tables and apply_twirl (src/noise.jl:136-255).
The channels themselves run on the GPU (bt_apply_kraus).
"""
import math
import random as _random

import numpy as np

from .gates import gate, is_measurement

__all__ = ["noise_model", "noise_model1", "noise_model2", "QuantumChannel", "NoiseModel", "Noise1", "Noise2",
           "is_valid_quantum_channel", "apply_twirl", "twirl_set"]


def _rx(t):
    return np.array([[math.cos(t / 2), -1j * math.sin(t / 2)], [-1j * math.sin(t / 2), math.cos(t / 2)]])


def _ry(t):
    return np.array([[math.cos(t / 2), -math.sin(t / 2)], [math.sin(t / 2), math.cos(t / 2)]], dtype=complex)


def _rz(t):
    return np.array([[np.exp(-1j * t / 2), 0], [0, np.exp(1j * t / 2)]])


def noise_model(model, p, two_qubit=False):
    """Kraus operators of a named channel (src/noise.jl:52-131)."""
    model = model.lower()
    I, X, Y, Z = gate["I"], gate["X"], gate["Y"], gate["Z"]
    if model == "amplitude_damping":
        ops = [np.array([[1.0, 0], [0, math.sqrt(1 - p)]], dtype=complex),
               np.array([[0, math.sqrt(p)], [0, 0]], dtype=complex)]
    elif model == "phase_damping":
        ops = [np.array([[1.0, 0], [0, math.sqrt(1 - p)]], dtype=complex),
               np.array([[0, 0], [0, math.sqrt(p)]], dtype=complex)]
    elif model in ("phase_flip", "bit_flip", "bit_phase_flip"):
        ops = [math.sqrt(1 - p) * I, math.sqrt(p) * (X if model == "bit_flip" else Y)]
    elif model == "depolarizing_amp":
        ops = [math.sqrt(1 - 3 * p / 4) * I, math.sqrt(p / 4) * X, math.sqrt(p / 4) * Y, math.sqrt(p / 4) * Z]
    elif model == "depolarizing":
        ops = [math.sqrt(1 - p) * I, math.sqrt(p / 3) * X, math.sqrt(p / 3) * Y, math.sqrt(p / 3) * Z]
    elif model == "rot_z":
        ops = [_rz(p)]
    elif model == "rot_y":
        ops = [_ry(p)]
    elif model == "rot_x":
        ops = [_rx(p)]
    elif model == "rot_p":
        ops = [np.array([[1, 0], [0, np.exp(1j * p)]])]
    elif model == "rot_xyz":
        ops = [_rx(p) / math.sqrt(3), _ry(p) / math.sqrt(3), _rz(p) / math.sqrt(3)]
    elif is_measurement(model):
        ops = [gate["P0"].copy(), gate["P1"].copy()]
    else:
        raise ValueError("Unknown quantum error model")
    ops = [np.asarray(o, dtype=np.complex128) for o in ops]
    if not two_qubit:
        return ops
    return [np.kron(a, b) for a in ops for b in ops]


def noise_model1(model, p):
    return noise_model(model, p, two_qubit=False)


def noise_model2(model, p):
    return noise_model(model, p, two_qubit=True)


def is_valid_quantum_channel(kraus):
    """Trace preservation and complete positivity (src/struct.jl:291-309)."""
    n = kraus[0].shape[0]
    s = sum(K.conj().T @ K for K in kraus)
    eye = np.eye(n)
    tp = np.linalg.norm(s - eye) <= 1.4901161193847656e-08 * max(np.linalg.norm(s), np.linalg.norm(eye))
    choi = sum(np.outer(K.reshape(-1, order="F"), K.reshape(-1, order="F").conj()) for K in kraus)
    herm = np.linalg.norm(choi - choi.conj().T) <= 1.4901161193847656e-08 * max(np.linalg.norm(choi), 1e-300)
    ev = np.linalg.eigvalsh((choi + choi.conj().T) / 2)
    cp = herm and bool(np.all(np.round(ev, 10) >= 0))
    return bool(tp and cp)


class QuantumChannel:
    """QuantumChannel(q, model, p) / QuantumChannel(model, kraus, p) (src/struct.jl:90-140)."""

    def __init__(self, *args):
        if len(args) == 3 and isinstance(args[0], int):
            q, model, p = args
            model = model.lower()
            kraus = noise_model1(model, p) if q == 1 else noise_model2(model, p)
        elif len(args) == 3:
            model, kraus, p = args
        elif len(args) == 2:
            model, p = args
            model = model.lower()
            kraus = noise_model1(model, p)
        else:
            raise TypeError("QuantumChannel(q, model, p) or QuantumChannel(model, kraus, p)")
        kraus = [np.asarray(K, dtype=np.complex128) for K in kraus]
        if not is_valid_quantum_channel(kraus):
            raise ValueError("not valid kraus operators: not CPTP!")
        q = int(round(math.log2(kraus[0].shape[0])))
        if q not in (1, 2):
            raise ValueError("Noise models are available only for 1 and 2 qubits!")
        self.q = q
        self.name = model.lower()
        self.p = float(p)
        self.kraus = kraus

    def prob(self, state, qubit, target=None):
        """Branch probabilities __calc_prob (src/struct.jl:9-29), computed on the GPU."""
        from .engine import channel_probs
        return channel_probs(state, self.kraus, qubit, target)

    def apply(self, state, qubit, target=None, rng=None, forced=None):
        from .engine import apply_channel
        return apply_channel(state, self.kraus, qubit, target, rng=rng, forced=forced)

    def __repr__(self):
        return f"QuantumChannel(q={self.q}, {self.name!r}, p={self.p})"


def Noise1(model, p):
    return QuantumChannel(1, model, p)


def Noise2(model, p):
    return QuantumChannel(2, model, p)


class NoiseModel:
    """NoiseModel(q1, q2) and its convenience constructors (src/struct.jl:147-173)."""

    def __init__(self, a, b=None, c=None, d=None):
        if isinstance(a, str) and isinstance(b, (int, float)) and c is None:
            n1, n2 = Noise1(a, b), Noise2(a, b)
        elif isinstance(a, str) and isinstance(c, str):
            n1, n2 = Noise1(a, b), Noise2(c, d)
        elif isinstance(a, (list, tuple)) and isinstance(b, (list, tuple)):
            n1, n2 = Noise1(a[0], a[1]), Noise2(b[0], b[1])
        elif isinstance(a, (list, tuple)) and b is False:
            n1, n2 = Noise1(a[0], a[1]), False
        elif a is False and isinstance(b, (list, tuple)):
            n1, n2 = False, Noise2(b[0], b[1])
        else:
            n1, n2 = a, b
        if isinstance(n1, QuantumChannel) and n1.q != 1:
            raise ValueError("size error in noise model (1)")
        if isinstance(n2, QuantumChannel) and n2.q != 2:
            raise ValueError("size error in noise model (2)")
        self.q1 = n1
        self.q2 = n2


# ---------------------------------------------------------------- twirling
# Pauli frames around CNOT/CX and ECR (src/noise.jl:136-219): entry i of a frame
# acts on `least` (odd i) or `least+1` (even i); the gate itself sits before entry 3.
_LIST_ECR = ["YYYY", "YZZI", "YIZZ", "YXYX", "ZYZY", "ZZYI", "ZIYZ", "ZXZX", "IYXX", "IZIZ", "IIII", "IXXY",
             "XYIX", "XZXZ", "XIXI", "XXIY"]
_LIST_ECR_REV = ["YYYY", "YZYZ", "YIXX", "YXXI", "ZYIZ", "ZZIY", "ZIZI", "ZXZX", "IYZZ", "IZZY", "IIII",
                 "IXIX", "XYXY", "XZXZ", "XIYX", "XXYI"]
_LIST_CNOT = ["YYXZ", "YZXY", "YIYX", "YXYI", "ZYIY", "ZZIZ", "ZIZI", "ZXZX", "IYZY", "IZZZ", "IIII", "IXIX",
              "XYYZ", "XZYY", "XIXX", "XXXI"]
_LIST_CNOT_REV = ["YYZX", "YZYI", "YIYZ", "YXZY", "ZYYX", "ZZZI", "ZIZZ", "ZXYY", "IYXY", "IZIZ", "IIII",
                  "IXXX", "XYIY", "XZXZ", "XIXI", "XXIX"]


def twirl_set(name, qubit, target, rng=None):
    """_twirl_set (src/noise.jl:136-219): one random Pauli frame."""
    r = rng if rng is not None else _random
    if qubit < target:
        lst = _LIST_ECR if name.upper() == "ECR" else _LIST_CNOT
    else:
        lst = _LIST_ECR_REV if name.upper() == "ECR" else _LIST_CNOT_REV
    idx = int(r.integers(0, 16)) if hasattr(r, "integers") else r.randrange(16)
    return list(lst[idx])


def apply_twirl(op, rng=None):
    """apply_twirl (src/noise.jl:230-255): [P1, P2, op, P3, P4] around CNOT/CX/ECR."""
    from .ops import Op
    if op.q == 2 and op.name.upper() in ("CNOT", "CX", "ECR"):
        least = min(op.qubit, op.target_qubit)
        out = []
        for i, p in enumerate(twirl_set(op.name, op.qubit, op.target_qubit, rng), start=1):
            fq = least if i % 2 == 1 else least + 1
            if i == 3:
                out.append(op)
            out.append(Op(p, fq))
        return out
    return [op]
