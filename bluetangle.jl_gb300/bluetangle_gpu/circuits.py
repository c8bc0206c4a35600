"""Seeded synthetic circuit generators for the hot-path workloads.

The reference publishes no benchmark circuits; these generators follow its
op semantics: a random brickwork (one gate per qubit from {H, X, S, T, RX, RY,
RZ} with angles U[0, 2pi), then CNOTs on nearest-neighbour pairs, even offsets
on even layers and odd offsets on odd layers), the noisy density-matrix variant
with depolarizing and amplitude-damping channels after every gate, a
transverse-field Ising Trotter circuit (RZZ then RX per step, the pattern of
src/trotter.jl:16-23), a hardware-efficient ansatz (RY/RZ layers plus a CNOT
ladder, the EfficientSU2 pattern of src/vqa.jl:302-314), and random_ops
(src/gates.jl:154-214).
"""
import math

import numpy as np

from .gates import gates, gates_with_phase, one_qubit_gates, two_qubit_gates
from .ops import Op, OpQC

BRICK_1Q = ["H", "X", "S", "T", "RX", "RY", "RZ"]


def brickwork(n, depth, rng):
    ops = []
    for layer in range(depth):
        for q in range(1, n + 1):
            g = BRICK_1Q[int(rng.integers(0, len(BRICK_1Q)))]
            if g in ("RX", "RY", "RZ"):
                th = float(rng.uniform(0, 2 * math.pi))
                ops.append(Op(f"{g}({th!r})", q))
            else:
                ops.append(Op(g, q))
        start = 1 if layer % 2 == 0 else 2
        for q in range(start, n, 2):
            ops.append(Op("CNOT", q, q + 1))
    return ops


def haar_unitary(rng, d):
    """A Haar-random d x d unitary (QR of a complex Gaussian matrix, phases fixed)."""
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def su4_brickwork(n, depth, rng):
    """Brickwork of generic two-qubit gates: every layer a Haar-random 4 x 4 unitary
    on each nearest-neighbour pair (q, q+1), pairs from qubit 1 on even layers and
    from qubit 2 on odd ones -- the circuit where the factored one-qubit forms do
    not apply and every gate is a dense 4 x 4 complex matrix."""
    ops = []
    for layer in range(depth):
        for q in range(1 if layer % 2 == 0 else 2, n, 2):
            ops.append(Op("U4", haar_unitary(rng, 4), q, q + 1))
    return ops


def noisy_brickwork_dm(n, depth, rng, p1=1e-3, p2=1e-2, gamma=5e-3):
    """Brickwork with channels after every gate (the density-matrix workload);
    returns (ops, readout) where readout is the final 2% bit flip per qubit."""
    ops = []
    for op in brickwork(n, depth, rng):
        ops.append(op)
        if op.q == 1:
            ops.append(OpQC("depolarizing", p1, op.qubit))
            ops.append(OpQC("amplitude_damping", gamma, op.qubit))
        else:
            ops.append(OpQC("depolarizing", p2, op.qubit, op.target_qubit))
            ops.append(OpQC("amplitude_damping", gamma, op.qubit))
            ops.append(OpQC("amplitude_damping", gamma, op.target_qubit))
    return ops


def tfim_trotter(n, steps, dt, J, h):
    """Open-chain transverse-field Ising Trotter steps: RZZ(2 J dt) on (i, i+1)
    in ascending order, then RX(2 h_i dt) on every site."""
    h = np.broadcast_to(np.asarray(h, dtype=float), (n,))
    ops = []
    for _ in range(steps):
        for q in range(1, n):
            ops.append(Op(f"RZZ({float(2 * J * dt)!r})", q, q + 1))
        for q in range(1, n + 1):
            ops.append(Op(f"RX({float(2 * h[q - 1] * dt)!r})", q))
    return ops


def hea(n, depth, rng, sigma=0.3):
    """Hardware-efficient ansatz: per layer RY and RZ on every qubit with
    theta ~ N(0, sigma^2), then a CNOT ladder (1,2), (2,3), ..."""
    ops = []
    for _ in range(depth):
        for q in range(1, n + 1):
            ops.append(Op(f"RY({float(rng.normal(0, sigma))!r})", q))
            ops.append(Op(f"RZ({float(rng.normal(0, sigma))!r})", q))
        for q in range(1, n):
            ops.append(Op("CNOT", q, q + 1))
    return ops


def random_ops(n, depth, rng):
    """random_ops(N, depth) (src/gates.jl:154-214) without measurements."""
    ops = []
    allg = sorted(set(one_qubit_gates) | set(two_qubit_gates))
    for _ in range(depth):
        c = 1
        while c <= n:
            s = one_qubit_gates[int(rng.integers(0, len(one_qubit_gates)))] if c == n else \
                allg[int(rng.integers(0, len(allg)))]
            p1, p2, p3 = (round(float(rng.normal()) * math.pi, 2) for _ in range(3))
            if s in one_qubit_gates:
                if s in gates_with_phase:
                    name = {"U2": f"U2({p1},{p2})", "U3": f"U3({p1},{p2},{p3})"}.get(s, f"{s}({p1})")
                    ops.append(Op(name, c))
                else:
                    ops.append(Op(s, c))
                c += 1
            else:
                if s in gates_with_phase:
                    name = f"FSIM({p1},{p2})" if s == "FSIM" else f"{s}({p1})"
                    ops.append(Op(name, c, c + 1))
                else:
                    ops.append(Op(s, c, c + 1))
                c += 2
    return ops


def op_qubits(op):
    return [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
