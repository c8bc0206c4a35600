"""Classical shadows (shadow, BlueTangle.jl src/ops.jl:145-185).

Per shot the reference re-simulates the circuit, rotates each qubit into a random
basis (X, Y, Z through H, HSP, I), samples one outcome and adds the snapshot
(x)_q (3 U^dagger |b><b| U - I) / shots to a 4^N density matrix.  Here the shots
are the members of one program: the circuit, per-member basis rotations, and a Z
measurement of every qubit (their joint outcome follows the Born distribution of
the rotated state, as one sample does); the snapshots are then summed into a
GPU-resident density matrix by one kernel (bt_shadow_accumulate).
"""
import numpy as np

from . import _lib as L
from .engine import Context, GPUDensity, GPUState, _ptr
from .gates import gate

__all__ = ["shadow", "snapshot_tables", "BASIS_ROTATIONS"]

# m_list of the reference: X, Y, Z bases through H, HSP, I (src/ops.jl:149)
BASIS_ROTATIONS = [gate["H"], gate["HSP"], gate["I"]]


def snapshot_tables():
    """The six single-qubit snapshot factors 3 U^dagger |b><b| U - I, code =
    2*basis + outcome, as row-major interleaved complex 2x2 matrices."""
    out = np.zeros((6, 2, 2), dtype=np.complex128)
    for b, U in enumerate(BASIS_ROTATIONS):
        for o in (0, 1):
            v = np.zeros((2, 1))
            v[o, 0] = 1
            out[2 * b + o] = 3 * (U.conj().T @ v @ v.T @ U) - np.eye(2)
    return out


def shadow(ops, shots, n=None, noise=False, prec="c128", ctx=None, rng=None, seed=0):
    """Classical-shadow density matrix of the circuit `ops` from `shots`
    snapshots.  rng draws the random bases (numpy Generator; default seeded by
    `seed`); branches and outcomes come from the device keyed by `seed`.  Returns
    (rho, bases, outcomes) with rho a GPUDensity and bases/outcomes shots x n."""
    from . import trajectories as T
    from .engine import _num_qubits
    ctx = ctx or Context.default()
    n = n or _num_qubits(ops)
    rng = rng if rng is not None else np.random.default_rng(seed)
    bases = rng.integers(0, 3, size=(shots, n))
    member_ops = T.member_programs([list(ops)], n, shots)
    slots = T.build_slots(member_ops, noise)
    for q in range(1, n + 1):
        slots.append(T.Slot("gate", [(BASIS_ROTATIONS[b], [q], []) for b in bases[:, q - 1]]))
    for q in range(1, n + 1):
        slots.append(T.Slot("measure", [("MZ", q)] * shots))
    prog, _ = T.compile_program(slots, n, shots, prec, ctx)
    st = GPUState(n, prec, shots, ctx)
    recs = prog.run(st, seed=seed)
    st.free()
    outcomes = np.array([r[-n:] for r in recs], dtype=np.int64)
    if outcomes.min() < 0:
        raise RuntimeError("a snapshot measurement failed")
    codes = np.ascontiguousarray((2 * bases + outcomes).astype(np.uint8))
    tab = np.ascontiguousarray(snapshot_tables().view(np.float64).ravel())
    rho = GPUDensity(n, prec, 1, ctx)
    ctx.check(L.lib().bt_shadow_accumulate(rho.h, shots, _ptr(codes), _ptr(tab)))
    return rho, bases, outcomes
