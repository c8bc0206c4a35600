"""Readout-error mitigation of measured probabilities.

The reference (_measurement_mitigate_inv_matrix, BlueTangle.jl src/ops.jl:472-488)
builds the 2^N x 2^N confusion matrix column by column -- for every basis state
|a> it applies the readout channel to |a><a| on each qubit and keeps the diagonal
-- and inverts it densely; measure then replaces the probabilities p by
normalize(abs.(inv(A) * p), 1) (src/ops.jl:544-545, :635-637).  The channel acts
on one qubit at a time, so A = A1 (x) ... (x) A1 with the single-qubit confusion
matrix A1[b', b] = sum_k |<b'|K_k|b>|^2, and inv(A) = inv(A1) (x) ... (x) inv(A1).
Here inv(A) * p is N two-by-two sweeps of the probability vector, compiled into
fused passes on the GPU: O(N 2^N) work instead of building and inverting 4^N
entries.
"""
import numpy as np

from .engine import Context, GPUState, Plan

__all__ = ["confusion_matrix_1q", "mitigation_matrix", "measurement_mitigate"]


def _kraus(channel):
    return [np.asarray(k, dtype=np.complex128) for k in getattr(channel, "kraus", channel)]


def confusion_matrix_1q(channel):
    """A1[b', b] = <b'| sum_k K_k |b><b| K_k^dagger |b'> of a one-qubit readout channel."""
    ks = _kraus(channel)
    if ks[0].shape != (2, 2):
        raise ValueError("readout noise must be a one-qubit channel")
    A = np.zeros((2, 2))
    for K in ks:
        A += np.abs(K) ** 2
    return A


def mitigation_matrix(n, channel):
    """inv(A) as a dense 2^n x 2^n matrix (the reference's return value; small n)."""
    Ai = np.linalg.inv(confusion_matrix_1q(channel))
    out = np.ones((1, 1))
    for _ in range(n):
        out = np.kron(out, Ai)
    return out


def measurement_mitigate(probs, n, channel, prec="c128", ctx=None):
    """normalize(abs.(inv(A) * probs), 1) with inv(A) applied on the GPU as n
    one-qubit sweeps (fused passes); probs indexed by basis state (qubit 1 the
    most significant bit), as the reference's avg_prob."""
    p = np.asarray(probs, dtype=np.float64)
    if p.shape != (2 ** n,):
        raise ValueError(f"expected 2^{n} probabilities")
    Ai = np.linalg.inv(confusion_matrix_1q(channel)).astype(np.complex128)
    ctx = ctx or Context.default()
    st = GPUState(n, prec, 1, ctx)
    st.upload(p.astype(np.complex128))
    plan = Plan(n, "sv", prec, ctx)
    for q in range(1, n + 1):
        plan.add_matrix(Ai, [q])
    plan.compile(True)
    plan.run(st)
    out = np.abs(st.to_numpy().real)
    st.free()
    s = out.sum()
    return out / s if s > 0 else out
