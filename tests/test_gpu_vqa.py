"""Parameter-shift gradients of a variational ansatz (loss_and_grad_paramshift,
BlueTangle.jl src/vqa.jl:590-611) against the oracle evaluating every shifted
circuit, on both batch executors, and against finite differences of the loss.

Tolerances: complex128 within 1e-10 of the oracle (sums of ~100 Pauli
expectations); complex64 within 2e-4 (float32 rounding through ~100 gates, on
gradients of order 1); finite differences (step 1e-5, central) within 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ry(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def _rz(t):
    return np.array([[np.exp(-0.5j * t), 0], [0, np.exp(0.5j * t)]], dtype=np.complex128)


def ansatz(n, depth):
    """EfficientSU2-style: parametrised RY, RZ on every qubit, then a CNOT ladder
    (src/vqa.jl:302-314), the last layer with a controlled RY."""
    import bluetangle_gpu as bt
    ops = []
    for _ in range(depth):
        for q in range(1, n + 1):
            ops += [bt.Op("RY", _ry, q), bt.Op("RZ", _rz, q)]
        for q in range(1, n):
            ops.append(bt.Op("CNOT", q, q + 1))
    ops.append(bt.Op("RY", _ry, 2, control=1))
    return ops


def oracle_loss(oracle, ops, n, p, terms):
    import bluetangle_gpu.vqa as V
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    for op, mat in V._bound(ops, V.arg_counts(ops), p):
        qs, cs = V._qubits(op)
        psi = oracle.apply_k(psi, op.mat if mat is None else mat, qs, cs)
    return sum(c * oracle.expect_pauli_sv(psi, x, z) for c, x, z in terms)


def terms_for(n, seed):
    from bluetangle_gpu.serving import random_terms
    return random_terms(np.random.default_rng(seed), n, 3 * n)


@pytest.mark.parametrize("n,executor,prec,tol", [(6, "program", "c128", 1e-10), (6, "plan", "c128", 1e-10),
                                                 (15, "auto", "c128", 1e-10), (8, "program", "c64", 2e-4)])
def test_paramshift_matches_oracle(ctx, oracle, n, executor, prec, tol):
    import bluetangle_gpu.vqa as V
    ops = ansatz(n, 2)
    P = sum(V.arg_counts(ops))
    rng = np.random.default_rng(n)
    p = rng.uniform(0, 2 * np.pi, P)
    terms = terms_for(n, n + 1)
    l, g = V.loss_and_grad_paramshift(p, ops, n, terms, prec=prec, executor=executor)
    assert abs(l - oracle_loss(oracle, ops, n, p, terms)) < tol
    ref = []
    for i in range(P):
        a, b = p.copy(), p.copy()
        a[i] += V.SHIFT
        b[i] -= V.SHIFT
        ref.append(0.5 * (oracle_loss(oracle, ops, n, a, terms) - oracle_loss(oracle, ops, n, b, terms)))
    assert np.abs(g - np.array(ref)).max() < tol


def test_paramshift_equals_finite_differences(ctx):
    """For Pauli rotations the shift rule is the exact derivative."""
    import bluetangle_gpu.vqa as V
    n = 5
    ops = ansatz(n, 2)[:-1]  # the controlled RY is not a Pauli rotation: leave it out
    P = sum(V.arg_counts(ops))
    p = np.random.default_rng(3).uniform(0, 2 * np.pi, P)
    terms = terms_for(n, 9)
    _, g = V.loss_and_grad_paramshift(p, ops, n, terms)
    h = 1e-5
    plist = []
    for i in range(P):
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        plist += [a, b]
    vals = V.losses(ops, n, plist, terms)
    fd = (vals[0::2] - vals[1::2]) / (2 * h)
    assert np.abs(g - fd).max() < 1e-6
