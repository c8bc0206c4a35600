"""Classical shadows (shadow, BlueTangle.jl src/ops.jl:145-185): the device sum of
snapshots equals the reference's kron construction from the same bases and
outcomes (exact dyadic sums, within 1e-12), the trace is one, and the shadow
estimates the state's correlations within statistical error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_rho(bases, outcomes):
    """rho += kron(3 U^dagger b b^dagger U - I ...) / shots, as the reference builds it."""
    from bluetangle_gpu.shadows import BASIS_ROTATIONS
    shots, n = bases.shape
    rho = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
    for m in range(shots):
        snap = np.ones((1, 1))
        for q in range(n):
            U = BASIS_ROTATIONS[bases[m, q]]
            v = np.zeros((2, 1))
            v[outcomes[m, q], 0] = 1
            snap = np.kron(snap, 3 * (U.conj().T @ v @ v.T @ U) - np.eye(2))
        rho += snap / shots
    return rho


def test_shadow_equals_reference_construction(ctx):
    import bluetangle_gpu as bt
    from bluetangle_gpu.shadows import shadow
    n = 4
    ops = [bt.Op("H", 1), bt.Op("CNOT", 1, 2), bt.Op("RY(0.7)", 3), bt.Op("CNOT", 3, 4), bt.Op("T", 2)]
    rho, bases, outcomes = shadow(ops, 300, n, seed=4)
    R = rho.to_numpy()
    assert abs(np.trace(R) - 1) < 1e-12
    assert np.abs(R - reference_rho(bases, outcomes)).max() < 1e-12


def test_shadow_estimates_correlations(ctx):
    """Bell pair on qubits 1, 2: <Z1 Z2> = <X1 X2> = 1 up to the shadow's
    statistical error (each snapshot factor has variance <= 9 per Pauli pair)."""
    import bluetangle_gpu as bt
    from bluetangle_gpu.shadows import shadow
    ops = [bt.Op("H", 1), bt.Op("CNOT", 1, 2)]
    shots = 20000
    rho, _, _ = shadow(ops, shots, 2, seed=11)
    zz = bt.correlation(rho, "Z,Z", [1, 2])
    xx = bt.correlation(rho, "X,X", [1, 2])
    tol = 5 * 9 / np.sqrt(shots)
    assert abs(zz - 1) < tol and abs(xx - 1) < tol
