"""Readout-error mitigation on the GPU (measure's normalize(abs.(inv(A) * p), 1),
BlueTangle.jl src/ops.jl:544-545) against the dense reference form, and a round
trip through the confusion matrix at a size where the dense form is out of reach."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [("c128", 1e-13), ("c64", 2e-6)])
def test_mitigation_matches_dense_inverse(ctx, prec, tol):
    import bluetangle_gpu.mitigation as Mi
    from bluetangle_gpu.noise import noise_model1
    n = 8
    kraus = noise_model1("amplitude_damping", 0.07)
    p = np.random.default_rng(2).random(2 ** n)
    p /= p.sum()
    ref = np.abs(Mi.mitigation_matrix(n, kraus) @ p)
    ref /= ref.sum()
    got = Mi.measurement_mitigate(p, n, kraus, prec=prec)
    assert np.abs(got - ref).max() < tol


def test_mitigation_round_trip_large(ctx):
    """p -> A p (readout errors applied qubit by qubit on the host) -> mitigated = p
    at 20 qubits (the dense inverse would hold 2^40 entries)."""
    import bluetangle_gpu.mitigation as Mi
    from bluetangle_gpu.noise import noise_model1
    n = 20
    kraus = noise_model1("bit_flip", 0.03)
    A1 = Mi.confusion_matrix_1q(kraus)
    p = np.random.default_rng(5).random(2 ** n)
    p /= p.sum()
    noisy = p.reshape((2,) * n)
    for ax in range(n):  # A1 on each qubit (axis 0 = qubit 1, the most significant bit)
        noisy = np.moveaxis(np.tensordot(A1, noisy, axes=([1], [ax])), 0, ax)
    got = Mi.measurement_mitigate(noisy.ravel(), n, kraus)
    assert np.abs(got - p).max() < 1e-13
