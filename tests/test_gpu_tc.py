"""Tensor-core plans (compile mode 3): every register phase of a fused pass as one
dense 32 x 32 complex block on the tcgen05 tensor cores, three TF32 products
accumulated in FP32.  Checked against the oracle (complex128) on the random
brickwork and on a brickwork of Haar-random two-qubit unitaries, against the
scalar complex64 plan on a larger state, and for the TF32 throughput diagnostic."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_state(oracle, ops, psi):
    for op in ops:
        qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
        psi = oracle.apply_k(psi, op.mat, qs, [op.control] if op.control != -2 else [])
    return psi


def _rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("kind", ["brickwork", "su4"])
@pytest.mark.parametrize("n", [13, 16])
def test_tensor_core_plan_matches_oracle(ctx, oracle, kind, n):
    """complex64 tolerance: FP32 rounding of the three-product TF32 split, 2e-5
    max-abs relative to the largest amplitude, as the scalar complex64 plans."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(60 + n)
    ops = C.brickwork(n, 8, rng) if kind == "brickwork" else C.su4_brickwork(n, 10, rng)
    plan = bt.Plan(n, "sv", "c64", ctx)
    for op in ops:
        plan.add(op)
    plan.compile(tensor_cores=True)
    psi = _rstate(rng, n)
    s = bt.state_from(psi, "c64")
    plan.run(s)
    ctx.synchronize()
    ref = _oracle_state(oracle, ops, psi)
    out = s.to_numpy()
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err
    assert abs(np.linalg.norm(out) - 1) < 5e-5  # FP32 rounding over the phases


def test_tensor_core_plan_equals_scalar_plan_large(ctx):
    """22 qubits (512 tiles per pass, every SM looping over tiles), both members of
    a batch: the tensor-core plan equals the scalar complex64 plan within FP32
    rounding."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    n = 22
    rng = np.random.default_rng(5)
    ops = C.su4_brickwork(n, 12, rng) + C.brickwork(n, 6, rng)
    res = []
    for tc in (False, True):
        plan = bt.Plan(n, "sv", "c64", ctx)
        for op in ops:
            plan.add(op)
        plan.compile(tensor_cores=tc)
        st = bt.zero_state(n, "c64", 2, ctx)
        st.set_basis(5, 1)
        plan.run(st)
        ctx.synchronize()
        res.append([st.to_numpy(0), st.to_numpy(1)])
        st.free()
    # the three-product TF32 split carries about 22 bits per operand against FP32's
    # 24: over 18 layers the two complex64 forms differ by a few 1e-5 relative per
    # amplitude, an infidelity far below 1e-6
    for m in range(2):
        a, b = res[0][m], res[1][m]
        assert np.abs(a - b).max() / np.abs(a).max() < 5e-5
        assert np.linalg.norm(a - b) / np.linalg.norm(a) < 5e-5
        infid = 1 - abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)
        assert infid < 1e-8, infid


def test_tf32_throughput_diagnostic(ctx):
    import bluetangle_gpu._lib as L
    v = ctypes.c_double(0)
    ctx.check(L.lib().bt_tc_tf32_peak(ctx.h, 2000, ctypes.byref(v)))
    assert v.value > 300, v.value  # TFLOP/s; about 1200 on a GB300
