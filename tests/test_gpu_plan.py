"""Fused plans (bt_plan_*): the fused tile passes apply the same map as the gates
one by one.  Checked against the oracle on state vectors and density matrices,
both precisions, batched members, and mixes with gates the tile cannot hold."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def runitary(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def oracle_op(oracle, psi, op):
    ctrls = [op.control] if op.control != -2 else []
    qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
    return oracle.apply_k(psi, op.mat, qs, ctrls)


def test_plan_tuning_configurations_and_autotune(ctx, oracle):
    """Every tuning configuration the autotuner tries (gates per pass, 4 or 5
    register bits, packed or scalar complex64 code) applies the same map; the
    autotuner keeps one of them compiled."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    n = 14
    rng = np.random.default_rng(7)
    ops = C.random_ops(n, 3, rng) + C.brickwork(n, 5, rng)
    psi = rstate(rng, n)
    ref = psi
    for op in ops:
        ref = oracle_op(oracle, ref, op)
    plan = bt.Plan(n, "sv", "c64")
    for op in ops:
        plan.add(op)
    for cfg in [(64, 5, 1), (64, 5, 0), (16, 5, 1), (64, 4, 1)]:
        plan.set_tuning(*cfg).compile(True)
        s = bt.state_from(psi, "c64")
        plan.run(s)
        assert np.abs(s.to_numpy() - ref).max() < 5e-5, cfg
    res = plan.autotune(bt.state_from(psi, "c64"), configs=[(64, 5, 1), (32, 5, 0)], reps=1)
    assert len(res) == 2 and all(t > 0 for _, t in res)
    s = bt.state_from(psi, "c64")
    plan.run(s)
    assert np.abs(s.to_numpy() - ref).max() < 5e-5


_DIRECT_SCRIPT = r"""
import sys, numpy as np
sys.path[:0] = sys.argv[2:4]
import bluetangle_gpu as bt
import bluetangle_gpu.circuits as C
out = {}
for prec, n in (("c64", 17), ("c128", 16)):
    rng = np.random.default_rng(23)
    ops = C.random_ops(n, 2, rng) + C.brickwork(n, 8, rng)
    plan = bt.plan_from_ops(ops, n, prec=prec)
    psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    s = bt.state_from(psi / np.linalg.norm(psi), prec)
    plan.run(s)
    out[prec] = s.to_numpy()
    out[prec + "_in"] = psi / np.linalg.norm(psi)
np.savez(sys.argv[1], **out)
"""


def test_plan_direct_and_staged_phases_identical(oracle, tmp_path):
    """The first/last phase of a specialised pass reads/writes its registers
    straight from/to global memory (BTGPU_JIT_DIRECT=1: where coalesced, 2:
    always) or through the shared-memory tile (0), with or without the next
    tile copied in by cp.async during a direct last phase (BTGPU_JIT_PREFETCH):
    the same arithmetic, so the states are bit-identical; the staged run is
    checked against the oracle."""
    import os
    import subprocess
    import sys
    import bluetangle_gpu.circuits as C
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    modes = {"0": ("0", "1"), "1": ("1", "1"), "2": ("2", "1"), "1np": ("1", "0"), "2np": ("2", "0")}
    for key, (direct, prefetch) in modes.items():
        f = str(tmp_path / f"d{key}.npz")
        env = dict(os.environ, BTGPU_JIT_DIRECT=direct, BTGPU_JIT_PREFETCH=prefetch)
        subprocess.run([sys.executable, "-c", _DIRECT_SCRIPT, f, root, os.path.join(root, "bluetangle.jl_gb300")],
                       env=env, check=True, timeout=600)
        res[key] = np.load(f)
    for prec in ("c64", "c128"):
        for key in modes:
            assert np.array_equal(res["0"][prec], res[key][prec]), (prec, key)
    rng = np.random.default_rng(23)
    ops = C.random_ops(16, 2, rng) + C.brickwork(16, 8, rng)
    ref = res["0"]["c128_in"]
    for op in ops:
        ref = oracle_op(oracle, ref, op)
    assert np.abs(res["0"]["c128"] - ref).max() < 1e-12


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 5e-5)])
@pytest.mark.parametrize("n", [12, 13, 16])
def test_plan_brickwork_matches_oracle(ctx, oracle, prec, tol, n):
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(100 + n)
    ops = C.brickwork(n, 12, rng)
    plan = bt.plan_from_ops(ops, n, prec=prec)
    st = plan.stats()
    assert st["gates"] == len(ops)
    psi = rstate(rng, n)
    s = bt.state_from(psi, prec)
    plan.run(s)
    ref = psi
    for o in ops:
        ref = oracle_op(oracle, ref, o)
    assert np.abs(s.to_numpy() - ref).max() < tol
    if n >= (13 if prec == "c64" else 12):
        assert st["fused_passes"] >= 1 and st["passes"] < len(ops) / 4


def _factored_forms(rng):
    """One-qubit matrices of every factored encoding: half diagonals (upper and
    lower half, exact -1 / i / -i), butterflies with each sign pattern,
    rotations with the diagonal or the off-diagonal entry the larger, RX-type in
    both regimes, non-unitary diagonals, and one diagonal small enough that the
    pass is encoded without factors."""
    c, s = math.cos(0.3), math.sin(0.3)
    h = 1 / math.sqrt(2)
    mats = [np.diag([1, -1]), np.diag([1, 1j]), np.diag([1, -1j]), np.diag([1, np.exp(0.7j)]),
            np.diag([0.2, 1.3]), np.diag([1.3j, 0.2]), np.diag([np.exp(-0.4j), np.exp(0.4j)]),
            h * np.array([[1, 1], [1, -1]]), h * np.array([[1, -1], [1, 1]]), h * np.array([[-1, 1], [1, 1]]),
            np.array([[c, -s], [s, c]]), np.array([[s, -c], [c, s]]), np.array([[c, s], [s, -c]]),
            np.array([[c, -1j * s], [-1j * s, c]]), np.array([[s, -1j * c], [-1j * c, s]]),
            np.array([[0.3, 0.9], [-0.9, 0.3]]), np.diag([1e-19, 1e-19])]
    return [np.asarray(m, dtype=complex) for m in mats]


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 5e-5)])
def test_plan_factored_encodings(ctx, oracle, prec, tol):
    """Plans whose passes hold every factored one-qubit form (the scalar taken out
    of each op and folded back into one op of the pass) apply the same map as the
    gates one by one; a dense two-qubit gate and a CNOT ride along."""
    import bluetangle_gpu as bt
    rng = np.random.default_rng(31)
    n = 14
    mats = _factored_forms(rng)
    seq = []
    for rep in range(3):
        for i, m in enumerate(mats):
            if i == len(mats) - 1 and rep:
                continue  # the tiny diagonal once (it scales the state by 1e-19)
            seq.append((m, [int(rng.integers(1, n + 1))]))
        a, b = [int(x) for x in rng.choice(np.arange(1, n + 1), 2, replace=False)]
        seq.append((runitary(rng, 4), [a, b]))
        seq.append((np.eye(4, dtype=complex)[[0, 1, 3, 2]], [b, a]))
    psi = rstate(rng, n)
    ref = psi.copy()
    plan = bt.Plan(n, prec=prec)
    for m, qs in seq:
        plan.add_matrix(m, qs)
        ref = oracle.apply_k(ref, m, qs, [])
    plan.compile()
    s = bt.state_from(psi, prec)
    plan.run(s)
    scale = np.abs(ref).max()  # errors relative to the state's scale
    assert np.abs(s.to_numpy() - ref).max() < tol * scale
    # in-place angle update of a rotation and a diagonal (the folded scalar changes)
    ref = psi.copy()
    upd = []
    for i, (m, qs) in enumerate(seq):
        if i in (3, 10):
            m = np.diag([1, np.exp(1.1j)]) if i == 3 else np.array([[s_, -c_], [c_, s_]])
            upd.append((i, m))
        ref = oracle.apply_k(ref, m, qs, [])
    plan.set_matrices(upd)
    s2 = bt.state_from(psi, prec)
    plan.run(s2)
    assert np.abs(s2.to_numpy() - ref).max() < tol * scale


c_, s_ = math.cos(1.2), math.sin(1.2)


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 5e-5)])
def test_plan_random_gates_controls_and_wide_gates(ctx, oracle, prec, tol):
    """random one/two-qubit gates on arbitrary pairs, controlled gates (folded or
    swept), three-qubit dense gates and Toffolis interleaved."""
    import bluetangle_gpu as bt
    rng = np.random.default_rng(7)
    n = 15
    plan = bt.Plan(n, prec=prec)
    psi = rstate(rng, n)
    ref = psi.copy()
    for i in range(160):
        kind = rng.integers(0, 7)
        qs = [int(x) for x in rng.choice(np.arange(1, n + 1), size=4, replace=False)]
        if kind <= 1:
            U = runitary(rng, 2)
            g = ([qs[0]], [])
        elif kind == 2:
            U = np.diag(np.exp(1j * rng.uniform(0, 6, 2)))
            g = ([qs[0]], [])
        elif kind == 3:
            U = runitary(rng, 4)
            g = (qs[:2], [])
        elif kind == 4:
            U = np.eye(4, dtype=complex)[[0, 1, 3, 2]] * np.exp(1j * rng.uniform(0, 6, 4))[:, None]
            g = (qs[:2], [])
        elif kind == 5:
            U = runitary(rng, 2)
            g = ([qs[0]], [qs[1]])
        else:
            if rng.random() < 0.5:
                U = runitary(rng, 8)
                g = (qs[:3], [])
            else:
                U = np.array([[0, 1], [1, 0]], dtype=complex)
                g = ([qs[0]], qs[1:3])
        plan.add_matrix(U, g[0], g[1])
        ref = oracle.apply_k(ref, U, g[0], g[1])
    plan.compile()
    s = bt.state_from(psi, prec)
    plan.run(s)
    assert np.abs(s.to_numpy() - ref).max() < tol * 3
    # unfused compilation of the same plan gives the same state
    plan.compile(fused=False)
    s2 = bt.state_from(psi, prec)
    plan.run(s2)
    assert np.abs(s2.to_numpy() - ref).max() < tol * 3


def test_plan_batched_members(ctx, oracle):
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(9)
    n, B = 14, 6
    ops = C.tfim_trotter(n, 5, 0.05, 1.0, rng.uniform(0.5, 1.5, n))
    plan = bt.plan_from_ops(ops, n, prec="c128")
    st = bt.zero_state(n, "c128", batch=B)
    psis = [rstate(rng, n) for _ in range(B)]
    for m, p in enumerate(psis):
        st.upload(p, m)
    plan.run(st)
    plan.run(st, member=3)
    for m, p in enumerate(psis):
        ref = p
        for rep in range(2 if m == 3 else 1):
            for o in ops:
                ref = oracle_op(oracle, ref, o)
        assert np.abs(st.to_numpy(m) - ref).max() < 1e-12


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 5e-5)])
def test_plan_density_matrix_noisy(ctx, oracle, prec, tol):
    """density-matrix plan: gates become row/column passes and Kraus sums become
    superoperators, fused over the 2n bits of vec(rho)."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(11)
    n = 7
    ops = C.noisy_brickwork_dm(n, 4, rng)
    plan = bt.plan_from_ops(ops, n, repr="dm", prec=prec)
    assert plan.stats()["fused_passes"] >= 1
    rho = bt.zero_rho(n, prec)
    plan.run(rho)
    ref = np.zeros((2 ** n, 2 ** n), complex)
    ref[0, 0] = 1
    for o in ops:
        if isinstance(o, bt.OpQC):
            ref = oracle.dm_channel(ref, o.kraus, o.qubit, o.target_qubit if o.q == 2 else -1)
        elif o.q == 1:
            ref = oracle.dm_hilbert1(ref, o.mat, o.qubit)
        else:
            ref = oracle.dm_hilbert2(ref, o.mat, o.qubit, o.target_qubit)
    assert np.abs(rho.to_numpy() - ref).max() < tol
    # the per-op path gives the same density matrix
    rho2 = bt.apply(ops, bt.zero_rho(n, prec))
    assert np.abs(rho2.to_numpy() - ref).max() < tol
