"""The large state-vector configuration at its own size: a 33-qubit complex64
(64 GiB) and a 32-qubit complex128 (64 GiB) random brickwork of depth 30, run as
the compiled fused plan the benchmark times, checked against the per-gate sweep
path (k_gate, one bt_apply_matrix per gate: the path the oracle pins gate by gate
at small n) on a second state, and against the inverse circuit's return to
|0...0>.  This is where 64-bit amplitude offsets, 13-bit tiles over 2^20 tiles per
pass, the window planner's passes of up to 96 gates, the direct HBM phases and the
L2 prefetch all run.  The sequential-vs-compiled comparison follows the
reference's own test of apply against a compiled circuit
(test/runtests.jl:54-73, atol 1e-12)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEPTH = 30
SEED = 2024  # the benchmark's circuit


def _free_bytes():
    try:
        import torch
        return torch.cuda.mem_get_info()[0]
    except Exception:
        return 0


def _block_starts(n, nblk, blk, rng):
    """Block starts spread over the high bits: block k lies in the k-th 1/nblk
    of the index range, at a random aligned offset inside it."""
    span = (1 << n) // nblk
    return [k * span + int(rng.integers(0, span // blk)) * blk for k in range(nblk)]


def _blocks(st, starts, blk):
    import ctypes

    import bluetangle_gpu._lib as L
    out = np.empty((len(starts), blk), dtype=np.complex128)
    for i, s0 in enumerate(starts):
        st.ctx.check(L.lib().bt_state_download(st.h, 0, int(s0), blk, out[i].ctypes.data_as(ctypes.c_void_p)))
    return out


def _z_all(st):
    import ctypes

    import bluetangle_gpu._lib as L
    z = np.empty(st.n)
    st.ctx.check(L.lib().bt_expect_z_all(st.h, 0, z.ctypes.data_as(ctypes.c_void_p)))
    return z


def _norm2(st):
    import ctypes

    import bluetangle_gpu._lib as L
    v = np.empty(1)
    st.ctx.check(L.lib().bt_norm2(st.h, 0, v.ctypes.data_as(ctypes.c_void_p)))
    return float(v[0])


def _plan(bt, ops, n, prec, inverse=False):
    p = bt.Plan(n, "sv", prec)
    seq = reversed(ops) if inverse else ops
    for op in seq:
        qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
        m = np.asarray(op.mat, dtype=np.complex128)
        p.add_matrix(m.conj().T if inverse else m, qs)
    return p.compile(True)


@pytest.mark.parametrize("n,prec,amp_tol,rel_tol,z_tol", [
    (33, "c64", 2e-5, 1e-4, 1e-5),
    (32, "c128", 1e-12, 1e-12, 1e-12),
])
def test_headline_plan_equals_gate_path(ctx, n, prec, amp_tol, rel_tol, z_tol):
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    esize = 8 if prec == "c64" else 16
    need = 2 * (1 << n) * esize + (4 << 30)
    if _free_bytes() < need:
        pytest.skip(f"needs {need / 2**30:.0f} GiB of free device memory")
    ops = C.brickwork(n, DEPTH, np.random.default_rng(SEED))
    assert len(ops) == n * DEPTH + sum(len(range(1 if l % 2 == 0 else 2, n, 2)) for l in range(DEPTH))
    plan = _plan(bt, ops, n, prec)
    st = plan.stats()
    assert st["fused_passes"] == st["passes"] and st["jit_passes"] == st["passes"], st
    a = bt.zero_state(n, prec, ctx=ctx)
    plan.run(a)
    b = bt.zero_state(n, prec, ctx=ctx)
    bt.apply(ops, b)  # one bt_apply_matrix sweep per gate
    ctx.synchronize()
    blk = 4096
    starts = _block_starts(n, 64, blk, np.random.default_rng(5))
    xa, xb = _blocks(a, starts, blk), _blocks(b, starts, blk)
    assert np.all(np.isfinite(xa))
    err = float(np.abs(xa - xb).max())
    rel = float(np.linalg.norm(xa - xb) / np.linalg.norm(xb))
    assert err <= amp_tol and rel <= rel_tol, (err, rel)
    # the blocks hold a spread of the state, not zeros: |psi|^2 over them is about
    # their share of the index range
    share = float((np.abs(xb) ** 2).sum()) * (1 << n) / (len(starts) * blk)
    assert 0.5 < share < 2.0, share
    za, zb = _z_all(a), _z_all(b)
    assert float(np.abs(za - zb).max()) <= z_tol, np.abs(za - zb).max()
    # the reference's T (and T-dagger) entries are rounded to 10 significant
    # digits (src/gates.jl:32-33), so T is not exactly unitary: the norm drifts by
    # ~2e-11 per T gate (~140 in this circuit) on both paths alike
    # (complex64 adds FP32 rounding: the per-gate path's norm moves by ~1e-5 over
    # the 1470 gates, and the plan's stays within 1e-5 of it)
    na, nb = _norm2(a), _norm2(b)
    assert abs(na - nb) < (1e-5 if prec == "c64" else 1e-13), (na, nb)
    assert abs(nb - 1) < (1e-4 if prec == "c64" else 1e-7), nb
    b.free()
    # the inverse circuit (adjoints in reverse order) takes the plan's output back
    # to |0...0>, up to the same T rounding
    inv = _plan(bt, ops, n, prec, inverse=True)
    inv.run(a)
    x0 = _blocks(a, [0], blk)[0]
    back = float(abs(x0[0]) ** 2)
    assert abs(back - 1) < (2e-4 if prec == "c64" else 1e-7), back
    assert float(np.abs(x0[1:]).max()) < (1e-4 if prec == "c64" else 1e-9)
    a.free()


def test_per_member_plan_runs_equal_single_runs(ctx):
    """bt_plan_run_members (one launch per pass for a batch whose members carry
    their own matrices for the variational gates) equals one bt_plan_run per
    member with set_matrices, at 20 qubits in both precisions and across passes
    with and without member-dependent gates."""
    import math

    import bluetangle_gpu as bt

    def ry(t):
        c, s = math.cos(t / 2), math.sin(t / 2)
        return np.array([[c, -s], [s, c]], dtype=np.complex128)

    def rz(t):
        return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])

    n, depth, B = 20, 3, 3
    rng = np.random.default_rng(31)
    seq, var = [], []
    for _ in range(depth):
        for q in range(1, n + 1):
            var.append(len(seq)); seq.append(("ry", [q]))
            seq.append(("h" if q % 3 else "t", [q]))
            var.append(len(seq)); seq.append(("rz", [q]))
        for q in range(1, n):
            seq.append(("cx", [q, q + 1]))
    H = np.array([[1, 1], [1, -1]], dtype=complex) / math.sqrt(2)
    T = np.diag([1, np.exp(0.25j * math.pi)])
    CX = np.eye(4, dtype=complex)[[0, 1, 3, 2]]
    fixed = {"h": H, "t": T, "cx": CX}
    thetas = rng.uniform(0, 2 * math.pi, (B, len(var)))

    def mat(kind, t):
        return ry(t) if kind == "ry" else rz(t)

    member_mats = [[mat(seq[j][0], thetas[m, k]) for k, j in enumerate(var)] for m in range(B)]
    for prec, tol in (("c64", 2e-5), ("c128", 1e-12)):
        plan = bt.Plan(n, "sv", prec, ctx)
        for kind, qs in seq:
            plan.add_matrix(fixed[kind] if kind in fixed else mat(kind, 0.3), qs)
        plan.set_variable(var).compile(True)
        batch = bt.zero_state(n, prec, B, ctx)
        plan.run_members(batch, var, member_mats)
        got = [batch.to_numpy(m) for m in range(B)]
        for m in range(B):
            plan.set_matrices(list(zip(var, member_mats[m])))
            one = bt.zero_state(n, prec, 1, ctx)
            plan.run(one)
            ref = one.to_numpy()
            one.free()
            assert np.abs(got[m] - ref).max() < tol, (prec, m)
        # members differ (their angles differ) and a second batched run repeats the first
        assert np.abs(got[0] - got[1]).max() > 1e-3
        batch.set_zero()
        plan.run_members(batch, var, member_mats)
        assert np.array_equal(batch.to_numpy(B - 1), got[B - 1])
        batch.free()
