"""Compiled plans checked on the host: the planner (tile bits among light-cone
windows, register phases) and the op encoding (classes, factored forms, the
folded scalar, variable gates) emulated pass by pass from bt_plan_pass_ops and
compared with the oracle.  No GPU: planning needs none and the specialised
kernels are not built (BTGPU_NO_JIT)."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import plan_emulator as E


@pytest.fixture(autouse=True)
def _no_jit(monkeypatch):
    monkeypatch.setenv("BTGPU_NO_JIT", "1")


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


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_host_plan_random_gates_controls_and_wide_gates(oracle, prec, tol):
    rng = np.random.default_rng(7)
    n = 15
    plan = E.host_plan(n, prec=prec)
    psi = rstate(rng, n)
    ref = psi.copy()
    for i in range(200):
        kind = rng.integers(0, 7)
        qs = [int(x) for x in rng.choice(np.arange(1, n + 1), size=4, replace=False)]
        if kind <= 1:
            U, g = runitary(rng, 2), ([qs[0]], [])
        elif kind == 2:
            U, g = np.diag(np.exp(1j * rng.uniform(0, 6, 2))), ([qs[0]], [])
        elif kind == 3:
            U, g = runitary(rng, 4), (qs[:2], [])
        elif kind == 4:
            U, g = np.eye(4, dtype=complex)[[0, 1, 3, 2]] * np.exp(1j * rng.uniform(0, 6, 4))[:, None], (qs[:2], [])
        elif kind == 5:
            U, g = runitary(rng, 2), ([qs[0]], [qs[1]])
        else:
            U, g = ((runitary(rng, 8), (qs[:3], [])) if rng.random() < 0.5 else
                    (np.array([[0, 1], [1, 0]], dtype=complex), ([qs[0]], qs[1:3])))
        plan.add_matrix(U, g[0], g[1])
        ref = oracle.apply_k(ref, U, g[0], g[1])
    plan.compile()
    assert np.abs(E.run(plan, psi) - ref).max() < tol


@pytest.mark.parametrize("prec,n,tol", [("c128", 16, 1e-12), ("c64", 17, 2e-5)])
def test_host_plan_brickwork_windows(oracle, prec, n, tol):
    """States wider than a tile: passes take light-cone windows of tile bits."""
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(100 + n)
    ops = C.random_ops(n, 2, rng) + C.brickwork(n, 14, rng)
    plan = E.host_plan(n, prec=prec)
    for op in ops:
        plan.add(op)
    plan.compile()
    st = plan.stats()
    assert st["gates"] == len(ops) and st["passes"] < len(ops) / 10
    psi = rstate(rng, n)
    ref = psi
    for op in ops:
        ref = oracle_op(oracle, ref, op)
    assert np.abs(E.run(plan, psi) - ref).max() < tol


def _forms():
    c, s = math.cos(0.3), math.sin(0.3)
    h = 1 / math.sqrt(2)
    mats = [np.diag([1, -1]), np.diag([1, 1j]), np.diag([1, -1j]), np.diag([1, np.exp(0.7j)]),
            np.diag([0.2, 1.3]), np.diag([1.3j, 0.2]), np.diag([np.exp(-0.4j), np.exp(0.4j)]),
            h * np.array([[1, 1], [1, -1]]), h * np.array([[1, -1], [1, 1]]), h * np.array([[-1, 1], [1, 1]]),
            np.array([[c, -s], [s, c]]), np.array([[s, -c], [c, s]]), np.array([[c, s], [s, -c]]),
            np.array([[c, -1j * s], [-1j * s, c]]), np.array([[s, -1j * c], [-1j * c, s]]),
            np.array([[0.3, 0.9], [-0.9, 0.3]]), np.diag([1e-19, 1e-19])]
    return [np.asarray(m, dtype=complex) for m in mats]


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_host_plan_factored_forms_and_updates(oracle, prec, tol):
    """Every factored one-qubit form with its scalar folded into one op of the
    pass; then angle updates (the gates turn variable: one recompile, then none)."""
    rng = np.random.default_rng(31)
    n = 14
    seq = []
    for rep in range(3):
        for i, m in enumerate(_forms()):
            if i == 16 and rep:
                continue
            seq.append((m, [int(rng.integers(1, n + 1))]))
        a, b = [int(x) for x in rng.choice(np.arange(1, n + 1), 2, replace=False)]
        seq.append((runitary(rng, 4), [a, b]))
        seq.append((np.eye(4, dtype=complex)[[0, 1, 3, 2]], [b, a]))
    psi = rstate(rng, n)
    plan = E.host_plan(n, prec=prec)
    for m, qs in seq:
        plan.add_matrix(m, qs)
    plan.compile()

    def check(mats):
        ref = psi.copy()
        for m, (_, qs) in zip(mats, seq):
            ref = oracle.apply_k(ref, m, qs, [])
        assert np.abs(E.run(plan, psi) - ref).max() < tol * np.abs(ref).max()

    mats = [m for m, _ in seq]
    check(mats)
    for th in (2.9, 0.2, 1.9):
        upd = []
        for i in (3, 10, 13, 20):
            c, s = math.cos(th / 2), math.sin(th / 2)
            m = {3: np.diag([1, np.exp(1j * th)]), 10: np.array([[c, -s], [s, c]]),
                 13: np.array([[c, -1j * s], [-1j * s, c]]), 20: np.diag([np.exp(-1j * th), 1])}[i]
            mats[i] = np.asarray(m, dtype=complex)
            upd.append((i, mats[i]))
        plan.set_matrices(upd)
        plan.compile()  # re-encodes only if an update changed a pass's structure
        check(mats)


def test_host_plan_density_matrix_noisy(oracle):
    """Density-matrix plan over 2n bits: gates as row/column ops, Kraus sums as
    superoperators (kron-pair channels split into one-qubit ones)."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(11)
    n = 6
    ops = C.noisy_brickwork_dm(n, 5, rng)
    plan = E.host_plan(n, repr="dm", prec="c128")
    for op in ops:
        plan.add(op)
    plan.compile()
    rho0 = np.zeros((2 ** n, 2 ** n), complex)
    rho0[0, 0] = 1
    ref = rho0
    for o in ops:
        if isinstance(o, bt.OpQC):
            ref = oracle.dm_channel(ref, o.kraus, o.qubit, o.target_qubit if o.q == 2 else -1)
        elif o.q == 1:
            ref = oracle.dm_hilbert1(ref, o.mat, o.qubit)
        else:
            ref = oracle.dm_hilbert2(ref, o.mat, o.qubit, o.target_qubit)
    out = E.run(plan, rho0).reshape(2 ** n, 2 ** n, order="F")
    assert np.abs(out - ref).max() < 1e-12


def test_host_plan_headline_pass_count():
    """The 33-qubit depth-30 brickwork plans into at most 26 passes (tile bits
    grown in gate order needed 63), and its arithmetic per amplitude stays at the
    factored forms' cost."""
    import ctypes
    import bluetangle_gpu.circuits as C
    from bluetangle_gpu import _lib as L
    ops = C.brickwork(33, 30, np.random.default_rng(2024))
    plan = E.host_plan(33, prec="c64")
    for op in ops:
        plan.add(op)
    plan.compile()
    st = plan.stats()
    assert st["gates"] == 1470 and st["passes"] <= 26, st
    if os.environ.get("BTGPU_PLAN_PHASE_WINDOWS") != "0":
        assert st["phases"] <= 100, st  # register-bit windows: 96 phases instead of 117
        if os.environ.get("BTGPU_PLAN_PHASE_BEAM", "8") != "1":
            assert st["phases"] <= 92, st  # beam search over phase sequences
    f, b = ctypes.c_double(), ctypes.c_double()
    L.check(L.lib().bt_plan_cost(plan.h, ctypes.byref(f), ctypes.byref(b)))
    assert b.value == 16 * st["passes"] and f.value < 2600, (f.value, b.value)


def test_host_plans_with_greedy_phases():
    """The same checks with the greedy choice of register phases
    (BTGPU_PLAN_PHASE_BEAM=1, read once per process: run in a child)."""
    if os.environ.get("BTGPU_PLAN_PHASE_BEAM") == "1":
        pytest.skip("already running with greedy phases")
    env = dict(os.environ, BTGPU_PLAN_PHASE_BEAM="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", __file__, "-k",
                        "not without_phase_windows"],
                       env=env, cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


def test_host_plans_without_phase_windows():
    """The same checks with register phases grown in gate order only
    (BTGPU_PLAN_PHASE_WINDOWS=0, read once per process: run in a child)."""
    if os.environ.get("BTGPU_PLAN_PHASE_WINDOWS") == "0":
        pytest.skip("already running without phase windows")
    env = dict(os.environ, BTGPU_PLAN_PHASE_WINDOWS="0")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", __file__],
                       env=env, cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


@pytest.mark.parametrize("cfg", [(16, 5, 0, 0), (0, 4, 0, 0), (0, 5, 0, 12), (0, 5, 0, 11), (0, 5, 0, 10),
                                 (128, 5, 1, 0)])
def test_host_plan_tuning_configurations(oracle, cfg, monkeypatch):
    """Every tuning the autotuner may keep (gates per pass, 4 or 5 register bits,
    smaller tiles, two-lane code) plans the same map.  A register width other than
    the default applies to specialised passes only, so that case lets NVRTC build
    the kernels (on the host; nothing runs)."""
    import bluetangle_gpu.circuits as C
    if cfg[1] == 4:
        monkeypatch.delenv("BTGPU_NO_JIT")
    rng = np.random.default_rng(55)
    n = 17
    ops = C.random_ops(n, 2, rng) + C.brickwork(n, 10, rng)
    plan = E.host_plan(n, prec="c64")
    for op in ops:
        plan.add(op)
    plan.set_tuning(*cfg).compile()
    psi = rstate(rng, n)
    ref = psi
    for op in ops:
        ref = oracle_op(oracle, ref, op)
    assert np.abs(E.run(plan, psi) - ref).max() < 2e-5


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_host_plan_edge_sizes(oracle, prec, tol):
    """An empty plan compiles to no passes and leaves the state as it was; states
    of 1 to 8 qubits, narrower than a tile, run every gate as its own pass and
    match the oracle."""
    rng = np.random.default_rng(11)
    p = E.host_plan(5, prec=prec)
    p.compile()
    psi = rstate(rng, 5)
    assert p.stats()["passes"] == 0 and np.array_equal(E.run(p, psi), psi)
    for n in range(1, 9):
        p = E.host_plan(n, prec=prec)
        psi = rstate(rng, n)
        ref = psi.copy()
        for _ in range(30):
            if n >= 2 and rng.random() < 0.5:
                qs = [int(x) for x in rng.choice(np.arange(1, n + 1), size=2, replace=False)]
                U = runitary(rng, 4)
            else:
                qs, U = [int(rng.integers(1, n + 1))], runitary(rng, 2)
            p.add_matrix(U, qs)
            ref = oracle.apply_k(ref, U, qs, [])
        p.compile()
        assert np.abs(E.run(p, psi) - ref).max() < tol, n
