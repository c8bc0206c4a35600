"""The generated fused-pass kernels run on the host (tests/kernel_emulator.py)
and compared with the oracle: brickworks wide enough for several tiles and the
window planner, every factored one-qubit form, and random gate mixes, in
complex64 (scalar code, the default; per-phase two-lane and pair-lane code) and
complex128, with the first/last phases
direct to memory, staged through shared memory, or as the coalescing rule picks,
and with register phases chosen among bit windows.
The generator's knobs are read once per process, so each configuration runs in a
child process, which writes the generated source without building it for the
device (BTGPU_JIT_DUMP_ONLY); nothing runs on a GPU."""
import os
import subprocess
import sys

import pytest

_CHILD = r"""
import math, os, sys, tempfile
import numpy as np
root = sys.argv[1]
sys.path[:0] = [os.path.join(root, "tests"), os.path.join(root, "bluetangle.jl_gb300"), os.path.join(root, "oracle")]
import oracle as O
import plan_emulator as E
import kernel_emulator as K
import bluetangle_gpu.circuits as C
O.build()
prec = sys.argv[2]
tol = 2e-5 if prec == "c64" else 1e-12
rng = np.random.default_rng(5)

def rstate(n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)

def check(n, seq, label):
    plan = E.host_plan(n, prec=prec)
    for m, qs, cs in seq:
        plan.add_matrix(m, qs, cs)
    plan.compile()
    src = open(os.environ["BTGPU_JIT_DUMP"]).read()
    psi = rstate(n)
    ref = psi.copy()
    for m, qs, cs in seq:
        ref = O.apply_k(ref, m, qs, cs)
    with tempfile.TemporaryDirectory() as d:
        out = K.run(plan, psi, src, d)
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < tol, (label, err)
    print(label, plan.stats()["passes"], "passes, rel err", err)

def ops_seq(ops):
    out = []
    for op in ops:
        qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
        out.append((op.mat, qs, [op.control] if op.control != -2 else []))
    return out

n = 15 if prec == "c64" else 14
check(n, ops_seq(C.random_ops(n, 1, rng) + C.brickwork(n, 6, rng)), "brickwork")
if prec == "c128":  # 2^16 entries and more: the float-float form of complex128 passes
    check(16, ops_seq(C.random_ops(16, 1, rng) + C.brickwork(16, 4, rng)), "brickwork 16")
c, s = math.cos(0.3), math.sin(0.3)
h = 1 / math.sqrt(2)
forms = [np.diag([1, -1]), np.diag([1, 1j]), np.diag([1, -1j]), np.diag([1, np.exp(0.7j)]),
         np.diag([0.2, 1.3]), np.diag([1.3j, 0.2]), h * np.array([[1, 1], [1, -1]]),
         h * np.array([[1, -1], [1, 1]]), h * np.array([[-1, 1], [1, 1]]), np.array([[c, -s], [s, c]]),
         np.array([[s, -c], [c, s]]), np.array([[c, s], [s, -c]]), np.array([[c, -1j * s], [-1j * s, c]]),
         np.array([[s, -1j * c], [-1j * c, s]]), np.array([[0.3, 0.9], [-0.9, 0.3]])]
seq = []
for rep in range(2):
    for m in forms:
        seq.append((np.asarray(m, dtype=complex), [int(rng.integers(1, 14))], []))
    a, b = [int(x) for x in rng.choice(np.arange(1, 14), 2, replace=False)]
    z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    q, r = np.linalg.qr(z)
    seq.append((q, [a, b], []))
    seq.append((np.eye(4, dtype=complex)[[0, 1, 3, 2]], [b, a], []))
check(13, seq, "factored forms")
seq = []
for i in range(48):
    qs = [int(x) for x in rng.choice(np.arange(1, 14), size=3, replace=False)]
    kind = rng.integers(0, 4)
    if kind == 0:
        z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)); u, _ = np.linalg.qr(z)
        seq.append((u, qs[:1], []))
    elif kind == 1:
        z = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)); u, _ = np.linalg.qr(z)
        seq.append((u, qs[:2], []))
    elif kind == 2:
        z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)); u, _ = np.linalg.qr(z)
        seq.append((u, qs[:1], qs[1:2]))
    else:
        seq.append((np.diag(np.exp(1j * rng.uniform(0, 6, 4))), qs[:2], []))
check(13, seq, "random gates")

# two members of one batch: the tile loop crosses the member boundary
n = 14
ops = ops_seq(C.brickwork(n, 4, rng))
plan = E.host_plan(n, prec=prec)
for m, qs, cs in ops:
    plan.add_matrix(m, qs, cs)
plan.compile()
src = open(os.environ["BTGPU_JIT_DUMP"]).read()
psis = [rstate(n), rstate(n)]
with tempfile.TemporaryDirectory() as d:
    out = K.run(plan, np.concatenate(psis), src, d, members=2).reshape(2, -1)
for k in range(2):
    ref = psis[k]
    for m, qs, cs in ops:
        ref = O.apply_k(ref, m, qs, cs)
    assert np.abs(out[k] - ref).max() < tol, ("members", k)
print("members ok")

# density matrix over 2n bits: row/column gates and Kraus sums as superoperators
import bluetangle_gpu as bt
n = 7
dops = C.noisy_brickwork_dm(n, 3, rng)
plan = E.host_plan(n, repr="dm", prec=prec)
for o in dops:
    plan.add(o)
plan.compile()
src = open(os.environ["BTGPU_JIT_DUMP"]).read()
rho0 = np.zeros((2 ** n, 2 ** n), complex)
rho0[0, 0] = 1
ref = rho0
for o in dops:
    if isinstance(o, bt.OpQC):
        ref = O.dm_channel(ref, o.kraus, o.qubit, o.target_qubit if o.q == 2 else -1)
    elif o.q == 1:
        ref = O.dm_hilbert1(ref, o.mat, o.qubit)
    else:
        ref = O.dm_hilbert2(ref, o.mat, o.qubit, o.target_qubit)
with tempfile.TemporaryDirectory() as d:
    out = K.run(plan, rho0, src, d).reshape(2 ** n, 2 ** n, order="F")
assert np.abs(out - ref).max() < tol, ("density", np.abs(out - ref).max())
print("density ok")
print("OK")
"""


@pytest.mark.parametrize("prec,env", [
    ("c64", {}),
    ("c128", {}),
    ("c64", {"BTGPU_JIT_PACKED": "1"}),
    ("c64", {"BTGPU_JIT_DIRECT": "0"}),
    ("c64", {"BTGPU_JIT_DIRECT": "2", "BTGPU_JIT_PACKED": "1"}),
    ("c128", {"BTGPU_JIT_DIRECT": "2"}),
    ("c64", {"BTGPU_PLAN_PHASE_WINDOWS": "0"}),
    ("c64", {"BTGPU_JIT_LANES": "1"}),
    ("c64", {"BTGPU_JIT_LANES": "1", "BTGPU_JIT_DIRECT": "0"}),
    ("c64", {"BTGPU_JIT_CPAIR": "1"}),
    ("c64", {"BTGPU_TILE_RB": "6"}),
    ("c128", {"BTGPU_JIT_FF": "0"}),
    ("c128", {"BTGPU_JIT_FF": "0", "BTGPU_JIT_DIRECT": "0"}),
    ("c64", {"BTGPU_JIT_CPAIR": "0"}),
])
def test_generated_kernels_on_host(prec, env, tmp_path):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    e = dict(os.environ, BTGPU_JIT_DUMP=str(tmp_path / "kernels.cu"), BTGPU_JIT_L2PF="0", BTGPU_JIT_PREFETCH="0",
             BTGPU_JIT_DUMP_ONLY="1", **env)
    e.pop("BTGPU_NO_JIT", None)
    r = subprocess.run([sys.executable, "-c", _CHILD, root, prec], env=e, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("OK"), r.stdout[-2000:] + r.stderr[-4000:]


_MEMBERS = r"""
import os, sys, tempfile, shutil
import numpy as np
root = sys.argv[1]
sys.path[:0] = [os.path.join(root, "tests"), os.path.join(root, "bluetangle.jl_gb300"), os.path.join(root, "oracle")]
import oracle as O
import plan_emulator as E
import kernel_emulator as K
from bluetangle_gpu import _lib as L
prec = sys.argv[2]
tol = 2e-5 if prec == "c64" else 1e-12
rng = np.random.default_rng(9)
n, B = 14, 3

def ry(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=complex)

def rz(t):
    return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])

# an ansatz: RY RZ on every qubit, a CNOT ladder, three layers; RY/RZ vary per member
seq, var = [], []
for layer in range(3):
    for q in range(1, n + 1):
        var.append(len(seq)); seq.append(["ry", [q]])
        var.append(len(seq)); seq.append(["rz", [q]])
    for q in range(1, n):
        seq.append(["cx", [q, q + 1]])
thetas = rng.uniform(0, 2 * np.pi, (B, len(var)))
cx = np.eye(4, dtype=complex)[[0, 1, 3, 2]]

def mat(kind, t):
    return ry(t) if kind == "ry" else rz(t)

plan = E.host_plan(n, prec=prec)
for i, (kind, qs) in enumerate(seq):
    plan.add_matrix(cx if kind == "cx" else mat(kind, 0.1), qs)
plan.set_variable(var).compile()
src = open(os.environ["BTGPU_JIT_DUMP"]).read()
idx = np.ascontiguousarray(var, dtype=np.int64)
P = __import__("ctypes").c_void_p
L.check(L.lib().bt_plan_prepare_members(plan.h, len(idx), idx.ctypes.data_as(P)))
src_pm = open(os.environ["BTGPU_JIT_DUMP"]).read()
member_mats = [[mat(seq[j][0], thetas[m, k]) for k, j in enumerate(var)] for m in range(B)]
psis = np.stack([np.eye(1, 2 ** n, 0).ravel() + 0j for _ in range(B)])
d = tempfile.mkdtemp()
out = K.run_members(plan, psis, src, src_pm, d, var, member_mats)
shutil.rmtree(d)
for m in range(B):
    ref = psis[m].copy()
    k = 0
    for kind, qs in seq:
        if kind == "cx":
            ref = O.apply_k(ref, cx, qs, [])
        else:
            ref = O.apply_k(ref, member_mats[m][k], qs, [])
            k += 1
    err = np.abs(out[m] - ref).max()
    assert err < tol, (m, err)
print("OK")
"""


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_per_member_matrices_on_host(prec, tmp_path):
    """bt_plan_run_members' host side: per-member kernels (entries from a member
    table) and the tables, run on the host for three members of one ansatz with
    different angles, each equal to the oracle with its own matrices."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    e = dict(os.environ, BTGPU_JIT_DUMP=str(tmp_path / "kernels.cu"), BTGPU_JIT_L2PF="0", BTGPU_JIT_PREFETCH="0",
             BTGPU_JIT_DUMP_ONLY="1")
    e.pop("BTGPU_NO_JIT", None)
    r = subprocess.run([sys.executable, "-c", _MEMBERS, root, prec], env=e, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("OK"), r.stdout[-2000:] + r.stderr[-4000:]



_COMPILE = r"""
import os, sys
import numpy as np
root = sys.argv[1]
sys.path[:0] = [os.path.join(root, "tests"), os.path.join(root, "bluetangle.jl_gb300")]
import plan_emulator as E
import bluetangle_gpu.circuits as C
n = 16  # complex128 passes of 2^16 entries take the float-float form
p = E.host_plan(n, prec=sys.argv[2])
rng = np.random.default_rng(3)
for o in C.random_ops(n, 3, rng) + C.brickwork(n, 3, rng):
    p.add(o)
p.compile()
print("OK")
"""


@pytest.mark.parametrize("prec,env", [("c64", {}), ("c128", {}), ("c128", {"BTGPU_JIT_FF": "0"})])
def test_generated_kernels_compile_for_sm103a(prec, env, tmp_path):
    """The generated source of every op type (random gates of the reference's set,
    dense two-qubit blocks included) compiles for sm_103a as the library's NVRTC
    would compile it (nvcc on the host: no GPU needed)."""
    import shutil
    if not shutil.which("nvcc"):
        pytest.skip("nvcc not on PATH")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "k.cu"
    e = dict(os.environ, BTGPU_JIT_DUMP=str(src), BTGPU_JIT_DUMP_ONLY="1", **env)
    e.pop("BTGPU_NO_JIT", None)
    r = subprocess.run([sys.executable, "-c", _COMPILE, root, prec], env=e, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.rstrip().endswith("OK"), r.stderr[-3000:]
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-cubin", "-O1", "-std=c++17",
                        "-o", str(tmp_path / "k.cubin"), str(src)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
