"""Host-side mirror of the reference interface: gate table, noise tables, op
descriptors, twirl frames.  CPU only (no kernels)."""
import math
import os

import numpy as np
import pytest


def test_gate_values_match_reference_tables(kref):
    from bluetangle_gpu.gates import gate, gates
    for name, m in kref.GATE.items():
        assert np.array_equal(gate[name], m), name
    # T rounded to 10 significant digits (src/gates.jl:32)
    assert gate["T"][1, 1] == complex(0.7071067812, 0.7071067812)
    assert np.allclose(gates("RX(0.1pi)"), kref.rx(0.1 * math.pi), atol=0, rtol=0)
    assert np.allclose(gates("RZ(.3π)"), kref.rz(0.3 * math.pi), atol=0, rtol=0)
    assert np.array_equal(gates("RZZ(0.7)"), kref.rzz(0.7))
    assert np.array_equal(gates("CP(1.25)"), kref.cp(1.25))
    assert np.array_equal(gates("MX"), gate["H"]) and np.array_equal(gates("MY"), gate["HSP"])
    with pytest.raises(KeyError):
        gates("NOPE")


def test_noise_tables_and_quirks(kref):
    from bluetangle_gpu.noise import noise_model
    for model in ("amplitude_damping", "phase_damping", "bit_flip", "phase_flip", "bit_phase_flip",
                  "depolarizing", "depolarizing_amp", "rot_x", "rot_y", "rot_z", "rot_p", "rot_xyz", "MZ"):
        for two in (False, True):
            # kron_ref builds each set from the channel's definition (Pauli weights,
            # damping actions, rotation generators), independently of noise.py: equal
            # up to the last bit of the trigonometric forms
            a, b = noise_model(model, 0.13, two), kref.noise_model(model, 0.13, two)
            assert len(a) == len(b) and all(np.allclose(x, y, rtol=0, atol=2e-16) for x, y in zip(a, b)), model
            s = sum(k.conj().T @ k for k in a)
            assert np.allclose(s, np.eye(s.shape[0]), atol=1e-14), model  # trace preserving
    # phase_flip yields Y (src/noise.jl:78-81); 2-qubit depolarizing is a 16-term product channel
    assert np.array_equal(noise_model("phase_flip", 0.25)[1], 0.5 * np.array([[0, -1j], [1j, 0]]))
    assert len(noise_model("depolarizing", 0.1, True)) == 16


def test_channel_validation_and_noise_model():
    from bluetangle_gpu import NoiseModel, QuantumChannel
    from bluetangle_gpu.noise import is_valid_quantum_channel
    with pytest.raises(ValueError, match="CPTP"):
        QuantumChannel("bad", [np.eye(2) * 1.1], 0.0)
    assert is_valid_quantum_channel([np.eye(2)])
    nm = NoiseModel("depolarizing", 0.1)
    assert nm.q1.q == 1 and nm.q2.q == 2 and len(nm.q2.kraus) == 16
    with pytest.raises(ValueError):
        NoiseModel(QuantumChannel(2, "bit_flip", 0.1), False)


def test_op_descriptors():
    from bluetangle_gpu import Op, OpQC, ifOp
    o = Op("CNOT", 2, 5)
    assert o.q == 2 and o.type == "op" and o.control == -2
    assert Op("RX(0.2)", 1).type == "phase"
    m = Op("MZ", 3)
    assert m.type == "🔬" and not m.noisy
    assert isinstance(Op("RES", 1), OpQC)
    t = Op("CCX", 1, 2, 3)
    assert t.name == "CX" and t.qubit == 1 and t.target_qubit == 3 and t.control == 2
    with pytest.raises(ValueError):
        Op("CNOT", 2, 2)
    with pytest.raises(ValueError):
        Op("X", 2, control=2)
    with pytest.raises(ValueError):
        Op("MZ", 1, control=2)
    with pytest.raises(ValueError):
        OpQC("depolarizing", 0.1, 1, 2).__class__("x", [np.eye(4)], 1)  # 2-qubit channel needs a target
    f = ifOp("MZ", 1, Op("I", 1), Op("X", 1))
    assert f.type == "🔬" and len(f.if01[1]) == 1


def test_twirl_frames_preserve_cnot():
    """Each Pauli frame P_a(x)P_b . CNOT . P_c(x)P_d equals CNOT up to a phase."""
    from bluetangle_gpu.gates import gate
    from bluetangle_gpu.noise import _LIST_CNOT, _LIST_CNOT_REV, _LIST_ECR, _LIST_ECR_REV
    P = {c: gate[c] for c in "IXYZ"}
    for frames, G, rev in ((_LIST_CNOT, gate["CNOT"], False), (_LIST_CNOT_REV, gate["CNOT"], True),
                           (_LIST_ECR, gate["ECR"], False), (_LIST_ECR_REV, gate["ECR"], True)):
        # applied on (least, least+1); the op acts on (q, t) = (least+1, least) when reversed
        Gq = G if not rev else G[np.ix_([0, 2, 1, 3], [0, 2, 1, 3])]
        for f in frames:
            before = np.kron(P[f[0]], P[f[1]])
            after = np.kron(P[f[2]], P[f[3]])
            tot = after @ Gq @ before
            ph = tot[np.nonzero(np.abs(tot) > 1e-12)][0] / Gq[np.nonzero(np.abs(Gq) > 1e-12)][0]
            assert np.allclose(tot, ph * Gq, atol=1e-12), f


@pytest.mark.parametrize("model,p", [("bit_flip", 0.02), ("amplitude_damping", 0.1), ("depolarizing", 0.05)])
def test_mitigation_matrix_equals_reference_construction(oracle, model, p):
    """inv(A) from the single-qubit confusion matrix equals the reference's
    construction (src/ops.jl:472-488): |a><a| through the readout channel on every
    qubit, diagonals as columns, dense inverse."""
    import bluetangle_gpu.mitigation as Mi
    from bluetangle_gpu.noise import noise_model1
    n = 3
    kraus = noise_model1(model, p)
    cols = []
    for a in range(2 ** n):
        rho = np.zeros((2 ** n, 2 ** n), complex)
        rho[a, a] = 1
        for q in range(1, n + 1):
            rho = oracle.dm_channel(rho, kraus, q)
        cols.append(np.real(np.diag(rho)))
    ref = np.linalg.inv(np.array(cols).T)
    assert np.abs(Mi.mitigation_matrix(n, kraus) - ref).max() < 1e-12


QASM_SAMPLE = """OPENQASM 2.0;
include "qelib1.inc";   // boilerplate
qreg q[4]; creg c[4];
h q[0]; sdg q[1]; tdg q[2]; sx q[3];
rx(pi/2) q[0]; u3(0.1,0.2,-pi/4) q[1]; u2(0.3, 0.4) q[2]; u1(0.5) q[3];
cx q[0],q[1]; cz q[2], q[3]; cp(0.25) q[1],q[2];
cu3(0.7,0,0) q[0],q[3]; crz(0.9) q[3],q[0];
swap q[1],q[2]; rzz(0.2) q[0],q[1]; fsim(0.1,0.2) q[2],q[3];
ccx q[0],q[1],q[2]; cswap q[3],q[0],q[1];
barrier q;
reset q[2];
measure q[1] -> c[1];
"""


def test_qasm_reader_follows_reference_rules():
    """Statement by statement as from_qasm (src/qasm.jl:285-421): names, 1-based
    qubits, cx/cz/cp/cu3/crz as controlled one-qubit ops, ccx/cswap with the
    reference's argument order."""
    import bluetangle_gpu.qasm as Q
    ops = Q.from_qasm(QASM_SAMPLE)
    got = [(type(o).__name__, o.name, o.qubit, getattr(o, "target_qubit", -1), getattr(o, "control", -2))
           for o in ops]
    want = [("Op", "H", 1, -1, -2), ("Op", "SD", 2, -1, -2), ("Op", "TD", 3, -1, -2), ("Op", "XSQRT", 4, -1, -2),
            ("Op", "rx(pi/2)", 1, -1, -2), ("Op", "U3(0.1,0.2,-pi/4)", 2, -1, -2), ("Op", "U2(0.3,0.4)", 3, -1, -2),
            ("Op", "U1(0.5)", 4, -1, -2), ("Op", "X", 2, -1, 1), ("Op", "Z", 4, -1, 3), ("Op", "U1(0.25)", 3, -1, 2),
            ("Op", "ry(0.7)", 4, -1, 1), ("Op", "rz(0.9)", 1, -1, 4), ("Op", "SWAP", 2, 3, -2),
            ("Op", "RZZ(0.2)", 1, 2, -2), ("Op", "FSIM(0.1,0.2)", 3, 4, -2), ("Op", "CX", 1, 3, 2),
            ("Op", "SWAP", 1, 2, 4)]  # cswap a,b,c -> Op("CSWAP", b, a, c): SWAP(b, c) controlled by a
    assert got[:len(want)] == want
    assert type(ops[-2]).__name__ == "OpQC" and ops[-1].name == "MZ" and ops[-1].qubit == 2
    with pytest.raises(ValueError):
        Q.from_qasm("qreg q[2]; foo q[0];")


def test_variational_parameter_binding():
    """Parameters are consumed in op order, as many per op as its matrix function
    takes (_find_argument_number, src/vqa.jl:224-235); a wrong count is an error."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.vqa as V

    def u2(a, b):
        return np.array([[1, -np.exp(1j * b)], [np.exp(1j * a), np.exp(1j * (a + b))]]) / np.sqrt(2)

    def ry(t):
        return np.array([[np.cos(t / 2), -np.sin(t / 2)], [np.sin(t / 2), np.cos(t / 2)]])

    ops = [bt.Op("RY", ry, 1), bt.Op("H", 2), bt.Op("U2", u2, 2), bt.Op("CNOT", 1, 2), bt.Op("RY", ry, 2)]
    assert V.arg_counts(ops) == [1, 0, 2, 0, 1]
    p = np.array([0.1, 0.2, 0.3, 0.4])
    b = V._bound(ops, V.arg_counts(ops), p)
    assert np.allclose(b[0][1], ry(0.1)) and b[1][1] is None and np.allclose(b[2][1], u2(0.2, 0.3))
    assert np.allclose(b[4][1], ry(0.4))
    with pytest.raises(ValueError):
        V._bound(ops, V.arg_counts(ops), p[:3])


def _host_plan(lib, n, thetas, variable=()):
    """A complex64 plan of RY(theta) RZ(theta) on every qubit and a CNOT ladder,
    planned without a device (the library plans and encodes passes on the host)."""
    import ctypes
    from bluetangle_gpu import _lib as L
    P = ctypes.c_void_p
    p = P()
    L.check(lib.bt_plan_create(None, n, L.BT_REPR_SV, L.BT_PREC_C64, ctypes.byref(p)))
    adds = []
    for q in range(1, n + 1):
        for th in thetas:
            c, s = math.cos(th / 2), math.sin(th / 2)
            for m in (np.array([[c, -s], [s, c]]), np.diag([np.exp(-0.5j * th), np.exp(0.5j * th)])):
                mm = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).T)
                qs = np.array([q], dtype=np.int32)
                L.check(lib.bt_plan_add_matrix(p, 1, qs.ctypes.data_as(P), mm.ctypes.data_as(P), 0, None))
                adds.append(len(adds))
    cx = np.ascontiguousarray(np.eye(4, dtype=np.complex128)[[0, 1, 3, 2]].T)
    for q in range(1, n):
        qs = np.array([q, q + 1], dtype=np.int32)
        L.check(lib.bt_plan_add_matrix(p, 2, qs.ctypes.data_as(P), cx.ctypes.data_as(P), 0, None))
    if variable:
        idx = np.ascontiguousarray(variable, dtype=np.int64)
        L.check(lib.bt_plan_set_variable(p, len(idx), idx.ctypes.data_as(P)))
    return p, adds


def _compiled(lib, p):
    import ctypes
    f, b = ctypes.c_double(), ctypes.c_double()
    return lib.bt_plan_cost(p, ctypes.byref(f), ctypes.byref(b)) == 0


def _update(lib, p, adds, th):
    """every rotation and diagonal rewritten at angle th"""
    import ctypes
    P = ctypes.c_void_p
    c, s = math.cos(th / 2), math.sin(th / 2)
    mats = []
    for i in adds:
        m = np.array([[c, -s], [s, c]]) if i % 2 == 0 else np.diag([np.exp(-0.5j * th), np.exp(0.5j * th)])
        mats.append(np.asarray(m, dtype=np.complex128).T.ravel())
    buf = np.ascontiguousarray(np.concatenate(mats))
    idx = np.ascontiguousarray(adds, dtype=np.int64)
    from bluetangle_gpu import _lib as L
    L.check(lib.bt_plan_set_matrices(p, len(idx), idx.ctypes.data_as(P), buf.ctypes.data_as(P)))


def test_plan_angle_updates_never_recompile(monkeypatch):
    """In-place angle updates keep the compiled passes (no recompile per update):
    a gate's encoding does not depend on its angle once it is variable, which it
    becomes at its first update (one recompile) or by bt_plan_set_variable before
    compiling (none).  Planned on the host; the specialised kernels are not built."""
    monkeypatch.setenv("BTGPU_NO_JIT", "1")
    from bluetangle_gpu import _lib as L
    lib = L.lib()
    n = 15
    # angles on both sides of |cos| = |sin|: the factored rotation form would flip
    p, adds = _host_plan(lib, n, [0.4])
    try:
        L.check(lib.bt_plan_compile(p, 0))
        assert _compiled(lib, p)
        _update(lib, p, adds, 2.9)   # first update: the gates turn variable, one recompile
        assert not _compiled(lib, p)
        L.check(lib.bt_plan_compile(p, 0))
        for th in (0.3, 2.8, 1.1, 3.0, 0.05):
            _update(lib, p, adds, th)
            assert _compiled(lib, p), th
    finally:
        lib.bt_plan_free(p)
    p, adds = _host_plan(lib, n, [0.4], variable=list(range(2 * n)))
    try:
        L.check(lib.bt_plan_compile(p, 0))
        for th in (2.9, 0.3, 2.8, 1.1):
            _update(lib, p, adds, th)
            assert _compiled(lib, p), th
    finally:
        lib.bt_plan_free(p)


def test_paramshift_member_matrices():
    """Per-member matrices of the batched parameter-shift evaluations: member 0
    is the unshifted circuit, members 2i + 1 / 2i + 2 shift parameter i's op by
    +/- (its other variable ops keep their base matrices)."""
    from bluetangle_gpu.vqa import paramshift_member_mats
    base = [(None, None), ("a", np.full((2, 2), 1.0)), (None, None), ("b", np.full((2, 2), 2.0))]
    var = [1, 3]
    shifted = [(np.full((2, 2), 10.0), np.full((2, 2), 11.0)), (np.full((2, 2), 20.0), np.full((2, 2), 21.0)),
               (np.full((2, 2), 30.0), np.full((2, 2), 31.0))]
    owner = [1, 3, 3]  # op 3 holds two parameters
    mm = paramshift_member_mats(base, var, shifted, owner, range(7))
    firsts = [[float(m[0, 0]) for m in member] for member in mm]
    assert firsts == [[1, 2], [10, 2], [11, 2], [1, 20], [1, 21], [1, 30], [1, 31]]


def test_reference_arm_maps_no_engine_library():
    """bench.py's reference arm builds its circuit with the host-only generator and
    times the oracle: the process maps no libbtgpu.so (the package loads the
    library at its first engine call, not at import)."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, sys.argv[1]); import bench; bench.layers_of(10, 4, 1); "
            "import bluetangle_gpu, bluetangle_gpu.circuits; "
            "maps = open('/proc/self/maps').read(); print('MAPPED' if 'libbtgpu' in maps else 'CLEAN')")
    r = subprocess.run([sys.executable, "-c", code, root], capture_output=True, text=True, timeout=300, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip().endswith("CLEAN"), r.stdout


def test_member_groups_share_one_slot_list():
    """Groups of members with different circuits in one batch: concat_members and
    concat_slots leave each group's slots in order with the other group idle;
    explicit_noise writes a NoiseModel's channels out as OpQC ops (the slots equal
    those build_slots adds under the model); grouped_bytes counts only the members
    that act in each group of ops."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    from bluetangle_gpu.noise import NoiseModel
    n = 4
    noise = NoiseModel(bt.Noise1("depolarizing", 0.05), bt.Noise2("depolarizing", 0.08))
    main = T.member_programs([[bt.Op("H", 1), bt.Op("CNOT", 1, 2)]], n, 3, measure_prob=0.5,
                             measure_rng=np.random.default_rng(1))
    copy_ops = [bt.Op("CNOT", q, q + 1) for q in range(1, n)]
    copies = T.member_programs([copy_ops], n, 2, zne_ids=[0, 1], twirl=True, frame_rng=np.random.default_rng(2))
    a = T.build_slots(T.explicit_noise(copies, noise))
    b = T.build_slots(copies, noise)
    assert [s.kind for s in a] == [s.kind for s in b]
    for sa, sb in zip(a, b):
        for ia, ib in zip(sa.items, sb.items):
            assert (ia is None) == (ib is None)
            if ia is not None and sa.kind == "channel":
                assert ia[1] == ib[1] and all(np.array_equal(x, y) for x, y in zip(ia[0], ib[0]))
    s1 = T.build_slots(T.concat_members(main, copies))
    s2 = T.concat_slots((T.build_slots(main), 3), (T.build_slots(copies), 2))
    assert len(s1) == len(s2)
    for x, y in zip(s1, s2):
        assert x.kind == y.kind and [i is None for i in x.items] == [i is None for i in y.items]
        on = [m for m, it in enumerate(x.items) if it is not None]
        assert on and (max(on) < 3 or min(on) >= 3)  # each slot belongs to one group
    member = 2 ** n * 8
    only_main = T.grouped_bytes(T.build_slots(main), n, 3)
    only_copies = T.grouped_bytes(T.build_slots(copies), n, 2)
    both = T.grouped_bytes(s2, n, 5)
    assert both <= only_main + only_copies and both % member == 0 and both > 0
