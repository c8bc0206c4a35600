"""Batched Monte-Carlo trajectories with uneven per-member programs (ZNE
repetitions, Pauli-twirl frames, random mid-circuit measurements, Kraus
branches) against the oracle replaying each member with the same draws."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tfim_cnot_steps(n, steps, dt, h, p1=0.02, p2=0.05, gamma=0.03):
    """TFIM Trotter steps in the CNOT.RZ.CNOT form with explicit channels after
    every gate (the form the reference's twirl and ZNE act on)."""
    import bluetangle_gpu as bt
    out = []
    for _ in range(steps):
        st = []
        for q in range(1, n):
            for op in (bt.Op("CNOT", q, q + 1), bt.Op(f"RZ({2 * dt!r})", q + 1), bt.Op("CNOT", q, q + 1)):
                st.append(op)
                if op.q == 2:
                    st += [bt.OpQC("depolarizing", p2, q, q + 1), bt.OpQC("amplitude_damping", gamma, q)]
                else:
                    st += [bt.OpQC("depolarizing", p1, q + 1), bt.OpQC("amplitude_damping", gamma, q + 1)]
        for q in range(1, n + 1):
            st += [bt.Op(f"RX({float(2 * h[q - 1] * dt)!r})", q), bt.OpQC("amplitude_damping", gamma, q)]
        out.append(st)
    return out


def replay(oracle, slots, B, n, rng, kref):
    psis = []
    for m in range(B):
        p = np.zeros(2 ** n, complex)
        p[0] = 1
        psis.append(p)
    recs = [[] for _ in range(B)]
    for sl in slots:
        if sl.kind == "gate":
            for m, it in enumerate(sl.items):
                if it is not None:
                    psis[m] = oracle.apply_k(psis[m], it[0], it[1], it[2])
        elif sl.kind == "channel":
            u = rng.random(B)
            for m, it in enumerate(sl.items):
                if it is not None:
                    kr, qs = it
                    t = qs[1] if len(qs) == 2 else -1
                    psis[m], _, _ = oracle.channel_traj(psis[m], kr, qs[0], t, u=u[m])
        else:
            u = rng.random(B)
            for m, it in enumerate(sl.items):
                if it is not None:
                    psis[m], ind, _ = oracle.born_measure_z(psis[m], it[1], u=u[m])
                    recs[m].append(ind)
    return psis, recs


@pytest.mark.parametrize("twirl", [False, True])
def test_trajectories_uneven_programs_match_oracle(ctx, oracle, kref, twirl):
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 5, 6
    h = np.random.default_rng(3).uniform(0.5, 1.5, n)
    steps = tfim_cnot_steps(n, 2, 0.3, h)
    member_ops = T.member_programs(steps, n, B, zne_ids=[0, 1, 2, 0, 1, 2], twirl=twirl,
                                   frame_rng=np.random.default_rng(7), measure_prob=0.3,
                                   measure_rng=np.random.default_rng(8))
    slots = T.build_slots(member_ops)
    st = bt.zero_state(n, "c128", batch=B)
    recs = T.run_slots(st, slots, rng=np.random.default_rng(11))
    ref, rrecs = replay(oracle, slots, B, n, np.random.default_rng(11), kref)
    for m in range(B):
        assert recs[m] == rrecs[m]
        assert np.abs(st.to_numpy(m) - ref[m]).max() < 1e-12
    assert sum(len(r) for r in recs) > 0  # some members were measured


@pytest.mark.parametrize("executor", ["shared", "grouped"])
@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
@pytest.mark.parametrize("twirl", [False, True])
def test_program_uneven_programs_match_oracle(ctx, oracle, kref, prec, tol, twirl, executor):
    """Programs on both executors (one CTA per member in shared memory; grouped
    ops within two qubits decided from one reduced matrix) against the oracle
    replaying each member with the same draws: ZNE repetitions, twirl frames,
    random mid-circuit measurements, Kraus branches.  complex64 tolerance: float32
    rounding over ~150 ops of a 5-qubit member."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 5, 6
    h = np.random.default_rng(3).uniform(0.5, 1.5, n)
    steps = tfim_cnot_steps(n, 2, 0.3, h)
    member_ops = T.member_programs(steps, n, B, zne_ids=[0, 1, 2, 0, 1, 2], twirl=twirl,
                                   frame_rng=np.random.default_rng(7), measure_prob=0.3,
                                   measure_rng=np.random.default_rng(8))
    slots = T.build_slots(member_ops)
    assert T.program_supported(slots, n, prec)
    st = bt.zero_state(n, prec, batch=B)
    prog, _ = T.compile_program(slots, n, B, prec, unitary_mix=False)
    prog.set_executor(executor)
    recs = prog.run(st, rng=np.random.default_rng(11))
    ref, rrecs = replay(oracle, slots, B, n, np.random.default_rng(11), kref)
    for m in range(B):
        assert recs[m] == rrecs[m]
        assert np.abs(st.to_numpy(m) - ref[m]).max() < tol
    assert sum(len(r) for r in recs) > 0


def test_program_equals_slots_engine(ctx):
    """Both trajectory engines with the same explicit draws give the same members
    and records (8 qubits, 32 members, measurements and 2-qubit channels)."""
    import bluetangle_gpu.trajectories as T
    n, B = 8, 32
    h = np.random.default_rng(4).uniform(0.5, 1.5, n)
    steps = tfim_cnot_steps(n, 2, 0.2, h)
    kw = dict(zne_ids=[i % 3 for i in range(B)], twirl=True, measure_prob=0.1, prec="c128")
    a, ra = T.run_trajectories(steps, n, B, rng=np.random.default_rng(5), frame_rng=np.random.default_rng(6),
                               measure_rng=np.random.default_rng(7), engine="program", **kw)
    b, rb = T.run_trajectories(steps, n, B, rng=np.random.default_rng(5), frame_rng=np.random.default_rng(6),
                               measure_rng=np.random.default_rng(7), engine="slots", **kw)
    assert ra == rb
    for m in range(B):
        assert np.abs(a.to_numpy(m) - b.to_numpy(m)).max() < 1e-12


def test_program_set_gate_matches_fresh_compile(ctx):
    """New gate matrices between runs (variational angles) give what a program
    compiled with those matrices gives."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 6, 4
    rng = np.random.default_rng(1)

    def ops(theta):
        out = []
        for q in range(1, n + 1):
            out += [bt.Op(f"RY({float(theta[q - 1])!r})", q), bt.OpQC("amplitude_damping", 0.05, q)]
        for q in range(1, n):
            out += [bt.Op("CNOT", q, q + 1), bt.OpQC("depolarizing", 0.02, q, q + 1)]
        return out

    t0, t1 = rng.uniform(0, 3, n), rng.uniform(0, 3, n)
    slots0 = T.build_slots(T.member_programs([ops(t0)], n, B))
    slots1 = T.build_slots(T.member_programs([ops(t1)], n, B))
    prog, gate_ops = T.compile_program(slots0, n, B, "c128", unitary_mix=False)
    st = bt.zero_state(n, "c128", batch=B)
    prog.run(st, rng=np.random.default_rng(2))
    for i, sl in enumerate(slots1):
        if gate_ops[i] is not None and sl.items[0][0].shape[0] == 2:
            prog.set_gate(gate_ops[i], sl.items[0][0])
    st.set_zero()
    prog.run(st, rng=np.random.default_rng(3))
    fresh, _ = T.compile_program(slots1, n, B, "c128", unitary_mix=False)
    st2 = bt.zero_state(n, "c128", batch=B)
    fresh.run(st2, rng=np.random.default_rng(3))
    for m in range(B):
        assert np.abs(st.to_numpy(m) - st2.to_numpy(m)).max() < 1e-14


def test_program_no_branch_leaves_member(ctx):
    """A Kraus set whose probabilities sum below u selects no branch (the
    reference's _weighted_sample returns nothing): the run reports it and that
    member keeps its state; the other members proceed."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 3, 2
    prog = T.Program(n, B, "c128")
    prog.add_gate(np.array([[1, 1], [1, -1]]) / np.sqrt(2), [1])
    prog.add_channel([np.sqrt(0.5) * np.eye(2)], [2])  # probabilities sum to 0.5
    st = bt.zero_state(n, "c128", batch=B)

    class Draws:
        def random(self, shape):
            return np.array([[0.25, 0.75]]).reshape(shape)

    with pytest.raises(bt.BTError) as e:
        prog.run(st, rng=Draws())
    assert e.value.code == -7
    plus = np.zeros(2 ** n, complex)
    plus[0] = plus[4] = 1 / np.sqrt(2)
    assert np.abs(st.to_numpy(1) - plus).max() < 1e-15      # untouched
    assert np.abs(st.to_numpy(0) - plus).max() < 1e-15      # K/sqrt(p) = I on a normalised member


@pytest.mark.parametrize("engine", ["program", "slots"])
def test_trajectories_device_rng_statistics(ctx, oracle, engine):
    """On-device Philox draws (with the unitary-mixture shortcut for depolarizing
    channels): the mean over trajectories of <Z_1> matches the density matrix."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 4, 2000
    h = [1.0, 0.8, 1.2, 0.9]
    steps = tfim_cnot_steps(n, 2, 0.25, h, p1=0.05, p2=0.1, gamma=0.05)
    st, _ = T.run_trajectories(steps, n, B, prec="c128", engine=engine, seed=17)
    zs = bt.expect(st, "Z", member=-1)[:, 0]
    rho = bt.zero_rho(n)
    for step in steps:
        bt.apply(step, rho)
    z_dm = bt.expect(rho, "Z")[0]
    assert abs(zs.mean() - z_dm) < 4 * zs.std() / np.sqrt(B) + 1e-3


def test_grouped_program_large_members_equal_slots_engine(ctx):
    """Members larger than shared memory (16 qubits, complex64) run grouped; with
    the same explicit draws they make the slots engine's decisions (records equal)
    and end in the same states (complex64 rounding)."""
    import bluetangle_gpu.trajectories as T
    n, B = 16, 12
    h = np.random.default_rng(9).uniform(0.5, 1.5, n)
    steps = tfim_cnot_steps(n, 1, 0.2, h)
    kw = dict(zne_ids=[i % 3 for i in range(B)], twirl=True, measure_prob=0.1, prec="c64")
    a, ra = T.run_trajectories(steps, n, B, rng=np.random.default_rng(5), frame_rng=np.random.default_rng(6),
                               measure_rng=np.random.default_rng(7), engine="program", **kw)
    b, rb = T.run_trajectories(steps, n, B, rng=np.random.default_rng(5), frame_rng=np.random.default_rng(6),
                               measure_rng=np.random.default_rng(7), engine="slots", **kw)
    assert ra == rb
    assert sum(len(r) for r in ra) > 0
    for m in range(B):
        assert np.abs(a.to_numpy(m) - b.to_numpy(m)).max() < 2e-5


@pytest.mark.parametrize("executor", ["shared", "grouped"])
def test_trajectories_and_copies_in_one_program(ctx, oracle, kref, executor):
    """Monte-Carlo trajectories and Pauli-twirled ZNE copies of another circuit in
    one program (one launch sequence for the whole batch): the members of each
    group are idle at the other group's slots (identity gates, skipped channels
    and measurements) and equal the oracle replaying each member with the same
    draws; with the grouped executor idle members are neither read nor written."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    from bluetangle_gpu.noise import NoiseModel
    n, B, NC = 5, 4, 3
    h = np.random.default_rng(3).uniform(0.5, 1.5, n)
    steps = tfim_cnot_steps(n, 1, 0.3, h)
    main = T.member_programs(steps, n, B, measure_prob=0.3, measure_rng=np.random.default_rng(8))
    copy_ops = [bt.Op("CNOT", q, q + 1) for q in range(1, n)] + [bt.Op("RX(0.7)", q) for q in range(1, n + 1)]
    copies = T.member_programs([copy_ops], n, NC, zne_ids=[0, 1, 2], twirl=True,
                               frame_rng=np.random.default_rng(7))
    noise = NoiseModel(bt.Noise1("depolarizing", 0.05), bt.Noise2("depolarizing", 0.08))
    members = T.concat_members(main, T.explicit_noise(copies, noise))
    slots = T.build_slots(members)
    st = bt.zero_state(n, "c128", batch=B + NC)
    prog, _ = T.compile_program(slots, n, B + NC, "c128", unitary_mix=False)
    prog.set_executor(executor)
    recs = prog.run(st, rng=np.random.default_rng(11))
    ref, rrecs = replay(oracle, slots, B + NC, n, np.random.default_rng(11), kref)
    for m in range(B + NC):
        assert recs[m] == rrecs[m]
        assert np.abs(st.to_numpy(m) - ref[m]).max() < 1e-12, m
    # the copies' own circuit: the same as building their slots alone under the model
    alone = T.build_slots(copies, noise)
    assert sum(len([i for i in s.items if i is not None]) for s in alone) == \
        sum(len([i for i in s.items[B:] if i is not None]) for s in slots)


def test_grouped_program_one_qubit_groups(ctx):
    """A group of ops on one qubit (a measurement between two-qubit gates on other
    qubits) in the grouped executor: its reduced matrices (2 x 2 per member) are
    read per member, so every member's outcome and state equal the one-CTA
    executor's with the same draws."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 5, 9

    def runitary(rng):
        q, r = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
        return q * (np.diag(r) / np.abs(np.diag(r)))

    prog = {}
    for ex in ("shared", "grouped"):
        p = T.Program(n, B, "c128")
        rng = np.random.default_rng(4)
        for q in range(1, n + 1):
            p.add_gate([runitary(rng) for _ in range(B)], [q])
        p.add_gate(np.eye(4)[[0, 1, 3, 2]], [1, 2])
        p.add_measure(5)
        p.add_gate(np.eye(4)[[0, 1, 3, 2]], [3, 4])
        p.add_measure(4, [m % 2 for m in range(B)])
        p.add_gate(np.eye(4)[[0, 1, 3, 2]], [1, 2])
        p.set_executor(ex)
        prog[ex] = p
    out = {}
    for ex, p in prog.items():
        st = bt.zero_state(n, "c128", batch=B)
        recs = p.run(st, rng=np.random.default_rng(12))
        out[ex] = (recs, [st.to_numpy(m) for m in range(B)])
    assert out["shared"][0] == out["grouped"][0]
    for a, b in zip(out["shared"][1], out["grouped"][1]):
        assert np.abs(a - b).max() < 1e-12
