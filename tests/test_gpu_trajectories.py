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


def test_trajectories_device_rng_statistics(ctx, oracle):
    """On-device Philox draws (with the unitary-mixture shortcut for depolarizing
    channels): the mean over trajectories of <Z_1> matches the density matrix."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.trajectories as T
    n, B = 4, 2000
    h = [1.0, 0.8, 1.2, 0.9]
    steps = tfim_cnot_steps(n, 2, 0.25, h, p1=0.05, p2=0.1, gamma=0.05)
    st, _ = T.run_trajectories(steps, n, B, prec="c128")
    zs = bt.expect(st, "Z", member=-1)[:, 0]
    rho = bt.zero_rho(n)
    for step in steps:
        bt.apply(step, rho)
    z_dm = bt.expect(rho, "Z")[0]
    assert abs(zs.mean() - z_dm) < 4 * zs.std() / np.sqrt(B) + 1e-3
