"""The reference's own test properties (BlueTangle.jl test/runtests.jl), run
through the GPU engine with the mirrored API, plus the workload configurations
checked against the oracle."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def oracle_apply(oracle, psi, op):
    if op.q == 1:
        return oracle.hilbert1(psi, op.mat, op.qubit, op.control)
    return oracle.hilbert2(psi, op.mat, op.qubit, op.target_qubit, op.control)


def test_nonlocal_cnot_equals_controlled_x(ctx):
    """test/runtests.jl:10-17 on every basis state of N=6."""
    import bluetangle_gpu as bt
    N = 6
    a = bt.zero_state(N)
    b = bt.zero_state(N)
    for idx in range(2 ** N):
        a.set_basis(idx)
        b.set_basis(idx)
        bt.apply(a, bt.Op("CNOT", 2, 5))
        bt.apply(b, bt.Op("X", 5, control=2))
        assert np.array_equal(a.to_numpy(), b.to_numpy())


def test_kraus_probabilities_three_ways(ctx, oracle):
    """test/runtests.jl:19-35: partial-trace probabilities == ||E psi||^2 == op.prob."""
    import bluetangle_gpu as bt
    rng = np.random.default_rng(31)
    N = 6
    psi = rstate(rng, N)
    st = bt.state_from(psi)
    nm = bt.QuantumChannel(2, "depolarizing", 0.5)
    probs = bt.channel_probs(st, nm.kraus, 2, 3)
    probs2 = []
    for K in nm.kraus:
        t = bt.state_from(psi)
        bt.apply_matrix(t, K, [2, 3])
        probs2.append(sum(np.abs(t.to_numpy()) ** 2))
    op = bt.OpQC("my quantum channel", nm.kraus, 2, 3)
    probs3 = bt.channel_probs(st, op.kraus, op.qubit, op.target_qubit)
    assert np.allclose(probs, probs2, atol=1e-14) and np.allclose(probs, probs3, atol=1e-14)


def test_circuit_unitary_n10_depth50(ctx, oracle):
    """test/runtests.jl:54-73: N=10, depth 50 random_ops, atol 1e-12."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(32)
    N = 10
    ops = C.random_ops(N, 50, rng)
    psi = rstate(rng, N)
    st = bt.state_from(psi)
    bt.apply(ops, st)
    ref = psi
    for o in ops:
        ref = oracle_apply(oracle, ref, o)
    assert np.abs(st.to_numpy() - ref).max() < 1e-12


def test_density_matrix_vs_state_and_trajectory_mean(ctx, oracle):
    """test/runtests.jl:89-133: rho == psi psi' (1e-10); mean over 1000 noisy
    trajectories of sum <T_i> == DM value (atol 10/1000).  The trajectories run as
    one batched state of 1000 members."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(33)
    N = 4
    ops = C.random_ops(N, 20, rng)
    st = bt.apply(ops, bt.zero_state(N))
    rho = bt.apply(ops, bt.zero_rho(N))
    psi = st.to_numpy()
    assert np.abs(np.outer(psi, psi.conj()) - rho.to_numpy()).max() < 1e-10
    nm = bt.NoiseModel("depolarizing", 0.1)
    traj = bt.apply(ops, bt.zero_state(N, batch=1000), noise=nm, rng=np.random.default_rng(34))
    rho_n = bt.apply(ops, bt.zero_rho(N), noise=nm)
    Tm = bt.gate["T"]
    mag = []
    for m in range(1000):
        p = traj.to_numpy(m)
        mag.append(sum(oracle.expect_matrix_sv(p, Tm, [q]) for q in range(1, N + 1)))
    mag_dm = sum(bt.expect(rho_n, bt.Op("T", q)) for q in range(1, N + 1))
    assert abs(np.mean(mag) - mag_dm) < 10 / 1000 * 4


def test_opqc_equals_noise_model_on_rho(ctx):
    """test/runtests.jl:136-160: explicit OpQC after each op == NoiseModel."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(35)
    N = 3
    ops = C.random_ops(N, 10, rng)
    p = 0.01
    nm = bt.NoiseModel("depolarizing", p)
    r1 = bt.zero_rho(N)
    r2 = bt.zero_rho(N)
    for o in ops:
        bt.apply(r1, o)
        c = bt.OpQC("depolarizing", p, o.qubit) if o.q == 1 else bt.OpQC("depolarizing", p, o.qubit, o.target_qubit)
        bt.apply(r1, c)
        bt.apply(r2, o, noise=nm)
    assert np.abs(r1.to_numpy() - r2.to_numpy()).max() < 1e-14


def test_mid_circuit_measure_reset_exact(ctx):
    """test/runtests.jl:195-231 (statevector backend)."""
    import bluetangle_gpu as bt
    Op, ifOp = bt.Op, bt.ifOp
    ops_reset = [Op("X", 1), Op("RES", 1), Op("MZ", 1)]
    ops_ifop = [Op("X", 1), ifOp("MZ", 1, Op("I", 1), Op("X", 1))]
    ops_mid = [Op("X", 1), Op("X", 2), Op("CX", 2, 3), Op("CX", 1, 2), Op("X", 2), Op("MZ", 2), Op("RES", 2),
               Op("CX", 2, 3), Op("CX", 1, 2), Op("CX", 2, 3), Op("X", 1)]
    for seed in range(5):
        rng = np.random.default_rng(seed)
        assert bt.run(ops_reset, 1, rng=rng)[0] == [0]
        assert bt.run(ops_ifop, 1, rng=rng)[0] == [1]
        assert bt.run(ops_mid, 1, rng=rng)[0] == [1]
        _, m = bt.apply(ops_reset, bt.zero_state(1), track_measurements=True, rng=rng)
        assert m == [0]
        _, m = bt.apply(ops_ifop, bt.zero_state(1), track_measurements=True)
        assert m == [1]
        _, m = bt.apply(ops_mid, bt.zero_state(3), track_measurements=True)
        assert m == [1]


def test_noisy_circuit_with_measurements_matches_oracle_under_same_draws(ctx, oracle, kref):
    """test/runtests.jl:233-285 compares two backends under one seed; here the GPU
    engine and the oracle consume the same uniform draws."""
    import bluetangle_gpu as bt
    Op = bt.Op
    ops = [Op("H", 1), Op("CX", 1, 2), Op("RY(0.37)", 1), Op("RZ(0.19)", 2), Op("MZ", 1), Op("X", 2), Op("MZ", 2)]
    nm = bt.NoiseModel("depolarizing", 0.03)
    k1 = kref.noise_model("depolarizing", 0.03)
    k2 = kref.noise_model("depolarizing", 0.03, True)
    for seed in range(20):
        st, mids = bt.apply(ops, bt.zero_state(2), noise=nm, track_measurements=True,
                            rng=np.random.default_rng(1000 + seed))
        r = np.random.default_rng(1000 + seed)
        psi = np.array([1, 0, 0, 0], complex)
        rmids = []
        for o in ops:
            if o.type == "🔬":
                psi, ind, _ = oracle.born_measure_z(psi, o.qubit, u=r.random(1)[0])
                rmids.append(ind)
                continue
            psi = oracle_apply(oracle, psi, o)
            if o.q == 1:
                psi, _, _ = oracle.channel_traj(psi, k1, o.qubit, u=r.random(1)[0])
            else:
                psi, _, _ = oracle.channel_traj(psi, k2, o.qubit, o.target_qubit, u=r.random(1)[0])
        assert mids == rmids
        assert np.abs(st.to_numpy() - psi).max() < 1e-12


# ---------------------------------------------------------------- workload configurations
def test_config_statevector_12q_brickwork(ctx, oracle):
    """12-qubit complex128 brickwork depth 20 from |0..0>: state within 1e-12,
    <Z_i> for all i, 10^4 shots (chi-square against |psi|^2)."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    from scipy import stats
    rng = np.random.default_rng(41)
    n = 12
    ops = C.brickwork(n, 20, rng)
    st = bt.apply(ops, bt.zero_state(n))
    ref = np.zeros(2 ** n, complex)
    ref[0] = 1
    for o in ops:
        ref = oracle_apply(oracle, ref, o)
    assert np.abs(st.to_numpy() - ref).max() < 1e-12
    z = bt.expect(st, "Z")
    zr = [oracle.expect_pauli_sv(ref, 0, 1 << (n - q)) for q in range(1, n + 1)]
    assert np.abs(np.array(z) - zr).max() < 1e-12
    shots = bt.sample(st, 10 ** 4, seed=5)
    p = np.abs(ref) ** 2
    # chi-square over outcome bins pooled so that every expected count >= 5
    order = np.argsort(p)
    cnt = np.bincount(shots, minlength=2 ** n)[order].astype(float)
    exp = (p[order] * 10 ** 4)
    edges = np.searchsorted(np.cumsum(exp), np.arange(5, exp.sum(), 5))
    oc = np.add.reduceat(cnt, np.unique(np.r_[0, edges[edges < len(exp)]]))
    ec = np.add.reduceat(exp, np.unique(np.r_[0, edges[edges < len(exp)]]))
    _, pval = stats.chisquare(oc, ec * oc.sum() / ec.sum())
    assert pval > 1e-4


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 5e-5)])
def test_config_density_matrix_noisy_brickwork(ctx, oracle, kref, prec, tol):
    """10-qubit density matrix, depth 16 with depolarizing + amplitude damping after
    every gate and a 2% readout flip; run here at 6 qubits depth 6 for the dense
    oracle, then properties at the full 10 qubits depth 16."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(42)
    n = 6
    ops = C.noisy_brickwork_dm(n, 6, rng)
    rho = bt.zero_rho(n, prec)
    bt.apply(ops, rho)
    flip = kref.noise_model("bit_flip", 0.02)
    for q in range(1, n + 1):
        bt.apply_channel(rho, flip, q)
    ref = np.zeros((2 ** n, 2 ** n), complex)
    ref[0, 0] = 1
    for o in ops:
        if isinstance(o, bt.OpQC):
            ref = oracle.dm_channel(ref, o.kraus, o.qubit, o.target_qubit if o.q == 2 else -1)
        elif o.q == 1:
            ref = oracle.dm_hilbert1(ref, o.mat, o.qubit)
        else:
            ref = oracle.dm_hilbert2(ref, o.mat, o.qubit, o.target_qubit)
    for q in range(1, n + 1):
        ref = oracle.dm_channel(ref, flip, q)
    assert np.abs(rho.to_numpy() - ref).max() < tol
    zz = [bt.correlation(rho, "Z,Z", [i, i + 1]) for i in range(1, n)]
    zzr = [oracle.expect_pauli_dm(ref, 0, (1 << (n - i)) | (1 << (n - i - 1))) for i in range(1, n)]
    assert np.abs(np.array(zz) - zzr).max() < max(tol, 1e-12) * 10
    # full size: trace 1 and hermiticity preserved
    n = 10
    ops = C.noisy_brickwork_dm(n, 16, np.random.default_rng(43))
    rho = bt.apply(ops, bt.zero_rho(n, prec))
    tr = sum(bt.expect(rho, "Z"))  # finite
    assert np.isfinite(tr)
    R = rho.to_numpy()
    # T/TD are rounded to 10 significant digits in the reference (src/gates.jl:32-33),
    # so |T[2,2]|^2 = 1 + 1.0e-10: the trace grows by up to that per T gate
    nT = sum(1 for o in ops if getattr(o, "name", "") == "T")
    assert abs(np.trace(R) - 1) < (1e-12 + nT * 1.01e-10 if prec == "c128" else 1e-4)
    assert np.abs(R - R.conj().T).max() < (1e-13 if prec == "c128" else 1e-6)
