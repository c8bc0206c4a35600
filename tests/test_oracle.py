"""The oracle (oracle/btoracle.c) pinned before it is trusted as the checker.

1. Against the golden fixtures frozen from the literal restatement of the
   reference's operator construction (tests/golden/make_golden.py).
2. Against every property the reference's own test suite asserts for this
   path (BlueTangle.jl test/runtests.jl), run on the oracle.
3. Against the outcomes the reference's documentation states for its
   mid-measurement and reset examples (docs/src/examples.md).
"""
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "kron_ref_cases.npz")


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_golden_gates(oracle, gold):
    for i in range(int(gold["ngates"][0])):
        kind = int(gold[f"gate{i}_kind"][0])
        q, t, c = (int(x) for x in gold[f"gate{i}_meta"])
        m, psi = gold[f"gate{i}_mat"], gold[f"gate{i}_in"]
        if kind == 1:
            out = oracle.hilbert1(psi, m, q, c)
        elif kind == 2:
            out = oracle.hilbert2(psi, m, q, t, c)
        else:
            out = oracle.hilbert3(psi, m, q)
        assert np.abs(out - gold[f"gate{i}_out"]).max() < 1e-13, (i, kind, q, t, c)


def test_golden_traces_probs_measure(oracle, gold, kref):
    kr2 = kref.noise_model("depolarizing", 0.5, two_qubit=True)
    kr1 = kref.noise_model("amplitude_damping", 0.3)
    for i in range(int(gold["npt"][0])):
        psi = gold[f"pt{i}_in"]
        q, t = (int(x) for x in gold[f"pt{i}_meta"])
        assert np.abs(oracle.partial_trace2(psi, q, t) - gold[f"pt{i}_rho2"]).max() < 1e-14
        assert np.abs(oracle.partial_trace(psi, [q]) - gold[f"pt{i}_rho1"]).max() < 1e-14
        assert np.abs(oracle.calc_prob(psi, kr2, q, t) - gold[f"pt{i}_probs2"]).max() < 1e-14
        assert np.abs(oracle.calc_prob(psi, kr1, q) - gold[f"pt{i}_probs1"]).max() < 1e-14
        out, br, _ = oracle.channel_traj(psi, kr2, q, t, forced=5)
        assert br == 5 and np.abs(out - gold[f"pt{i}_traj_forced5"]).max() < 1e-13
        out, br, _ = oracle.channel_traj(psi, kr1, q, u=float(gold[f"pt{i}_traj_u"][0]))
        assert br == int(gold[f"pt{i}_traj_branch"][0])
        assert np.abs(out - gold[f"pt{i}_traj_out"]).max() < 1e-13
        for o in (0, 1):
            out, ind, p0 = oracle.born_measure_z(psi, q, forced=o)
            assert ind == o and abs(p0 - gold[f"pt{i}_p0"][0]) < 1e-14
            assert np.abs(out - gold[f"pt{i}_meas{o}"]).max() < 1e-13
            assert np.array_equal(out == 0, gold[f"pt{i}_meas{o}"] == 0)


def test_golden_density_and_observables(oracle, gold, kref):
    rho = gold["dm_in"]
    U = gold["dm_U"]
    assert np.abs(oracle.dm_hilbert2(rho, U, 3, 1) - gold["dm_gate_out"]).max() < 1e-13
    kr2 = kref.noise_model("depolarizing", 0.5, two_qubit=True)
    kr1 = kref.noise_model("amplitude_damping", 0.3)
    assert np.abs(oracle.dm_channel(rho, kr2, 1, 2) - gold["dm_ch2_out"]).max() < 1e-13
    assert np.abs(oracle.dm_channel(rho, kr1, 3) - gold["dm_ch1_out"]).max() < 1e-13
    psi = gold["obs_in"]
    n = 5
    from kron_ref import GATE

    def masks(names, qs, nn):
        x = z = 0
        for s, q in zip(names, qs):
            b = 1 << (nn - q)
            x |= b if s in "XY" else 0
            z |= b if s in "ZY" else 0
        return x, z
    strings = [(["Z"], [3]), (["X", "Y"], [1, 4]), (["Z", "Z"], [2, 3]), (["Y", "X", "Z"], [5, 1, 2])]
    for (names, qs), v in zip(strings, gold["obs_vals"][:4]):
        assert abs(oracle.expect_pauli_sv(psi, *masks(names, qs, n)) - v) < 1e-13
    # non-Pauli one-qubit observable through the matrix form
    assert abs(oracle.expect_matrix_sv(psi, GATE["T"], [2]) - gold["obs_vals"][4]) < 1e-13
    for (names, qs), v in zip([(["Z"], [1]), (["X", "Z"], [1, 3]), (["Y", "Y"], [2, 3])], gold["obs_rho_vals"]):
        assert abs(oracle.expect_pauli_dm(rho, *masks(names, qs, 3)) - v) < 1e-13
    assert np.array_equal(oracle.sample(gold["samp_in"], gold["samp_u"]), gold["samp_out"])


# ---------------------------------------------------------------- reference test properties
def test_ref_int2bin_bit_order(oracle, kref):
    """int2bin(2,4) == [0,0,1,0] (test/runtests.jl:8): qubit 3 of 4 is bit 1."""
    psi = np.zeros(16, complex)
    psi[0] = 1
    out = oracle.hilbert1(psi, kref.GATE["X"], 3)
    assert np.argmax(np.abs(out)) == 2


def test_ref_nonlocal_cnot_equals_controlled_x(oracle, kref):
    """Op("CNOT",2,5).expand(6) == Op("X",5;control=2).expand(6) (test/runtests.jl:10-17)."""
    N = 6
    assert np.array_equal(kref.hilbert2(N, kref.GATE["CNOT"], 2, 5), kref.hilbert1(N, kref.GATE["X"], 5, control=2))
    for b in range(2 ** N):
        e = np.zeros(2 ** N, complex)
        e[b] = 1
        assert np.array_equal(oracle.hilbert2(e, kref.GATE["CNOT"], 2, 5), oracle.hilbert1(e, kref.GATE["X"], 5, 2))


def test_ref_kraus_probabilities(oracle, kref):
    """probs from partial trace == ||E_k psi||^2 == op.prob (test/runtests.jl:19-35)."""
    rng = np.random.default_rng(3)
    N = 6
    psi = rstate(rng, N)
    kr = kref.noise_model("depolarizing", 0.5, two_qubit=True)
    p1 = oracle.calc_prob(psi, kr, 2, 3)
    p2 = np.array([np.sum(np.abs(oracle.hilbert2(psi, K, 2, 3)) ** 2) for K in kr])
    p3 = kref.calc_prob(psi, kr, 2, 3)
    assert np.allclose(p1, p2, atol=1e-14) and np.allclose(p1, p3, atol=1e-14)


def test_ref_circuit_unitary(oracle, kref):
    """sequential apply == compiled operator (test/runtests.jl:54-73), atol 1e-12."""
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(4)
    N = 7
    ops = C.random_ops(N, 12, rng)
    psi = rstate(rng, N)
    s1 = psi.copy()
    U = np.eye(2 ** N, dtype=complex)
    for o in ops:
        if o.q == 1:
            s1 = oracle.hilbert1(s1, o.mat, o.qubit, o.control)
            U = kref.hilbert1(N, o.mat, o.qubit, o.control) @ U
        else:
            s1 = oracle.hilbert2(s1, o.mat, o.qubit, o.target_qubit, o.control)
            U = kref.hilbert2(N, o.mat, o.qubit, o.target_qubit, o.control) @ U
    assert np.abs(s1 - U @ psi).max() < 1e-12


def test_ref_density_vs_state_and_trajectories(oracle, kref):
    """noiseless rho == psi psi' (atol 1e-10) and the mean of noisy trajectories
    matches the noisy density matrix (atol 10/1000) (test/runtests.jl:89-133)."""
    import bluetangle_gpu.circuits as C
    rng = np.random.default_rng(5)
    N = 4
    ops = C.random_ops(N, 8, rng)
    psi = np.zeros(2 ** N, complex)
    psi[0] = 1
    rho = np.outer(psi, psi.conj())
    for o in ops:
        if o.q == 1:
            psi = oracle.hilbert1(psi, o.mat, o.qubit, o.control)
            rho = oracle.dm_hilbert1(rho, o.mat, o.qubit, o.control)
        else:
            psi = oracle.hilbert2(psi, o.mat, o.qubit, o.target_qubit, o.control)
            rho = oracle.dm_hilbert2(rho, o.mat, o.qubit, o.target_qubit, o.control)
    assert np.abs(np.outer(psi, psi.conj()) - rho).max() < 1e-10
    # noisy: NoiseModel("depolarizing", 0.1) after every gate
    k1 = kref.noise_model("depolarizing", 0.1)
    k2 = kref.noise_model("depolarizing", 0.1, two_qubit=True)
    rho = np.zeros((2 ** N, 2 ** N), complex)
    rho[0, 0] = 1
    for o in ops:
        if o.q == 1:
            rho = oracle.dm_hilbert1(rho, o.mat, o.qubit)
            rho = oracle.dm_channel(rho, k1, o.qubit)
        else:
            rho = oracle.dm_hilbert2(rho, o.mat, o.qubit, o.target_qubit)
            rho = oracle.dm_channel(rho, k2, o.qubit, o.target_qubit)
    zmask = [1 << (N - q) for q in range(1, N + 1)]
    mag_r = sum(oracle.expect_pauli_dm(rho, 0, z) for z in zmask)
    mags = []
    for _ in range(1000):
        s = np.zeros(2 ** N, complex)
        s[0] = 1
        for o in ops:
            if o.q == 1:
                s = oracle.hilbert1(s, o.mat, o.qubit)
                s, _, _ = oracle.channel_traj(s, k1, o.qubit, u=rng.random())
            else:
                s = oracle.hilbert2(s, o.mat, o.qubit, o.target_qubit)
                s, _, _ = oracle.channel_traj(s, k2, o.qubit, o.target_qubit, u=rng.random())
        mags.append(sum(oracle.expect_pauli_sv(s, 0, z) for z in zmask))
    assert abs(np.mean(mags) - mag_r) < 10 / 1000 * N


def test_ref_channel_vs_stochastic_pauli_fidelity(oracle):
    """N=1, depth 20, p=0.01: OpQC("depolarizing") after every op == the op with
    NoiseModel("depolarizing") (t1), and fidelity(rho1, rho0) equals the mean over
    1000 runs of fidelity(rho3, rho0), rho3 the ops with X, Y or Z drawn with
    probability p after each, within atol 100/1000 (t2) (test/runtests.jl:136-193)."""
    import scipy.linalg as sl

    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    from bluetangle_gpu.gates import gate
    rng = np.random.default_rng(134)
    N, p = 1, 0.01
    ops = C.random_ops(N, 20, rng)
    nm = bt.NoiseModel("depolarizing", p)
    psi0 = rstate(rng, N)
    rho0 = np.outer(psi0, psi0.conj())

    def fid(r, s):  # fidelity(rho, sigma) = tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2 (src/tensor.jl:222-229)
        sr = sl.sqrtm(r)
        return float(np.real(np.trace(sl.sqrtm(sr @ s @ sr)) ** 2))

    rho1, rho2 = rho0.copy(), rho0.copy()
    for o in ops:
        rho1 = oracle.dm_hilbert1(rho1, o.mat, o.qubit)
        rho1 = oracle.dm_channel(rho1, bt.OpQC("depolarizing", p, o.qubit).kraus, o.qubit)
        rho2 = oracle.dm_hilbert1(rho2, o.mat, o.qubit)
        rho2 = oracle.dm_channel(rho2, nm.q1.kraus, o.qubit)
    assert np.linalg.norm(rho1 - rho2) < 1e-14
    paulis = [gate["X"], gate["Y"], gate["Z"]]
    avg = 0.0
    for _ in range(1000):
        rho3 = rho0.copy()
        for o in ops:
            rho3 = oracle.dm_hilbert1(rho3, o.mat, o.qubit)
            if rng.random() <= p:
                rho3 = oracle.dm_hilbert1(rho3, paulis[int(rng.integers(0, 3))], o.qubit)
        avg += fid(rho3, rho0) / 1000
    assert abs(fid(rho1, rho0) - avg) < 100 / 1000, (fid(rho1, rho0), avg)


def test_ref_mid_circuit_exact_outcomes(oracle, kref):
    """X,RES,MZ -> [0]; X, ifOp(MZ, I, X) -> [1]; the 11-op circuit -> [1]
    (test/runtests.jl:195-231), for any uniform draw."""
    X = kref.GATE["X"]
    rng = np.random.default_rng(6)
    for _ in range(20):
        s = np.array([1, 0], complex)
        s = oracle.hilbert1(s, X, 1)
        s, ind, _ = oracle.born_measure_z(s, 1, u=rng.random())
        if ind == 1:
            s = oracle.hilbert1(s, X, 1)
        s, ind, _ = oracle.born_measure_z(s, 1, u=rng.random())
        assert ind == 0
        s = oracle.hilbert1(np.array([1, 0], complex), X, 1)
        s, ind, _ = oracle.born_measure_z(s, 1, u=rng.random())
        assert ind == 1
        s = np.zeros(8, complex)
        s[0] = 1
        CX = kref.GATE["CX"]
        s = oracle.hilbert1(s, X, 1)
        s = oracle.hilbert1(s, X, 2)
        s = oracle.hilbert2(s, CX, 2, 3)
        s = oracle.hilbert2(s, CX, 1, 2)
        s = oracle.hilbert1(s, X, 2)
        s, ind, _ = oracle.born_measure_z(s, 2, u=rng.random())
        assert ind == 1


def test_ref_docs_mid_measurement_ghz_or_111(oracle, kref):
    """The reference's documented mid-measurement example: X on qubit 1,
    ifOp("MX", 1, "Z", "H"), CNOT(1,2), CNOT(2,3) ends in (|000> - |111>)/sqrt(2)
    after outcome 0 and in -|111> after outcome 1, each with probability 1/2
    (docs/src/examples.md:257-262, :283; ifOp: rotate by H, measure Z, rotate back,
    then the branch's ops, src/struct.jl:578-594)."""
    H, X, Z, CX = (kref.GATE[g] for g in ("H", "X", "Z", "CX"))
    want = {0: np.zeros(8, complex), 1: np.zeros(8, complex)}
    want[0][0], want[0][7] = 1 / np.sqrt(2), -1 / np.sqrt(2)
    want[1][7] = -1
    for u, outcome in ((0.25, 0), (0.75, 1)):
        s = np.zeros(8, complex)
        s[0] = 1
        s = oracle.hilbert1(s, X, 1)
        s = oracle.hilbert1(s, H, 1)
        s, ind, p0 = oracle.born_measure_z(s, 1, u=u)
        s = oracle.hilbert1(s, H.conj().T, 1)
        s = oracle.hilbert1(s, Z if ind == 0 else H, 1)
        s = oracle.hilbert2(s, CX, 1, 2)
        s = oracle.hilbert2(s, CX, 2, 3)
        assert ind == outcome and abs(p0 - 0.5) < 1e-12
        assert np.abs(s - want[outcome]).max() < 1e-12, (outcome, s)


def test_ref_docs_reset_of_a_bell_state(oracle, kref):
    """The reference's documented reset example: Op("RES", 1) on the Bell state
    (|00> + |11>)/sqrt(2) leaves |00> or |01>, each with probability 1/2
    (docs/src/examples.md:337-343; _reset_Z: measure, X on outcome 1,
    src/hilbert.jl:752-759)."""
    H, X, CX = (kref.GATE[g] for g in ("H", "X", "CX"))
    for u, outcome, idx in ((0.25, 0, 0), (0.75, 1, 1)):
        s = np.zeros(4, complex)
        s[0] = 1
        s = oracle.hilbert2(oracle.hilbert1(s, H, 1), CX, 1, 2)
        s, ind, p0 = oracle.born_measure_z(s, 1, u=u)
        if ind == 1:
            s = oracle.hilbert1(s, X, 1)
        want = np.zeros(4, complex)
        want[idx] = 1
        assert ind == outcome and abs(p0 - 0.5) < 1e-12
        assert np.abs(s - want).max() < 1e-12, (outcome, s)


def test_ref_channel_cptp_and_sample_semantics(oracle):
    """weighted sample: first i with u <= cumsum(p) (src/hilbert.jl:810-819); sample
    picks the first index whose cumulative weight reaches u*sum (StatsBase direct)."""
    p = np.array([0.2, 0.3, 0.5])
    assert oracle.weighted_sample(p, 0.2) == 0
    assert oracle.weighted_sample(p, 0.2000001) == 1
    assert oracle.weighted_sample(p, 0.9999) == 2
    assert oracle.weighted_sample(np.array([0.2, 0.3]), 0.9) is None
    psi = np.sqrt(np.array([0.25, 0, 0.25, 0.5], complex))
    assert list(oracle.sample(psi, [0.0, 0.2, 0.25, 0.26, 0.5, 0.51, 0.999])) == [0, 0, 0, 2, 2, 3, 3]


def test_ref_two_qubit_born_measurement(oracle, kref):
    """born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721): the C restatement
    equals the literal projection construction (expand_multi_op with P0/P1 on
    (q1, q2), weights |psi' slist[k]|, _weighted_sample, normalize) for every
    forced outcome and for drawn ones, with q1 < q2, q1 > q2 and non-adjacent
    pairs; a Bell pair measured on both qubits gives only outcomes 1 and 4."""
    rng = np.random.default_rng(44)
    n = 5
    for q1, q2 in ((1, 2), (4, 2), (1, 5), (3, 4)):
        psi = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        psi /= np.linalg.norm(psi)
        for f in (1, 2, 3, 4):
            a, oa, pa = oracle.born_measure_z2(psi, q1, q2, forced=f)
            b, ob, pb = kref.born_measure_z2(psi, q1, q2, forced=f)
            assert oa == ob == f and np.abs(a - b).max() < 1e-13 and np.abs(pa - pb).max() < 1e-14
        for u in rng.random(6):
            a, oa, _ = oracle.born_measure_z2(psi, q1, q2, u=u)
            b, ob, _ = kref.born_measure_z2(psi, q1, q2, u=u)
            assert oa == ob and np.abs(a - b).max() < 1e-13
    bell = np.zeros(4, complex)
    bell[0] = bell[3] = 1 / np.sqrt(2)
    outs = {oracle.born_measure_z2(bell, 1, 2, u=u)[1] for u in np.linspace(0.01, 0.99, 25)}
    assert outs == {1, 4}
