"""Circuit-level measure with Options, the two-qubit Born measurement, state
preparation and fidelity of density matrices, against the oracle (complex128,
1e-12), the literal kron restatement, and shots compared exactly under shared
uniform draws."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def rdensity(rng, n, rank=None):
    d = 2 ** n
    r = rank or d
    A = rng.normal(size=(d, r)) + 1j * rng.normal(size=(d, r))
    R = A @ A.conj().T
    return R / np.trace(R).real


@pytest.mark.parametrize("q1,q2", [(2, 5), (5, 2), (1, 2), (6, 3)])
def test_born_measure_two_qubits_matches_oracle(ctx, oracle, kref, q1, q2):
    """born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721): every forced
    outcome 1..4, and drawn outcomes under shared uniforms for a batch; kept
    amplitudes within 1e-12, the zeroed set exactly the reference's, weights
    equal to |psi' P psi| of the literal projection."""
    import bluetangle_gpu as bt
    n = 6
    rng = np.random.default_rng(40 + q1 + 7 * q2)
    psi = rstate(rng, n)
    for f in (1, 2, 3, 4):
        st = bt.state_from(psi)
        _, out, probs = bt.born_measure_Z(st, q1, q2, forced=f)
        ref, oc, rp = oracle.born_measure_z2(psi, q1, q2, forced=f)
        kr, koc, kp = kref.born_measure_z2(psi, q1, q2, forced=f)
        got = st.to_numpy()
        assert out == oc == koc == f
        assert np.abs(got - ref).max() < 1e-12 and np.abs(ref - kr).max() < 1e-12
        assert np.array_equal(got == 0, ref == 0)
        assert np.abs(probs - rp).max() < 1e-13 and np.abs(rp - kp).max() < 1e-13
    # a batch: every member its own state and draw
    B = 8
    st = bt.zero_state(n, "c128", B, ctx)
    psis = [rstate(rng, n) for _ in range(B)]
    for m, p in enumerate(psis):
        st.upload(p, m)
    u = np.random.default_rng(3).random(B)
    _, outs, probs = bt.born_measure_Z(st, q1, q2, rng=np.random.default_rng(3))
    for m in range(B):
        ref, oc, rp = oracle.born_measure_z2(psis[m], q1, q2, u=u[m])
        assert outs[m] == oc
        assert np.abs(st.to_numpy(m) - ref).max() < 1e-12
        assert np.abs(probs[m] - rp).max() < 1e-13


def test_born_measure_two_qubits_complex64(ctx, oracle):
    import bluetangle_gpu as bt
    n = 8
    psi = rstate(np.random.default_rng(9), n)
    st = bt.state_from(psi, "c64")
    _, out, _ = bt.born_measure_Z(st, 3, 7, rng=np.random.default_rng(2))
    ref, oc, _ = oracle.born_measure_z2(psi, 3, 7, u=np.random.default_rng(2).random(1)[0])
    assert out == oc
    got = st.to_numpy()
    assert np.abs(got - ref).max() < 2e-6 and np.array_equal(got == 0, ref == 0)


def test_state_preparation_matches_reference(ctx, kref):
    """product_state and its wrappers (src/hilbert.jl:835-877): the kron of
    single-qubit basis vectors, qubit 1 first; sign(x) != 0 means |1>."""
    import bluetangle_gpu as bt

    def kron_bits(bits):
        v = np.array([1.0 + 0j])
        for b in bits:
            v = np.kron(v, np.array([1, 0], complex) if int(np.sign(b)) == 0 else np.array([0, 1], complex))
        return v

    n = 7
    for bits in ([0, 1, 1, 0, 1, 0, 0], [1, -1, 0, 2, 0, 0, 1]):
        assert np.array_equal(bt.product_state(bits).to_numpy(), kron_bits(bits))
    neel01 = kron_bits([0 if i % 2 == 1 else 1 for i in range(1, n + 1)])
    neel10 = kron_bits([1 if i % 2 == 1 else 0 for i in range(1, n + 1)])
    assert np.array_equal(bt.neel_state01(n).to_numpy(), neel01)
    assert np.array_equal(bt.neel_state10(n).to_numpy(), neel10)
    assert np.abs(bt.neel_state_s(n).to_numpy() - (neel01 + neel10) / math.sqrt(2)).max() < 1e-15
    z3 = [kron_bits([1 if (i + 2 - j + 1) % 3 == 0 else 0 for i in range(1, n + 1)]) for j in (1, 2, 3)]
    for j in (1, 2, 3):
        assert np.array_equal(bt.Z3(n, j).to_numpy(), z3[j - 1])
    zs = z3[0] + z3[1] + z3[2]
    assert np.abs(bt.Z3_s(n).to_numpy() - zs / np.linalg.norm(zs)).max() < 1e-15
    one = np.zeros(2 ** n, complex)
    one[-1] = 1
    assert np.array_equal(bt.one_state(n).to_numpy(), one)
    assert np.abs(bt.plus_state(n).to_numpy() - 2 ** (-n / 2)).max() < 1e-15
    H = np.array([[1, 1], [1, -1]]) / math.sqrt(2)
    Hn = np.array([[1.0]])
    for _ in range(n):
        Hn = np.kron(Hn, H)
    assert np.abs(bt.minus_state(n).to_numpy() - Hn @ one).max() < 1e-14
    # random_product_state(N) = product_state(rand([0,1], N)) with the caller's draws
    bits = np.random.default_rng(12).integers(0, 2, n)
    assert np.array_equal(bt.random_product_state(n, rng=np.random.default_rng(12)).to_numpy(), kron_bits(bits))
    # random_state: unit norm, real and imaginary parts drawn from [0, 1) before scaling
    r1, r2 = bt.random_state(12, seed=1).to_numpy(), bt.random_state(12, seed=2).to_numpy()
    assert abs(np.linalg.norm(r1) - 1) < 1e-13
    assert r1.real.min() >= 0 and r1.imag.min() >= 0 and np.abs(r1 - r2).max() > 1e-3
    scale = 1 / r1.real.max()  # undo the normalisation: uniform parts have mean 1/2
    assert abs(np.mean(np.concatenate([r1.real, r1.imag])) * scale - 0.5) < 0.02
    assert np.array_equal(bt.random_state(12, seed=1).to_numpy(), r1)


@pytest.mark.parametrize("n", [1, 3, 5])
def test_fidelity_of_density_matrices(ctx, n):
    """fidelity(rho, sigma) (src/tensor.jl:222-229) against the same formula with
    scipy's matrix square roots, and the pure-state and rho = sigma identities."""
    import scipy.linalg as sl

    import bluetangle_gpu as bt
    rng = np.random.default_rng(n)
    # a rank-2 sigma leaves d - 2 eigenvalues of sqrt(rho) sigma sqrt(rho) at
    # rounding level (~1e-17); every square-root formula, the reference's included,
    # turns each into a ~3e-9 term of the trace, so that case is compared at 1e-8
    for prec, rank, tol in (("c128", None, 1e-10), ("c128", 2, 1e-8), ("c64", None, 1e-5)):
        R, S = rdensity(rng, n), rdensity(rng, n, rank=rank)
        a, b = bt.rho_from(R, prec), bt.rho_from(S, prec)
        sr = sl.sqrtm(R)
        ref = float(np.real(np.trace(sl.sqrtm(sr @ S @ sr)) ** 2))
        assert abs(bt.fidelity(a, b) - ref) < tol, (prec, rank, bt.fidelity(a, b), ref)
        assert abs(bt.fidelity(a, a) - 1) < max(tol, 1e-10)
    # pure states: rank 1, the same rounding-level eigenvalues as above
    psi, phi = rstate(rng, n), rstate(rng, n)
    a, b = bt.rho_from(np.outer(psi, psi.conj())), bt.rho_from(np.outer(phi, phi.conj()))
    assert abs(bt.fidelity(a, b) - abs(np.vdot(psi, phi)) ** 2) < 1e-8


def _apply_basis(oracle, psi, names):
    from bluetangle_gpu.gates import gate
    for q, g in enumerate(names, start=1):
        if g is not None:
            psi = oracle.apply_k(psi, gate[g], [q], [])
    return psi


@pytest.mark.parametrize("basis", ["Z", "X", "Y", "R"])
def test_measure_circuit_noiseless(ctx, oracle, basis):
    """measure(circuit, shots) without noise (src/ops.jl:605-614): one state,
    the final basis rotation (_final_measurement, src/ops.jl:856-914; R draws
    rand(1:3) per qubit), every shot from it; density_matrix gives state*state'.
    Shots equal the oracle's under the same uniforms."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuits as C
    n, shots = 6, 2000
    ops = C.brickwork(n, 5, np.random.default_rng(17))
    circ = bt.compile(ops, bt.Options(measurement_basis=basis.lower(), density_matrix=True, circuit_name="bw"))
    assert circ.options.measurement_basis == basis and circ.stats["N"] == n
    m = bt.measure(circ, shots, rng=np.random.default_rng(5))
    rr = np.random.default_rng(5)
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    for op in ops:
        psi = oracle.apply_k(psi, op.mat, [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit], [])
    names = {"Z": [None] * n, "X": ["H"] * n, "Y": ["HSP"] * n}.get(basis)
    if names is None:
        names = [["H", "HSP", None][int(rr.integers(0, 3))] for _ in range(n)]
    psi = _apply_basis(oracle, psi, names)
    s = oracle.sample(psi, rr.random(shots))
    vals, cnt = np.unique(s, return_counts=True)
    assert np.array_equal(m.bitstr, vals) and np.array_equal(m.sample, cnt / shots)
    assert m.measurement_basis == basis and m.circuit_name == "bw" and m.number_of_experiment == shots
    fock = (vals[:, None] >> (n - 1 - np.arange(n))[None, :]) & 1
    assert np.abs(np.array(m.expect) - [(np.where(fock[:, i] == 0, 1, -1) * cnt / shots).sum() for i in range(n)]).max() < 1e-15
    assert np.abs(m.density_matrix.to_numpy() - np.outer(psi, psi.conj())).max() < 1e-12


@pytest.mark.parametrize("basis,zne_id,twirl", [("Z", 0, False), ("X", 1, False), ("R", 0, True)])
def test_measure_circuit_noisy(ctx, oracle, kref, basis, zne_id, twirl):
    """measure(circuit, shots, id) with a NoiseModel, a readout channel and
    (optionally) ZNE repetitions and twirling (src/ops.jl:615-630): every shot a
    re-simulated trajectory with its own Kraus branches and final basis, one
    sample each; the members and shots equal the oracle replaying each member
    with the same draws; density_matrix averages state*state' over the shots."""
    import bluetangle_gpu as bt
    import bluetangle_gpu.circuit as CI
    import bluetangle_gpu.trajectories as T
    from test_gpu_trajectories import replay
    n, shots = 4, 24
    ops = [bt.Op("H", 1), bt.Op("CNOT", 1, 2), bt.Op("RY(0.4)", 3), bt.Op("CNOT", 2, 3), bt.Op("T", 4),
           bt.Op("CNOT", 3, 4), bt.Op("MZ", 2), bt.Op("RX(1.1)", 2)]
    noise = bt.NoiseModel(bt.Noise1("depolarizing", 0.05), bt.Noise2("depolarizing", 0.08))
    ro = bt.QuantumChannel("bit_flip", 0.1)
    opts = bt.Options(measurement_basis=basis, noise=noise, readout_noise=ro, twirl=twirl, density_matrix=True)
    circ = bt.compile(ops, opts)
    m = bt.measure(circ, shots, zne_id, rng=np.random.default_rng(21))
    # replay: the same per-member programs (same draws for bases and frames), then
    # each member's channel draws and its one shot
    rr = np.random.default_rng(21)
    member_ops = CI._noisy_members(circ, shots, zne_id, rr, rr)
    slots = T.build_slots(member_ops, noise)
    psis, _ = replay(oracle, slots, shots, n, rr, kref)
    u = rr.random(shots)
    s = np.array([oracle.sample(p, u[k:k + 1])[0] for k, p in enumerate(psis)])
    assert np.array_equal(np.sort(m.samples), np.sort(s)) and np.array_equal(m.samples, s)
    vals, cnt = np.unique(s, return_counts=True)
    assert np.array_equal(m.bitstr, vals) and np.allclose(m.sample, cnt / shots, atol=0)
    rho = sum(np.outer(p, p.conj()) for p in psis) / shots
    assert np.abs(m.density_matrix.to_numpy() - rho).max() < 1e-12


def test_measure_circuit_mitigation(ctx):
    """measurement_mitigate with a readout channel (src/ops.jl:635-638):
    normalize(abs.(inv(A) avg_prob), 1) with A the reference's confusion matrix,
    here when every outcome was observed (the reference's vector sizes agree only
    then)."""
    import bluetangle_gpu as bt
    from bluetangle_gpu.mitigation import mitigation_matrix
    n, shots = 2, 400
    ops = [bt.Op("H", 1), bt.Op("H", 2)]
    ro = bt.QuantumChannel("bit_flip", 0.1)
    opts = bt.Options(readout_noise=ro, measurement_mitigate=True)
    m = bt.measure(bt.compile(ops, opts), shots, rng=np.random.default_rng(8))
    raw = bt.measure(bt.compile(ops, bt.Options(readout_noise=ro)), shots, rng=np.random.default_rng(8))
    assert np.array_equal(m.bitstr, np.arange(4)) and np.array_equal(raw.bitstr, m.bitstr)
    ref = np.abs(mitigation_matrix(n, ro) @ raw.sample)
    assert np.abs(m.sample - ref / ref.sum()).max() < 1e-12
