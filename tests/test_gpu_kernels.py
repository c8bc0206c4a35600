"""Parity of every engine kernel against the oracle, through the C ABI.

Tolerances: complex128 states match within 1e-12 max-abs per amplitude or
density entry (the drop-in bar); complex64 within 2e-5 (float32 rounding over
a handful of operations); collapse zero sets are compared exactly; branch and
outcome indices exactly.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 2e-5


def rstate(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def runitary(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def rrho(rng, n, k=3):
    rho = 0
    w = rng.random(k)
    w /= w.sum()
    for i in range(k):
        p = rstate(rng, n)
        rho = rho + w[i] * np.outer(p, p.conj())
    return rho


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_gates_every_target_and_control(ctx, oracle, prec):
    import bluetangle_gpu as bt
    tol = TOL128 if prec == "c128" else TOL64
    rng = np.random.default_rng(11)
    n = 9
    psi = rstate(rng, n)
    st = bt.state_from(psi, prec)
    ref = psi.copy()
    for q in range(1, n + 1):
        U = runitary(rng, 2)
        bt.apply_matrix(st, U, [q])
        ref = oracle.apply_k(ref, U, [q])
        c = 1 + (q % n)
        bt.apply_matrix(st, U.conj().T @ U @ U, [q], [c])
        ref = oracle.apply_k(ref, U.conj().T @ U @ U, [q], [c])
    for q, t in [(1, 2), (2, 1), (3, 7), (9, 1), (5, 4), (8, 9)]:
        U = runitary(rng, 4)
        bt.apply_matrix(st, U, [q, t])
        ref = oracle.hilbert2(ref, U, q, t)
    for q, t, c in [(2, 3, 7), (6, 5, 1), (1, 9, 4)]:
        U = runitary(rng, 4)
        bt.apply_matrix(st, U, [q, t], [c])
        ref = oracle.apply_k(ref, U, [q, t], [c])
    for k in (3, 4, 5):
        qs = list(rng.choice(np.arange(1, n + 1), size=k, replace=False))
        U = runitary(rng, 2 ** k)
        bt.apply_matrix(st, U, [int(x) for x in qs])
        ref = oracle.apply_k(ref, U, [int(x) for x in qs])
    assert np.abs(st.to_numpy() - ref).max() < (TOL128 if prec == "c128" else 10 * TOL64)


def test_gate_matches_reference_hilbert_semantics(ctx, oracle):
    """bt_apply_matrix with (q, t) equals hilbert(N,U,q,t;control) incl. CCZX."""
    import bluetangle_gpu as bt
    from bluetangle_gpu.gates import gate
    rng = np.random.default_rng(12)
    n = 7
    for q, t, c in [(1, 5, 3), (6, 2, 4), (3, 4, 1), (4, 3, 7)]:
        for M in (gate["CX"], gate["CZ"]):
            psi = rstate(rng, n)
            st = bt.state_from(psi)
            bt.apply_matrix(st, M, [q, t], [c])
            assert np.abs(st.to_numpy() - oracle.hilbert2(psi, M, q, t, c)).max() < TOL128


def test_batched_members_and_member_select(ctx, oracle):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(13)
    n, B = 6, 5
    st = bt.zero_state(n, batch=B)
    psis = [rstate(rng, n) for _ in range(B)]
    for m, p in enumerate(psis):
        st.upload(p, m)
    U = runitary(rng, 4)
    bt.apply_matrix(st, U, [2, 5])
    V = runitary(rng, 2)
    bt.apply_matrix(st, V, [3], member=2)
    for m, p in enumerate(psis):
        ref = oracle.apply_k(p, U, [2, 5])
        if m == 2:
            ref = oracle.apply_k(ref, V, [3])
        assert np.abs(st.to_numpy(m) - ref).max() < TOL128


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_measure_forced_and_drawn(ctx, oracle, prec):
    import bluetangle_gpu as bt
    tol = TOL128 if prec == "c128" else TOL64
    rng = np.random.default_rng(14)
    n = 8
    for q in (1, 4, 8):
        for forced in (0, 1):
            psi = rstate(rng, n)
            st = bt.state_from(psi, prec)
            _, ind, p0 = bt.born_measure_Z(st, q, forced=forced)
            ref, rind, rp0 = oracle.born_measure_z(psi, q, forced=forced)
            out = st.to_numpy()
            assert ind == forced == rind
            assert abs(p0 - rp0) < (1e-14 if prec == "c128" else 1e-6)
            assert np.array_equal(out == 0, ref == 0)  # bit-exact zero set
            assert np.abs(out - ref).max() < tol
        psi = rstate(rng, n)
        st = bt.state_from(psi, prec)
        u = rng.random(1)
        _, ind, p0 = bt.born_measure_Z(st, q, rng=np.random.default_rng(99))
        u = np.random.default_rng(99).random(1)[0]
        ref, rind, _ = oracle.born_measure_z(psi, q, u=u)
        assert ind == rind and np.abs(st.to_numpy() - ref).max() < tol


def test_measure_batched_members(ctx, oracle):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(15)
    n, B = 7, 16
    psis = [rstate(rng, n) for _ in range(B)]
    st = bt.zero_state(n, batch=B)
    for m, p in enumerate(psis):
        st.upload(p, m)
    u = np.random.default_rng(7).random(B)
    _, ind, p0 = bt.born_measure_Z(st, 3, rng=np.random.default_rng(7))
    for m, p in enumerate(psis):
        ref, rind, rp0 = oracle.born_measure_z(p, 3, u=u[m])
        assert ind[m] == rind and abs(p0[m] - rp0) < 1e-14
        assert np.abs(st.to_numpy(m) - ref).max() < TOL128


def test_measure_zero_probability_forced_is_an_error(ctx):
    import bluetangle_gpu as bt
    st = bt.zero_state(4)
    with pytest.raises(bt.BTError):
        bt.born_measure_Z(st, 2, forced=1)
    # the context stays usable
    bt.born_measure_Z(st, 2, forced=0)


def test_reduced_dm(ctx, oracle):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(16)
    n = 8
    psi = rstate(rng, n)
    st = bt.state_from(psi)
    for keep in ([3], [2, 6], [1, 2], [4, 5, 8]):
        assert np.abs(bt.partial_trace(st, keep) - oracle.partial_trace(psi, keep)).max() < 1e-14
    # listed order matters: (6, 2) is the permuted matrix
    a = bt.partial_trace(st, [6, 2])
    b = oracle.partial_trace(psi, [2, 6])
    p = [0, 2, 1, 3]
    assert np.abs(a - b[np.ix_(p, p)]).max() < 1e-14


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_kraus_trajectory_matches_oracle(ctx, oracle, kref, prec):
    import bluetangle_gpu as bt
    tol = TOL128 if prec == "c128" else TOL64
    rng = np.random.default_rng(17)
    n = 8
    channels = [(kref.noise_model("amplitude_damping", 0.3), 3, None),
                (kref.noise_model("depolarizing", 0.2), 8, None),
                (kref.noise_model("depolarizing", 0.4, True), 2, 3),
                (kref.noise_model("amplitude_damping", 0.5, True), 6, 2),  # q > t: reference branch order
                (kref.noise_model("phase_damping", 0.35, True), 1, 8)]
    for kr, q, t in channels:
        for trial in range(4):
            psi = rstate(rng, n)
            st = bt.state_from(psi, prec)
            seed = int(rng.integers(1 << 30))
            _, br, pr = bt.apply_channel(st, kr, q, t, rng=np.random.default_rng(seed), probs_out=True)
            u = np.random.default_rng(seed).random(1)[0]
            ref, rbr, rpr = oracle.channel_traj(psi, kr, q, -1 if t is None else t, u=u)
            assert br[0] == rbr
            assert np.abs(pr[0] - rpr).max() < (1e-14 if prec == "c128" else 1e-6)
            assert np.abs(st.to_numpy() - ref).max() < tol
        # forced branch
        psi = rstate(rng, n)
        st = bt.state_from(psi, prec)
        bt.apply_channel(st, kr, q, t, forced=1)
        ref, _, _ = oracle.channel_traj(psi, kr, q, -1 if t is None else t, forced=1)
        assert np.abs(st.to_numpy() - ref).max() < tol


def test_kraus_three_qubit_channel(ctx, oracle):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(18)
    n = 7
    U = [runitary(rng, 8) for _ in range(3)]
    kr = [np.sqrt(w) * u for w, u in zip([0.5, 0.3, 0.2], U)]
    psi = rstate(rng, n)
    st = bt.state_from(psi)
    _, br, _ = bt.apply_channel(st, kr, 3, None, rng=np.random.default_rng(5), probs_out=True)
    ref, rbr, _ = oracle.channel_traj(psi, kr, 3, -1, u=np.random.default_rng(5).random(1)[0])
    assert br[0] == rbr and np.abs(st.to_numpy() - ref).max() < TOL128


def test_non_cptp_rejected(ctx):
    import bluetangle_gpu as bt
    st = bt.zero_state(3)
    with pytest.raises(bt.BTError, match="CPTP"):
        bt.apply_channel(st, [np.eye(2) * 1.01], 1)


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_density_matrix_gates_channels_dephase(ctx, oracle, kref, prec):
    import bluetangle_gpu as bt
    tol = TOL128 if prec == "c128" else TOL64
    rng = np.random.default_rng(19)
    n = 5
    rho = rrho(rng, n)
    g = bt.rho_from(rho, prec)
    ref = rho.copy()
    for q in (1, 3, 5):
        U = runitary(rng, 2)
        bt.apply_matrix(g, U, [q])
        ref = oracle.dm_hilbert1(ref, U, q)
    for q, t in [(1, 2), (4, 2), (5, 1)]:
        U = runitary(rng, 4)
        bt.apply_matrix(g, U, [q, t])
        ref = oracle.dm_hilbert2(ref, U, q, t)
    U = runitary(rng, 2)
    bt.apply_matrix(g, U, [2], [4])
    ref = oracle.dm_hilbert1(ref, U, 2, 4)
    U = runitary(rng, 8)
    bt.apply_matrix(g, U, [1, 3, 5])
    ref = oracle.dm_gate(ref, U, [1, 3, 5])
    for kr, q, t in [(kref.noise_model("depolarizing", 0.1, True), 2, 3),
                     (kref.noise_model("amplitude_damping", 0.2), 4, -1),
                     (kref.noise_model("amplitude_damping", 0.3, True), 5, 2)]:
        bt.apply_channel(g, kr, q, None if t < 0 else t)
        ref = oracle.dm_channel(ref, kr, q, t)
    _, _, p0 = bt.born_measure_Z(g, 3)
    assert abs(p0 - np.real(sum(ref[i, i] for i in range(2 ** n) if not (i >> (n - 3)) & 1))) < 1e-6
    ref = oracle.dm_dephase(ref, 3)
    assert np.abs(g.to_numpy() - ref).max() < (TOL128 if prec == "c128" else 10 * TOL64)


def _random_pauli_terms(rng, n, count, maxw=3):
    terms = []
    for _ in range(count):
        w = int(rng.integers(1, maxw + 1))
        qs = rng.choice(np.arange(1, n + 1), size=w, replace=False)
        x = z = 0
        for q in qs:
            p = "XYZ"[int(rng.integers(0, 3))]
            b = 1 << (n - int(q))
            x |= b if p in "XY" else 0
            z |= b if p in "ZY" else 0
        terms.append((x, z))
    return terms


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("n,batch", [(9, 1), (16, 1), (11, 3)])
def test_pauli_sums_tiled_match_oracle(ctx, oracle, prec, n, batch):
    """Many Pauli strings with distinct x-masks (the tiled path: one state read per
    tile group) against the oracle, per member, with coefficients; complex64
    within 1e-5 (FP32 micro-sums of complex64 amplitudes)."""
    import ctypes
    import bluetangle_gpu as bt
    tol = 1e-12 if prec == "c128" else 1e-5
    rng = np.random.default_rng(40 + n)
    terms = _random_pauli_terms(rng, n, 70)
    st = bt.zero_state(n, prec, batch=batch)
    psis = [rstate(rng, n) for _ in range(batch)]
    for m, p in enumerate(psis):
        st.upload(p, m)
    xs = np.ascontiguousarray([t[0] for t in terms], dtype=np.uint64)
    zs = np.ascontiguousarray([t[1] for t in terms], dtype=np.uint64)
    cs = np.ascontiguousarray(rng.normal(size=len(terms)))
    out = np.empty(batch * len(terms))
    P = ctypes.c_void_p
    st.ctx.check(bt.lib().bt_expect_pauli(st.h, len(terms), xs.ctypes.data_as(P), zs.ctypes.data_as(P),
                                          cs.ctypes.data_as(P), -1, out.ctypes.data_as(P)))
    out = out.reshape(batch, len(terms))
    for m, p in enumerate(psis):
        ref = np.array([c * oracle.expect_pauli_sv(p, x, z) for (x, z), c in zip(terms, cs)])
        assert np.abs(out[m] - ref).max() < tol, (m, np.abs(out[m] - ref).max())


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_pauli_expectations(ctx, oracle, prec):
    import bluetangle_gpu as bt
    tol = 1e-13 if prec == "c128" else 1e-5
    rng = np.random.default_rng(20)
    n = 9
    psi = rstate(rng, n)
    st = bt.state_from(psi, prec)
    terms = [(["Z"], [3]), (["X"], [1]), (["Y"], [9]), (["X", "Y"], [2, 7]), (["Z", "Z"], [4, 5]),
             (["Y", "Y", "X"], [1, 2, 3]), (["X", "Z", "Y", "Z"], [9, 1, 5, 4])]
    for names, qs in terms:
        x, z = bt.pauli_masks(names, qs, n)
        v = bt.correlation(st, ",".join(names), qs)
        assert abs(v - oracle.expect_pauli_sv(psi, x, z)) < tol, names
    zs = bt.expect(st, "Z")
    assert np.abs(np.array(zs) - [oracle.expect_pauli_sv(psi, 0, 1 << (n - q)) for q in range(1, n + 1)]).max() < tol
    # non-Pauli observable on a state: T on qubit 2, and a controlled op
    T = bt.gate["T"]
    assert abs(bt.expect(st, bt.Op("T", 2)) - oracle.expect_matrix_sv(psi, T, [2])) < tol
    o = bt.Op("CNOT", 3, 6)
    assert abs(bt.expect(st, o) - oracle.expect_matrix_sv(psi, o.mat, [3, 6])) < tol
    # density matrix
    rho = rrho(rng, 5)
    g = bt.rho_from(rho, prec)
    for names, qs in [(["Z"], [1]), (["X", "Z"], [1, 3]), (["Y", "Y"], [2, 5]), (["X", "Y", "Z"], [5, 4, 3])]:
        x, z = bt.pauli_masks(names, qs, 5)
        assert abs(bt.correlation(g, ",".join(names), qs) - oracle.expect_pauli_dm(rho, x, z)) < tol
    zs = bt.expect(g, "Z")
    assert np.abs(np.array(zs) - [oracle.expect_pauli_dm(rho, 0, 1 << (5 - q)) for q in range(1, 6)]).max() < tol


@pytest.mark.parametrize("prec,tol", [("c64", 2e-6), ("c128", 1e-12)])
def test_z_all_large_and_batched(ctx, prec, tol):
    """<Z_i> of every qubit (bt_expect_z_all: per-bit sums; complex64 states of
    2^15 amplitudes and more take the super-chunk form) at 15, 16 and 20 qubits,
    for one member and for all members of a batch of 3, against FP64 sums of the
    stored amplitudes' |psi|^2 on the host."""
    import bluetangle_gpu as bt
    rng = np.random.default_rng(77)
    for n in (15, 16, 20):
        psis = [rstate(rng, n) for _ in range(3)]
        st = bt.zero_state(n, prec, 3)
        for m, psi in enumerate(psis):
            st.upload(psi, m)
        idx = np.arange(2 ** n)
        refs = []
        for psi in psis:
            stored = psi.astype(np.complex64 if prec == "c64" else np.complex128).astype(np.complex128)
            p = np.abs(stored) ** 2
            refs.append(np.array([p.sum() - 2 * p[((idx >> (n - q)) & 1) == 1].sum() for q in range(1, n + 1)]))
        allz = bt.expect(st, "Z", member=-1)
        for m in range(3):
            assert np.abs(np.asarray(bt.expect(st, "Z", member=m)) - refs[m]).max() < tol, (n, m)
            assert np.abs(allz[m] - refs[m]).max() < tol, (n, m)


def test_fidelity_and_norm(ctx):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(21)
    a, b = rstate(rng, 10), rstate(rng, 10)
    sa, sb = bt.state_from(a), bt.state_from(b)
    assert abs(bt.fidelity(sa, sb) - abs(np.vdot(a, b)) ** 2) < 1e-14


@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_sample_with_given_uniforms_matches_oracle(ctx, oracle, prec):
    import bluetangle_gpu as bt
    rng = np.random.default_rng(22)
    for n in (3, 12, 15):
        psi = rstate(rng, n)
        if prec == "c64":
            psi = psi.astype(np.complex64).astype(np.complex128)
        st = bt.state_from(psi, prec)
        u = np.random.default_rng(n).random(5000)
        got = bt.sample(st, 5000, rng=np.random.default_rng(n))
        ref = oracle.sample(psi, u)
        w = np.abs(psi) ** 2
        cdf = np.cumsum(w)
        t = u * cdf[-1]
        # identical except where t sits within rounding of a cumulative boundary
        near = np.min(np.abs(cdf[None, :] - t[:, None]), axis=1) < 1e-12
        assert np.all((got == ref) | near)


def test_sample_device_rng_chi_square(ctx):
    import bluetangle_gpu as bt
    from scipy import stats
    rng = np.random.default_rng(23)
    n = 6
    psi = rstate(rng, n)
    st = bt.state_from(psi)
    shots = 200000
    got = bt.sample(st, shots, seed=77)
    counts = np.bincount(got, minlength=2 ** n)
    expected = np.abs(psi) ** 2 * shots
    chi2, p = stats.chisquare(counts, expected)
    assert p > 1e-4
    # different seeds give different streams
    assert not np.array_equal(got[:100], bt.sample(st, 100, seed=78))
