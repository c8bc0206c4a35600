"""Literal numpy restatement of BlueTangle.jl's operator construction.

TEST INFRASTRUCTURE ONLY: this module is a checker.  Only tests/, the golden
fixture generator (tests/golden/make_golden.py), __graft_entry__.smoke() and
bench.py's CPU-baseline leg may import it; the product path never does.

Unlike the dense index-arithmetic oracle (btoracle.c), this file follows the
reference's own construction step by step -- full 2^N x 2^N operators built
with kron, the SWAP-permutation of two-qubit matrices, the Pauli decomposition
and reconstruction for non-adjacent pairs, CCZX for controlled non-adjacent
pairs -- so that it stands in for running the Julia reference itself (Julia is
not installed where these checks run).  It is only practical for N <= 10.

Matrices here are ordinary (row-major) numpy arrays M[r, c].
"""
import itertools
import math

import numpy as np

# ---------------------------------------------------------------- gate table
# src/gates.jl:22-59


def _round_sig(x, sig=10):
    """round(x, sigdigits=10) applied to real and imaginary parts (src/gates.jl:32-33)."""
    def r(v):
        if v == 0:
            return 0.0
        return float(f"{v:.{sig - 1}e}")
    return complex(r(x.real), r(x.imag))


S2 = 1 / math.sqrt(2)
GATE = {
    "I": np.array([[1, 0], [0, 1]], dtype=complex),
    "X": np.array([[0, 1], [1, 0]], dtype=complex),
    "SX": 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "XSQRT": 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "Y": np.array([[0, -1j], [1j, 0]]),
    "Z": np.array([[1, 0], [0, -1]], dtype=complex),
    "H": S2 * np.array([[1, 1], [1, -1]], dtype=complex),
    "S": np.array([[1, 0], [0, 1j]]),
    "SD": np.array([[1, 0], [0, -1j]]),
    "T": np.array([[1, 0], [0, _round_sig(np.exp(1j * np.pi / 4))]]),
    "TD": np.array([[1, 0], [0, _round_sig(np.exp(-1j * np.pi / 4))]]),
    "HSP": S2 * np.array([[1, -1j], [1, 1j]]),
    "HY": S2 * np.array([[1, 1j], [1, -1j]]),
    "P0": np.array([[1, 0], [0, 0]], dtype=complex),
    "P1": np.array([[0, 0], [0, 1]], dtype=complex),
    "SP": np.array([[0, 1], [0, 0]], dtype=complex),
    "SM": np.array([[0, 0], [1, 0]], dtype=complex),
    "CX": np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=complex),
    "CNOT": np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=complex),
    "CY": np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]]),
    "CZ": np.diag([1, 1, 1, -1]).astype(complex),
    "CS": np.diag([1, 1, 1, 1j]),
    "CSD": np.diag([1, 1, 1, -1j]),
    "CT": np.diag([1, 1, 1, _round_sig(np.exp(1j * np.pi / 4))]),
    "CTD": np.diag([1, 1, 1, _round_sig(np.exp(-1j * np.pi / 4))]),
    "CH": np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, S2, S2], [0, 0, S2, -S2]], dtype=complex),
    "SWAP": np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=complex),
    "ISWAP": np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]]),
    "FSWAP": np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, -1]], dtype=complex),
    "ECR": S2 * np.array([[0, 1, 0, 1j], [1, 0, -1j, 0], [0, 1j, 0, 1], [-1j, 0, 1, 0]]),
}


def rx(t):
    return np.array([[math.cos(t / 2), -1j * math.sin(t / 2)], [-1j * math.sin(t / 2), math.cos(t / 2)]])


def ry(t):
    return np.array([[math.cos(t / 2), -math.sin(t / 2)], [math.sin(t / 2), math.cos(t / 2)]], dtype=complex)


def rz(t):
    return np.array([[np.exp(-1j * t / 2), 0], [0, np.exp(1j * t / 2)]])


def phase(lam):
    return np.array([[1, 0], [0, np.exp(1j * lam)]])


def rzz(p):
    return np.diag([np.exp(-1j * p / 2), np.exp(1j * p / 2), np.exp(1j * p / 2), np.exp(-1j * p / 2)])


def rxx(p):
    c, s = math.cos(p), -1j * math.sin(p)
    return np.array([[c, 0, 0, s], [0, c, s, 0], [0, s, c, 0], [s, 0, 0, c]])


def cp(lam):
    return np.diag([1, 1, 1, np.exp(1j * lam)])


# ---------------------------------------------------------------- noise
# src/noise.jl:52-131


# Written from the channels' definitions, independently of the engine's table:
# Pauli channels as weights over (I, X, Y, Z) with K = sqrt(w) sigma; the two
# damping channels from their action on |1>; the coherent errors as the rotation
# generators exp(-i theta sigma / 2).  The reference's quirks are part of the
# definitions: `model == :phase_flip` compares a String with a Symbol, so
# phase_flip uses Y like bit_phase_flip (src/noise.jl:78-81); rot_xyz divides the
# three rotations by sqrt(3) (src/noise.jl:117); two-qubit channels are all
# ordered kron pairs of the one-qubit set (src/noise.jl:126).
_PAULI_WEIGHTS = {
    "bit_flip": lambda p: {"I": 1 - p, "X": p},
    "phase_flip": lambda p: {"I": 1 - p, "Y": p},
    "bit_phase_flip": lambda p: {"I": 1 - p, "Y": p},
    "depolarizing": lambda p: {"I": 1 - p, "X": p / 3, "Y": p / 3, "Z": p / 3},
    "depolarizing_amp": lambda p: {"I": 1 - 3 * p / 4, "X": p / 4, "Y": p / 4, "Z": p / 4},
}


def _rot(axis, theta):
    s = {"X": GATE["X"], "Y": GATE["Y"], "Z": GATE["Z"]}[axis]
    return math.cos(theta / 2) * np.eye(2) - 1j * math.sin(theta / 2) * s


def noise_model(model, p, two_qubit=False):
    model = model.lower()
    if model in _PAULI_WEIGHTS:
        ops = [math.sqrt(w) * GATE[name] for name, w in _PAULI_WEIGHTS[model](p).items()]
    elif model in ("amplitude_damping", "phase_damping"):
        keep = np.diag([1.0, math.sqrt(1 - p)])  # no-jump: |1> shrinks by sqrt(1 - gamma)
        jump = np.zeros((2, 2))
        if model == "amplitude_damping":
            jump[0, 1] = math.sqrt(p)  # |1> -> |0>
        else:
            jump[1, 1] = math.sqrt(p)  # |1> -> |1>, phase information lost
        ops = [keep, jump]
    elif model in ("rot_x", "rot_y", "rot_z"):
        ops = [_rot(model[-1].upper(), p)]
    elif model == "rot_p":
        ops = [np.diag([1.0, np.exp(1j * p)])]
    elif model == "rot_xyz":
        ops = [_rot(a, p) / math.sqrt(3) for a in "XYZ"]
    elif model in ("mz", "m(z)", "mx", "m(x)", "my", "m(y)", "mr", "m(r)"):
        ops = [np.diag([1.0, 0.0]), np.diag([0.0, 1.0])]
    else:
        raise ValueError("Unknown quantum error model")
    ops = [np.asarray(o, dtype=complex) for o in ops]
    if not two_qubit:
        return ops
    out = []
    for a in ops:
        for b in ops:
            out.append(np.einsum("ij,kl->ikjl", a, b).reshape(4, 4))
    return out


# ---------------------------------------------------------------- hilbert
# src/hilbert.jl:18-159, src/decompose.jl:5-100


def _foldl_kron(mats):
    out = mats[0]
    for m in mats[1:]:
        out = np.kron(out, m)
    return out


def hilbert1(N, mat, qubit, control=-2):
    """hilbert(N, mat, qubit; control) (src/hilbert.jl:143-159)."""
    if N < qubit or N < control:
        raise ValueError("N must be larger than qubit")
    I2 = np.eye(2, dtype=complex)
    if control == -2:
        return _foldl_kron([mat if x == qubit else I2 for x in range(1, N + 1)])
    lst = _foldl_kron([mat if x == qubit else (GATE["P1"] if x == control else I2) for x in range(1, N + 1)])
    return lst + _foldl_kron([GATE["P0"] if x == control else I2 for x in range(1, N + 1)])


def _swap_control_target(m):
    """src/hilbert.jl:191-237."""
    if np.all(m @ GATE["SWAP"] - GATE["SWAP"] @ m == 0):
        return m
    p = [0, 2, 1, 3]
    return m[np.ix_(p, p)]


def _pauli_tensors(n, qubit=0, distance=2):
    """pauli_decomposition_tensor (src/decompose.jl:5-50); the first index varies fastest."""
    paulis = [GATE["I"], GATE["X"], GATE["Y"], GATE["Z"]]
    out = []
    for idx in itertools.product(range(4), repeat=n):
        idx = idx[::-1]  # Iterators.product varies the first index fastest
        mats = [paulis[i] for i in idx]
        if qubit:
            mats = [paulis[0]] * (qubit - 1) + mats
            for _ in range(distance - 1):
                mats.insert(qubit, paulis[0])
        out.append(_foldl_kron(mats))
    return out


def pauli_decomposition(A):
    n = int(round(math.log2(A.shape[0])))
    return [np.trace(A @ P) / 2 ** n for P in _pauli_tensors(n)]


def pauli_reconstruction(coefs, qubit, distance):
    n = int(round(math.log(len(coefs), 4)))
    tens = _pauli_tensors(n, qubit=qubit, distance=distance)
    return sum(c * T for c, T in zip(coefs, tens))


def cczx(sym, N, i, j, k):
    """CCZX (src/hilbert.jl:73-103)."""
    i, j, k = N - i, N - j, N - k
    H = np.zeros((2 ** N, 2 ** N), dtype=complex)
    for a in range(2 ** N):
        if sym == "CCZ":
            H[a, a] += -1 if ((a >> i) & (a >> j) & (a >> k) & 1) == 1 else 1
        else:
            if ((a >> i) & (a >> j) & 1) == 1:
                H[a, a ^ (1 << k)] += 1
            else:
                H[a, a] += 1
    return H


def hilbert2(N, mat, qubit, target, control=-2):
    """hilbert(N, mat, qubit, target; control) (src/hilbert.jl:18-70)."""
    distance = abs(qubit - target)
    if N < qubit or N < target or N < control:
        raise ValueError("N must be larger than qubits")
    I2 = np.eye(2, dtype=complex)
    final = _swap_control_target(mat) if qubit > target else mat
    if control == -2:
        if distance == 1:
            return _foldl_kron([final if x == qubit else I2 for x in range(1, N + 1) if x != target])
        coefs = pauli_decomposition(final)
        out = pauli_reconstruction(coefs, min(qubit, target), distance)
        for _ in range(N - max(qubit, target)):
            out = np.kron(out, I2)
        return out
    if distance == 1:
        lst = _foldl_kron([final if x == qubit else (GATE["P1"] if x == control else I2)
                           for x in range(1, N + 1) if x != target])
        return lst + _foldl_kron([GATE["P0"] if x == control else I2 for x in range(1, N + 1)])
    if np.array_equal(mat, GATE["CX"]):
        return cczx("CCX", N, qubit, control, target)
    if np.array_equal(mat, GATE["CZ"]):
        return cczx("CCZ", N, qubit, control, target)
    raise ValueError("Unsupported operation. Use 'CCZ' or 'CCX'.")


def hilbert3(N, mat, first):
    """hilbert3 (src/hilbert.jl:106-128)."""
    I2 = np.eye(2, dtype=complex)
    e = [I2] * N
    e.insert(first - 1, mat)
    for _ in range(3):
        e.pop(first)
    return _foldl_kron(e)


# ---------------------------------------------------------------- partial traces
# src/linalg.jl:83-230


def partial_trace1(psi, keep):
    N = int(round(math.log2(len(psi))))
    qi = N - keep + 1
    t = psi.reshape((2 ** (N - qi), 2, 2 ** (qi - 1)))  # row-major view of (right, mid, left)
    rho = np.zeros((2, 2), dtype=complex)
    for r in range(t.shape[0]):
        for l in range(t.shape[2]):
            v = t[r, :, l]
            rho += np.outer(v, v.conj())
    return rho


def partial_trace2(psi, k1, k2):
    """adjacent (src/linalg.jl:198-230) and non-adjacent (src/linalg.jl:83-86) pairs;
    both return the kept pair in (min, max) order."""
    N = int(round(math.log2(len(psi))))
    keep = sorted([k1, k2])
    return partial_trace_general(np.outer(psi, psi.conj()), N, keep)


def partial_trace_general(rho, N, keep):
    """partial_trace(rho, dims, trace_out) for qubits (src/linalg.jl:88-140)."""
    t = rho.reshape([2] * (2 * N))
    trace_out = [q for q in range(1, N + 1) if q not in keep]
    # axes 0..N-1 are row qubits 1..N (MSB first), N..2N-1 column qubits
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    rows = list(letters[:N])
    cols = list(letters[N:2 * N])
    for q in trace_out:
        cols[q - 1] = rows[q - 1]
    out = "".join(rows[q - 1] for q in keep) + "".join(cols[q - 1] for q in keep)
    red = np.einsum("".join(rows) + "".join(cols) + "->" + out, t)
    d = 2 ** len(keep)
    return red.reshape(d, d)


def calc_prob(psi, kraus, qubit, target=None):
    """__calc_prob (src/struct.jl:9-29)."""
    if target is None:
        pA = partial_trace1(psi, qubit)
    else:
        pA = partial_trace2(psi, qubit, target)
    return np.array([np.real(np.trace(K @ pA @ K.conj().T)) for K in kraus])


def weighted_sample(probs, u):
    """_weighted_sample (src/hilbert.jl:810-819), 0-based; None when no index."""
    for i, cw in enumerate(np.cumsum(probs)):
        if u <= cw:
            return i
    return None


def channel_traj(psi, kraus, qubit, target=None, u=None, forced=None):
    """__QuantumChannel_new_apply on a state (src/struct.jl:31-41)."""
    N = int(round(math.log2(len(psi))))
    p = calc_prob(psi, kraus, qubit, target)
    ind = forced if forced is not None else weighted_sample(p, u)
    E = hilbert1(N, kraus[ind], qubit) if target is None else hilbert2(N, kraus[ind], qubit, target)
    out = E @ psi
    return out / np.linalg.norm(out), ind, p


def born_measure_z(psi, qubit, u=None, forced=None):
    """born_measure_Z (src/hilbert.jl:682-696)."""
    N = int(round(math.log2(len(psi))))
    p0 = np.real(partial_trace1(psi, qubit))[0, 0]
    ind = forced if forced is not None else (0 if u < p0 else 1)
    out = hilbert1(N, [GATE["P0"], GATE["P1"]][ind], qubit) @ psi
    return out / np.linalg.norm(out), ind, p0


def born_measure_z2(psi, q1, q2, u=None, forced=None):
    """born_measure_Z(N, psi, q1, q2) (src/hilbert.jl:705-721), literally: the four
    projections by expand_multi_op, weights |psi' slist[k]|, _weighted_sample,
    normalize(slist[ind]); outcome 1-based as the reference returns it."""
    N = int(round(math.log2(len(psi))))
    slist = [expand_multi_op(names, [q1, q2], N) @ psi
             for names in (["P0", "P0"], ["P1", "P0"], ["P0", "P1"], ["P1", "P1"])]
    probs = np.array([abs(np.vdot(psi, s)) for s in slist])
    ind = (forced - 1) if forced is not None else weighted_sample(probs, u)
    out = slist[ind]
    return out / np.linalg.norm(out), ind + 1, probs


def dm_channel(rho, kraus, qubit, target=None):
    """__QuantumChannel_new_apply on rho (src/struct.jl:58-76)."""
    N = int(round(math.log2(rho.shape[0])))
    new = np.zeros_like(rho)
    for K in kraus:
        E = hilbert1(N, K, qubit) if target is None else hilbert2(N, K, qubit, target)
        new += E @ rho @ E.conj().T
    return new


def string_to_matrix(names):
    """string_to_matrix over a list of 1-qubit gate names (src/ops.jl:1016-1019)."""
    return _foldl_kron([GATE[s] for s in names])


def expand_multi_op(ops, qubits, N):
    """expand_multi_op (src/ops.jl:928-944)."""
    res = ["I"] * N
    for o, q in zip(ops, qubits):
        res[q - 1] = o
    return string_to_matrix(res)


def sample_direct(psi, u):
    """StatsBase's direct weighted sample: t = u*sum(w); first i with cumsum >= t."""
    w = np.abs(psi) ** 2
    cw = np.cumsum(w)
    t = np.asarray(u) * cw[-1]
    return np.searchsorted(cw, t, side="left")
