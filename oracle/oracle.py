"""ctypes binding of the C oracle (btoracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import it.

All matrices are passed as ordinary numpy arrays M[r, c] and converted to the
column-major complex128 layout of the C ABI here.  States are complex128
numpy vectors; density matrices are 2-D complex128 arrays rho[i, j].
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libbtoracle.so")
SRC = os.path.join(HERE, "btoracle.c")


def build(force=False):
    """Compile btoracle.c with gcc (OpenMP, no architecture-specific flags)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        try:  # a library built on another architecture does not load: rebuild it
            ctypes.CDLL(LIB)
            return LIB
        except OSError:
            pass
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-o", LIB, SRC, "-lm"]
    subprocess.check_call(cmd)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i, d, i64, u64 = ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_uint64
        sig = {
            "bto_hilbert1": (i, [i, P, P, i, i]),
            "bto_hilbert2": (i, [i, P, P, i, i, i]),
            "bto_hilbert3": (i, [i, P, P, i]),
            "bto_apply_k": (i, [i, P, i, P, P, i, P]),
            "bto_partial_trace1": (i, [i, P, i, P]),
            "bto_partial_trace2": (i, [i, P, i, i, P]),
            "bto_partial_trace_k": (i, [i, P, i, P, P]),
            "bto_calc_prob": (i, [i, P, i, i, i, i, P, P]),
            "bto_weighted_sample": (i, [i, P, d]),
            "bto_channel_traj": (i, [i, P, i, i, i, i, P, d, i, P, P]),
            "bto_born_measure_z": (i, [i, P, i, d, i, P, P]),
            "bto_born_measure_z2": (i, [i, P, i, i, d, i, P, P]),
            "bto_dm_gate": (i, [i, P, i, P, P, i, P]),
            "bto_dm_hilbert1": (i, [i, P, P, i, i]),
            "bto_dm_hilbert2": (i, [i, P, P, i, i, i]),
            "bto_dm_channel": (i, [i, P, i, i, i, i, P]),
            "bto_dm_dephase": (i, [i, P, i]),
            "bto_expect_pauli_sv": (d, [i, P, u64, u64]),
            "bto_expect_pauli_dm": (d, [i, P, u64, u64]),
            "bto_expect_matrix_sv": (d, [i, P, i, P, P, i, P]),
            "bto_sample": (i, [i, P, i64, P, P]),
            "bto_probs": (None, [i, P, P]),
            "bto_run_gates": (i64, [i, P, i, P, P, P, i]),
            "bto_num_threads": (i, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _cm(m):
    """numpy matrix -> contiguous column-major complex128 buffer."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128).T)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _ints(xs):
    return np.ascontiguousarray(np.asarray(xs, dtype=np.int32))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


def _nq(psi):
    return int(len(psi)).bit_length() - 1


def hilbert1(psi, m, q, control=-2):
    psi = np.array(psi, dtype=np.complex128)
    M = _cm(m)
    _check(lib().bto_hilbert1(_nq(psi), _ptr(psi), _ptr(M), q, control), "hilbert1")
    return psi


def hilbert2(psi, m, q, t, control=-2):
    psi = np.array(psi, dtype=np.complex128)
    M = _cm(m)
    _check(lib().bto_hilbert2(_nq(psi), _ptr(psi), _ptr(M), q, t, control), "hilbert2")
    return psi


def hilbert3(psi, m, first):
    psi = np.array(psi, dtype=np.complex128)
    M = _cm(m)
    _check(lib().bto_hilbert3(_nq(psi), _ptr(psi), _ptr(M), first), "hilbert3")
    return psi


def apply_k(psi, m, qubits, ctrls=()):
    psi = np.array(psi, dtype=np.complex128)
    M = _cm(m)
    q = _ints(qubits)
    c = _ints(ctrls if len(ctrls) else [0])
    _check(lib().bto_apply_k(_nq(psi), _ptr(psi), len(qubits), _ptr(q), _ptr(M), len(ctrls), _ptr(c)), "apply_k")
    return psi


def partial_trace(psi, keep):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    keep = list(keep)
    d = 2 ** len(keep)
    out = np.zeros(d * d, dtype=np.complex128)
    k = _ints(keep)
    _check(lib().bto_partial_trace_k(_nq(psi), _ptr(psi), len(keep), _ptr(k), _ptr(out)), "partial_trace")
    return out.reshape(d, d).T  # column-major -> rho[a, b]


def partial_trace2(psi, q, t):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    out = np.zeros(16, dtype=np.complex128)
    _check(lib().bto_partial_trace2(_nq(psi), _ptr(psi), q, t, _ptr(out)), "partial_trace2")
    return out.reshape(4, 4).T


def _kraus_buf(kraus):
    return np.ascontiguousarray(np.concatenate([_cm(K).ravel() for K in kraus]))


def calc_prob(psi, kraus, q, t=-1, k=None):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    if k is None:
        k = int(np.asarray(kraus[0]).shape[0]).bit_length() - 1
    K = _kraus_buf(kraus)
    out = np.zeros(len(kraus))
    _check(lib().bto_calc_prob(_nq(psi), _ptr(psi), k, q, t, len(kraus), _ptr(K), _ptr(out)), "calc_prob")
    return out


def weighted_sample(p, u):
    p = np.ascontiguousarray(p, dtype=np.float64)
    r = lib().bto_weighted_sample(len(p), _ptr(p), float(u))
    return None if r < 0 else r


def channel_traj(psi, kraus, q, t=-1, u=0.5, forced=-1):
    psi = np.array(psi, dtype=np.complex128)
    k = int(np.asarray(kraus[0]).shape[0]).bit_length() - 1
    K = _kraus_buf(kraus)
    br = ctypes.c_int(-1)
    probs = np.zeros(len(kraus))
    _check(lib().bto_channel_traj(_nq(psi), _ptr(psi), k, q, t, len(kraus), _ptr(K), float(u), int(forced),
                                  ctypes.byref(br), _ptr(probs)), "channel_traj")
    return psi, br.value, probs


def born_measure_z(psi, q, u=0.5, forced=-1):
    psi = np.array(psi, dtype=np.complex128)
    out = ctypes.c_int(-1)
    p0 = ctypes.c_double(0)
    _check(lib().bto_born_measure_z(_nq(psi), _ptr(psi), q, float(u), int(forced), ctypes.byref(out),
                                    ctypes.byref(p0)), "born_measure_z")
    return psi, out.value, p0.value


def born_measure_z2(psi, q1, q2, u=0.5, forced=-1):
    """born_measure_Z(N, psi, q1, q2): (state, outcome 1..4 or -1, weights[4])."""
    psi = np.array(psi, dtype=np.complex128)
    out = ctypes.c_int(-1)
    probs = np.zeros(4)
    _check(lib().bto_born_measure_z2(_nq(psi), _ptr(psi), int(q1), int(q2), float(u), int(forced),
                                     ctypes.byref(out), _ptr(probs)), "born_measure_z2")
    return psi, out.value, probs


def _dm_buf(rho):
    return np.ascontiguousarray(np.asarray(rho, dtype=np.complex128).T)  # column-major


def _dm_back(buf, dim):
    return buf.reshape(dim, dim).T.copy()


def dm_gate(rho, m, qubits, ctrls=()):
    dim = rho.shape[0]
    b = _dm_buf(rho)
    M = _cm(m)
    q = _ints(qubits)
    c = _ints(ctrls if len(ctrls) else [0])
    _check(lib().bto_dm_gate(_nq(np.empty(dim)), _ptr(b), len(qubits), _ptr(q), _ptr(M), len(ctrls), _ptr(c)),
           "dm_gate")
    return _dm_back(b, dim)


def dm_hilbert1(rho, m, q, control=-2):
    dim = rho.shape[0]
    b = _dm_buf(rho)
    M = _cm(m)
    _check(lib().bto_dm_hilbert1(_nq(np.empty(dim)), _ptr(b), _ptr(M), q, control), "dm_hilbert1")
    return _dm_back(b, dim)


def dm_hilbert2(rho, m, q, t, control=-2):
    dim = rho.shape[0]
    b = _dm_buf(rho)
    M = _cm(m)
    _check(lib().bto_dm_hilbert2(_nq(np.empty(dim)), _ptr(b), _ptr(M), q, t, control), "dm_hilbert2")
    return _dm_back(b, dim)


def dm_channel(rho, kraus, q, t=-1):
    dim = rho.shape[0]
    b = _dm_buf(rho)
    k = int(np.asarray(kraus[0]).shape[0]).bit_length() - 1
    K = _kraus_buf(kraus)
    _check(lib().bto_dm_channel(_nq(np.empty(dim)), _ptr(b), k, q, t, len(kraus), _ptr(K)), "dm_channel")
    return _dm_back(b, dim)


def dm_dephase(rho, q):
    dim = rho.shape[0]
    b = _dm_buf(rho)
    _check(lib().bto_dm_dephase(_nq(np.empty(dim)), _ptr(b), q), "dm_dephase")
    return _dm_back(b, dim)


def expect_pauli_sv(psi, xmask, zmask):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    return lib().bto_expect_pauli_sv(_nq(psi), _ptr(psi), int(xmask), int(zmask))


def expect_pauli_dm(rho, xmask, zmask):
    b = _dm_buf(rho)
    return lib().bto_expect_pauli_dm(_nq(np.empty(rho.shape[0])), _ptr(b), int(xmask), int(zmask))


def expect_matrix_sv(psi, m, qubits, ctrls=()):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    M = _cm(m)
    q = _ints(qubits)
    c = _ints(ctrls if len(ctrls) else [0])
    return lib().bto_expect_matrix_sv(_nq(psi), _ptr(psi), len(qubits), _ptr(q), _ptr(M), len(ctrls), _ptr(c))


def sample(psi, u):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros(len(u), dtype=np.int64)
    _check(lib().bto_sample(_nq(psi), _ptr(psi), len(u), _ptr(u), _ptr(out)), "sample")
    return out


def probs(psi):
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    out = np.zeros(len(psi))
    lib().bto_probs(_nq(psi), _ptr(psi), _ptr(out))
    return out


def run_gates(psi, gates, nthreads=0):
    """gates: list of (matrix, qubits).  Applies them in place with OpenMP."""
    ks = _ints([len(q) for _, q in gates])
    qs = _ints([x for _, q in gates for x in q])
    ms = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for m, _ in gates]))
    n = _nq(psi)
    r = lib().bto_run_gates(n, _ptr(psi), len(gates), _ptr(ks), _ptr(qs), _ptr(ms), int(nthreads))
    if r < 0:
        raise RuntimeError("oracle run_gates failed")
    return r


def num_threads():
    return lib().bto_num_threads()
