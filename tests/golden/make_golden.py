"""Generates tests/golden/kron_ref_cases.npz from the literal restatement of the
reference's operator construction (oracle/kron_ref.py).

Julia is not installed where this runs, so the reference itself cannot produce
vectors; kron_ref follows the reference's own algorithm step by step (full
operators by kron, SWAP permutation, Pauli reconstruction of non-adjacent
pairs, CCZX) and these fixtures freeze its outputs on seeded inputs.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import kron_ref as K  # noqa: E402

OUT = os.path.join(HERE, "kron_ref_cases.npz")


def rand_state(rng, n):
    v = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return v / np.linalg.norm(v)


def rand_unitary(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def main():
    rng = np.random.default_rng(20240601)
    N = 5
    data = {}
    # 1q gates, every qubit, with and without a control
    cases = []
    for q in range(1, N + 1):
        for c in [-2] + [x for x in range(1, N + 1) if x != q][:2]:
            cases.append(("g1", rand_unitary(rng, 2), q, -1, c))
    # 2q gates: adjacent, non-adjacent, both orders, controlled adjacent, CCX/CCZ non-adjacent
    for q, t in [(1, 2), (2, 1), (2, 4), (5, 2), (1, 5), (4, 3)]:
        cases.append(("g2", rand_unitary(rng, 4), q, t, -2))
    for q, t, c in [(2, 3, 5), (4, 3, 1), (1, 2, 4)]:
        cases.append(("g2", rand_unitary(rng, 4), q, t, c))
    for q, t, c in [(1, 3, 5), (5, 2, 3), (2, 5, 1)]:
        cases.append(("g2", K.GATE["CX"], q, t, c))
        cases.append(("g2", K.GATE["CZ"], q, t, c))
    cases.append(("g3", rand_unitary(rng, 8), 2, -1, -2))
    for i, (kind, m, q, t, c) in enumerate(cases):
        psi = rand_state(rng, N)
        if kind == "g1":
            E = K.hilbert1(N, m, q, c)
        elif kind == "g2":
            E = K.hilbert2(N, m, q, t, c)
        else:
            E = K.hilbert3(N, m, q)
        data[f"gate{i}_kind"] = np.array([{"g1": 1, "g2": 2, "g3": 3}[kind]])
        data[f"gate{i}_meta"] = np.array([q, t, c])
        data[f"gate{i}_mat"] = m
        data[f"gate{i}_in"] = psi
        data[f"gate{i}_out"] = E @ psi
    data["ngates"] = np.array([len(cases)])

    # partial traces and channel probabilities (Noise2 depolarizing 0.5 as in the reference test)
    kr2 = K.noise_model("depolarizing", 0.5, two_qubit=True)
    kr1 = K.noise_model("amplitude_damping", 0.3)
    pairs = [(2, 3), (3, 2), (1, 4), (5, 2)]
    for i, (q, t) in enumerate(pairs):
        psi = rand_state(rng, N)
        data[f"pt{i}_in"] = psi
        data[f"pt{i}_meta"] = np.array([q, t])
        data[f"pt{i}_rho2"] = K.partial_trace2(psi, q, t)
        data[f"pt{i}_rho1"] = K.partial_trace1(psi, q)
        data[f"pt{i}_probs2"] = K.calc_prob(psi, kr2, q, t)
        data[f"pt{i}_probs1"] = K.calc_prob(psi, kr1, q)
        # trajectory step with a forced branch and with a drawn uniform
        out, ind, _ = K.channel_traj(psi, kr2, q, t, forced=5)
        data[f"pt{i}_traj_forced5"] = out
        u = float(rng.random())
        out, ind, _ = K.channel_traj(psi, kr1, q, u=u)
        data[f"pt{i}_traj_u"] = np.array([u])
        data[f"pt{i}_traj_branch"] = np.array([ind])
        data[f"pt{i}_traj_out"] = out
        for o in (0, 1):
            out, _, p0 = K.born_measure_z(psi, q, forced=o)
            data[f"pt{i}_meas{o}"] = out
            data[f"pt{i}_p0"] = np.array([p0])
    data["npt"] = np.array([len(pairs)])

    # density-matrix gate and channel steps
    Nd = 3
    psi = rand_state(rng, Nd)
    phi = rand_state(rng, Nd)
    rho = 0.7 * np.outer(psi, psi.conj()) + 0.3 * np.outer(phi, phi.conj())
    data["dm_in"] = rho
    U = rand_unitary(rng, 4)
    data["dm_U"] = U
    data["dm_gate_out"] = K.hilbert2(Nd, U, 3, 1) @ rho @ K.hilbert2(Nd, U, 3, 1).conj().T
    data["dm_ch2_out"] = K.dm_channel(rho, kr2, 1, 2)
    data["dm_ch1_out"] = K.dm_channel(rho, kr1, 3)
    # observables through expand_multi_op
    psi = rand_state(rng, N)
    data["obs_in"] = psi
    strings = [(["Z"], [3]), (["X", "Y"], [1, 4]), (["Z", "Z"], [2, 3]), (["Y", "X", "Z"], [5, 1, 2]), (["T"], [2])]
    vals = [np.real(psi.conj() @ K.expand_multi_op(o, q, N) @ psi) for o, q in strings]
    data["obs_vals"] = np.array(vals)
    data["obs_rho_vals"] = np.array([np.real(np.trace(rho @ K.expand_multi_op(o, q, Nd)))
                                     for o, q in [(["Z"], [1]), (["X", "Z"], [1, 3]), (["Y", "Y"], [2, 3])]])
    # sampling with fixed uniforms
    u = rng.random(200)
    data["samp_in"] = psi
    data["samp_u"] = u
    data["samp_out"] = K.sample_direct(psi, u)
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
