"""A QASM circuit compiled into a device plan equals the oracle applying the
reader's ops one by one (complex128 within 1e-12; complex64 within 2e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_qasm(n, depth, rng):
    lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', f"qreg q[{n}];"]
    one = ["h", "x", "s", "sdg", "t", "tdg", "sx"]
    for _ in range(depth):
        for q in range(n):
            r = rng.integers(0, 4)
            if r == 0:
                lines.append(f"{one[rng.integers(0, len(one))]} q[{q}];")
            elif r == 1:
                lines.append(f"u3({rng.uniform(0, 3):.4f},{rng.uniform(0, 3):.4f},{rng.uniform(0, 3):.4f}) q[{q}];")
            else:
                lines.append(f"r{'xyz'[rng.integers(0, 3)]}({rng.uniform(0, 3):.4f}) q[{q}];")
        for q in range(0, n - 1, 2):
            a, b = (q, q + 1) if rng.random() < 0.5 else (q + 1, q)
            g = rng.integers(0, 5)
            lines.append([f"cx q[{a}],q[{b}];", f"cz q[{a}],q[{b}];", f"cp(0.37) q[{a}],q[{b}];",
                          f"rzz(0.21) q[{a}],q[{b}];", f"swap q[{a}],q[{b}];"][g])
        lines.append(f"ccx q[0],q[{n - 1}],q[{n // 2}];")
    return "\n".join(lines)


@pytest.mark.parametrize("prec,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_qasm_plan_matches_oracle(ctx, oracle, prec, tol):
    import bluetangle_gpu as bt
    import bluetangle_gpu.qasm as Q
    n = 9
    text = random_qasm(n, 6, np.random.default_rng(4))
    plan, nq = Q.qasm_plan(text, prec=prec)
    assert nq == n
    st = plan.run(bt.zero_state(n, prec))
    psi = np.zeros(2 ** n, complex)
    psi[0] = 1
    for op in Q.from_qasm(text):
        qs = [op.qubit] if op.q == 1 or op.target_qubit < 0 else [op.qubit, op.target_qubit]
        cs = [op.control] if op.control != -2 else []
        psi = oracle.apply_k(psi, op.mat, qs, cs)
    assert np.abs(st.to_numpy() - psi).max() < tol
