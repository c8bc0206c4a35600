"""Host-side gate matrices with the reference's exact values.

The engine receives matrices already built; values must equal the ones the
reference builds (BlueTangle.jl src/gates.jl:22-59 for the constant table,
src/gates.jl:369-453 for the parametric gates and the name parser), including
the 10-significant-digit rounding of T/TD/CT/CTD (src/gates.jl:32-33, :47-48).
Matrices are ordinary numpy arrays M[r, c]; qubit order inside a two-qubit
matrix is |b_qubit b_target> with `qubit` the most significant bit.
"""
import ast
import math
import operator
import re

import numpy as np

__all__ = ["gate", "gates", "gates_with_phase", "one_qubit_gates", "two_qubit_gates", "is_measurement"]


def _round_sig(z, sig=10):
    def r(v):
        return 0.0 if v == 0 else float(f"{v:.{sig - 1}e}")
    return complex(r(z.real), r(z.imag))


_S2 = 1 / math.sqrt(2)
_T = _round_sig(complex(math.cos(math.pi / 4), math.sin(math.pi / 4)))
_TD = _round_sig(complex(math.cos(-math.pi / 4), math.sin(-math.pi / 4)))


def _c(rows):
    return np.array(rows, dtype=np.complex128)


gate = {
    "I": _c([[1, 0], [0, 1]]),
    "X": _c([[0, 1], [1, 0]]),
    "SX": 0.5 * _c([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "XSQRT": 0.5 * _c([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "Y": _c([[0, -1j], [1j, 0]]),
    "Z": _c([[1, 0], [0, -1]]),
    "H": _S2 * _c([[1, 1], [1, -1]]),
    "S": _c([[1, 0], [0, 1j]]),
    "SD": _c([[1, 0], [0, -1j]]),
    "T": _c([[1, 0], [0, _T]]),
    "TD": _c([[1, 0], [0, _TD]]),
    "HSP": _S2 * _c([[1, -1j], [1, 1j]]),
    "HY": _S2 * _c([[1, 1j], [1, -1j]]),
    "H2": _c([[0.5, 0.5, 0.5, 0.5], [0.5, -0.5, 0.5, -0.5], [0.5, 0.5, -0.5, -0.5], [0.5, -0.5, -0.5, 0.5]]),
    "P0": _c([[1, 0], [0, 0]]),
    "P1": _c([[0, 0], [0, 1]]),
    "SP": _c([[0, 1], [0, 0]]),
    "SM": _c([[0, 0], [1, 0]]),
    "CX": _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]),
    "CNOT": _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]),
    "CY": _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, -1j], [0, 0, 1j, 0]]),
    "CZ": _c(np.diag([1, 1, 1, -1])),
    "CS": _c(np.diag([1, 1, 1, 1j])),
    "CT": _c(np.diag([1, 1, 1, _T])),
    "CTD": _c(np.diag([1, 1, 1, _TD])),
    "CSD": _c(np.diag([1, 1, 1, -1j])),
    "CI": _c(np.eye(4)),
    "CH": _c([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, _S2, _S2], [0, 0, _S2, -_S2]]),
    "SWAP": _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]),
    "ISWAP": _c([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]]),
    "FSWAP": _c([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, -1]]),
    "SYC": _c([[1, 0, 0, 0], [0, 0, -1j, 0], [0, -1j, 0, 0], [0, 0, 0, np.exp(-1j * math.pi / 6)]]),
    "ECR": _S2 * _c([[0, 1, 0, 1j], [1, 0, -1j, 0], [0, 1j, 0, 1], [-1j, 0, 1, 0]]),
    "CCX": _c(np.eye(8)[[0, 1, 2, 3, 4, 5, 7, 6]]),
    "CCZ": _c(np.diag([1, 1, 1, 1, 1, 1, 1, -1])),
}

one_qubit_gates = ["I", "X", "Y", "Z", "SX", "XSQRT", "H", "T", "S", "SD", "P", "U2", "U3"]
two_qubit_gates = ["CX", "CNOT", "CY", "CZ", "CP", "RXX", "RYY", "RZZ", "RXY", "GIVENS", "FSIM", "SWAP",
                   "ISWAP", "FSWAP", "SYC", "ECR"]
gates_with_phase = ["P", "RX", "RY", "RZ", "U1", "U2", "U3", "CP", "GIVENS", "FSIM", "SWAPA", "RXX", "RYY",
                    "RZZ", "RXY"]


def _P(lam):
    return _c([[1, 0], [0, np.exp(1j * lam)]])


def _RX(t):
    return _c([[math.cos(t / 2), -1j * math.sin(t / 2)], [-1j * math.sin(t / 2), math.cos(t / 2)]])


def _RY(t):
    return _c([[math.cos(t / 2), -math.sin(t / 2)], [math.sin(t / 2), math.cos(t / 2)]])


def _RZ(t):
    return _c([[np.exp(-1j * t / 2), 0], [0, np.exp(1j * t / 2)]])


def _U2(phi, lam):
    return (1 / math.sqrt(2)) * _c([[1, -np.exp(1j * lam)], [np.exp(1j * phi), np.exp(1j * (phi + lam))]])


def _U3(t, phi, lam):
    return _c([[math.cos(t / 2), -np.exp(1j * lam) * math.sin(t / 2)],
               [np.exp(1j * phi) * math.sin(t / 2), np.exp(1j * (phi + lam)) * math.cos(t / 2)]])


def _CP(lam):
    return _c(np.diag([1, 1, 1, np.exp(1j * lam)]))


def _GIVENS(t):
    return _c([[1, 0, 0, 0], [0, math.cos(t), -math.sin(t), 0], [0, math.sin(t), math.cos(t), 0], [0, 0, 0, 1]])


def _FSIM(t, phi):
    return _c([[1, 0, 0, 0], [0, math.cos(t), -1j * math.sin(t), 0], [0, -1j * math.sin(t), math.cos(t), 0],
               [0, 0, 0, np.exp(1j * phi)]])


def _SWAPA(a):
    e = np.exp(1j * math.pi * a)
    return 0.5 * _c([[2, 0, 0, 0], [0, 1 + e, 1 - e, 0], [0, 1 - e, 1 + e, 0], [0, 0, 0, 2]])


def _RXX(p):
    c, s = math.cos(p), -1j * math.sin(p)
    return _c([[c, 0, 0, s], [0, c, s, 0], [0, s, c, 0], [s, 0, 0, c]])


def _RYY(p):
    c, s = math.cos(p), math.sin(p)
    return _c([[c, 0, 0, 1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [1j * s, 0, 0, c]])


def _RZZ(p):
    return _c(np.diag([np.exp(-1j * p / 2), np.exp(1j * p / 2), np.exp(1j * p / 2), np.exp(-1j * p / 2)]))


def _RXY(p):
    c, s = math.cos(p), -1j * math.sin(p)
    return _c([[1, 0, 0, 0], [0, c, s, 0], [0, s, c, 0], [0, 0, 0, 1]])


local_functions = {"P": _P, "RX": _RX, "RY": _RY, "RZ": _RZ, "U1": _P, "U2": _U2, "U3": _U3, "CP": _CP,
                   "GIVENS": _GIVENS, "SWAPA": _SWAPA, "FSIM": _FSIM, "RXX": _RXX, "RYY": _RYY, "RZZ": _RZZ,
                   "RXY": _RXY}

_OPS = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow, ast.USub: operator.neg, ast.UAdd: operator.pos}


def _eval_number(text):
    """Evaluates a gate argument the way Julia's parser reads it: numbers, pi/π,
    juxtaposition ("0.1pi" is 0.1*pi), + - * / ^ and parentheses."""
    t = text.strip().replace("π", "pi")
    t = re.sub(r"(\d)\s*(pi)", r"\1*\2", t)
    t = t.replace("^", "**")
    node = ast.parse(t, mode="eval").body

    def ev(n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name) and n.id == "pi":
            return math.pi
        if isinstance(n, ast.BinOp) and type(n.op) in _OPS:
            return _OPS[type(n.op)](ev(n.left), ev(n.right))
        if isinstance(n, ast.UnaryOp) and type(n.op) in _OPS:
            return _OPS[type(n.op)](ev(n.operand))
        raise ValueError(f"cannot parse gate argument {text!r}")
    return ev(node)


def clean_name(name):
    return name.split("(")[0].upper()


def is_measurement(name):
    """_is_it_measurement (src/gates.jl:334-338)."""
    return name.upper() in ("MZ", "M(Z)", "MX", "M(X)", "MY", "M(Y)", "MR", "M(R)")


def gate_arguments(name):
    inner = name.split("(", 1)[1].rsplit(")", 1)[0]
    return [_eval_number(e) for e in inner.split(",")]


def gates(name):
    """gates(op_name) (src/gates.jl:369-453): matrix of a named gate."""
    cn = clean_name(name)
    up = name.upper()
    if cn in local_functions:
        return local_functions[cn](*gate_arguments(name))
    if up in ("M(Z)", "MZ", "M(R)", "MR", "RES"):
        return gate["I"].copy()
    if up in ("M(X)", "MX"):
        return gate["H"].copy()
    if up in ("M(Y)", "MY"):
        return gate["HSP"].copy()
    if up in gate:
        return gate[up].copy()
    raise KeyError(f"Gate {name} not found")
