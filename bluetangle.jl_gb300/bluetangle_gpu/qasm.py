"""OpenQASM 2 circuits into ops and device plans.

from_qasm follows the reference's reader (from_qasm, BlueTangle.jl
src/qasm.jl:285-421) statement by statement: comments stripped, statements split
at ';', boilerplate (OPENQASM, include, qreg, creg, opaque, gate, barrier)
skipped; measure -> MZ, reset -> RES, one-qubit gates (sdg -> SD, tdg -> TD,
sx -> XSQRT), rx/ry/rz/u1/u2/u3 with their angle expressions, cu1/cp/cu3/crx/
cry/crz and cx/cy/cz as controlled one-qubit ops (cx on the controlled-X path,
src/qasm.jl:371-375), swap/iswap/fswap/syc/ecr, ccx/ccy/ccz/cswap, and
rxx/ryy/rzz/rxy/givens/fsim/swapa; anything else is an error.  Qubit tokens
like q[3] map to package qubits (0-based -> 1-based), any register name.

qasm_plan compiles a measurement-free circuit into a device plan (fused tile
passes), the form in which a circuit read from QASM runs on the GPU.
"""
import os
import re

from .engine import Plan
from .ops import Op, OpQC

__all__ = ["from_qasm", "qasm_plan", "qasm_num_qubits"]

_BOILER = ("openqasm", "include", "qreg", "creg", "opaque", "gate", "barrier")


def _q1(tok):
    m = re.search(r"\[(\d+)\]\s*[;,]?\s*$", tok.strip())
    if m is None:
        raise ValueError(f"Expected qubit like q[<int>]; got: {tok}")
    return int(m.group(1)) + 1


def _statements(text):
    src = re.sub(r"//.*", "", text)
    src = "\n".join(line.strip() for line in src.split("\n"))
    return [s.strip() + ";" for s in src.split(";") if s.strip()]


_Q = r"([^\s,;]+)"      # a qubit token
_QL = r"([^\s;]+)"      # the last qubit token of a statement
_A = r"\s*\(\s*(.+?)\s*\)\s+"


def _rules():
    """(pattern, builder) pairs, tried in order (as the reference's chain of matches)."""
    r = []

    def add(pat, fn):
        r.append((re.compile(pat), fn))

    add(r"^measure\s+([^\s]+)\s*->\s*([^\s]+)\s*;", lambda m: [Op("MZ", _q1(m[1]))])
    add(r"^reset\s+([^\s;]+)\s*;", lambda m: [Op("RES", _q1(m[1]))])

    def unary(m):
        kw = m[1]
        name = {"sdg": "SD", "tdg": "TD", "sx": "XSQRT"}.get(kw, kw.upper())
        return [Op(name, _q1(m[2]))]

    add(r"^(x|y|z|h|s|sdg|t|tdg|sx)\s+" + _QL + r"\s*;", unary)
    add(r"^(rx|ry|rz)" + _A + _QL + r"\s*;", lambda m: [Op(f"{m[1]}({m[2].strip()})", _q1(m[3]))])
    add(r"^u1" + _A + _QL + r"\s*;", lambda m: [Op(f"U1({m[1].strip()})", _q1(m[2]))])
    add(r"^u2\s*\(\s*(.+?)\s*,\s*(.+?)\s*\)\s+" + _QL + r"\s*;",
        lambda m: [Op(f"U2({m[1].strip()},{m[2].strip()})", _q1(m[3]))])
    add(r"^u3\s*\(\s*(.+?)\s*,\s*(.+?)\s*,\s*(.+?)\s*\)\s+" + _QL + r"\s*;",
        lambda m: [Op(f"U3({m[1].strip()},{m[2].strip()},{m[3].strip()})", _q1(m[4]))])
    add(r"^(?:cu1|cp)" + _A + _Q + r"\s*,\s*" + _QL + r"\s*;",
        lambda m: [Op(f"U1({m[1].strip()})", _q1(m[3]), control=_q1(m[2]))])

    def cu3(m):
        th, ph, la = m[1].strip(), m[2].strip(), m[3].strip()
        ctrl, tgt = _q1(m[4]), _q1(m[5])
        if ph == "0" and la == "0":
            return [Op(f"ry({th})", tgt, control=ctrl)]
        return [Op(f"U3({th},{ph},{la})", tgt, control=ctrl)]

    add(r"^cu3\s*\(\s*(.+?)\s*,\s*(.+?)\s*,\s*(.+?)\s*\)\s+" + _Q + r"\s*,\s*" + _QL + r"\s*;", cu3)
    for kw in ("rx", "ry", "rz"):
        add(r"^c" + kw + _A + _Q + r"\s*,\s*" + _QL + r"\s*;",
            lambda m, kw=kw: [Op(f"{kw}({m[1].strip()})", _q1(m[3]), control=_q1(m[2]))])

    def binary(m):
        head, a, b = m[1], _q1(m[2]), _q1(m[3])
        if head in ("cx", "cnot"):
            return [Op("X", b, control=a)]
        if head == "cy":
            return [Op("Y", b, control=a)]
        if head == "cz":
            return [Op("Z", b, control=a)]
        return [Op(head.upper(), a, b)]

    add(r"^(cx|cnot|cy|cz|swap|iswap|fswap|syc|ecr)\s+" + _Q + r"\s*,\s*" + _QL + r"\s*;", binary)

    def ternary(m):
        head, a, b, c = m[1], _q1(m[2]), _q1(m[3]), _q1(m[4])
        if head == "cswap":
            return [Op("CSWAP", b, a, c)]
        return [Op(head.upper(), a, b, c)]

    add(r"^(ccx|ccy|ccz|cswap)\s+" + _Q + r"\s*,\s*" + _Q + r"\s*,\s*" + _QL + r"\s*;", ternary)
    add(r"^(rxx|ryy|rzz|rxy)" + _A + _Q + r"\s*,\s*" + _QL + r"\s*;",
        lambda m: [Op(f"{m[1].upper()}({m[2].strip()})", _q1(m[3]), _q1(m[4]))])
    add(r"^givens" + _A + _Q + r"\s*,\s*" + _QL + r"\s*;",
        lambda m: [Op(f"GIVENS({m[1].strip()})", _q1(m[2]), _q1(m[3]))])
    add(r"^fsim\s*\(\s*(.+?)\s*,\s*(.+?)\s*\)\s+" + _Q + r"\s*,\s*" + _QL + r"\s*;",
        lambda m: [Op(f"FSIM({m[1].strip()},{m[2].strip()})", _q1(m[3]), _q1(m[4]))])
    add(r"^swapa" + _A + _Q + r"\s*,\s*" + _QL + r"\s*;",
        lambda m: [Op(f"SWAPA({m[1].strip()})", _q1(m[2]), _q1(m[3]))])
    return r


_RULES = _rules()


def from_qasm(qasm):
    """OpenQASM 2 text (or a path to a file) -> list of ops."""
    text = open(qasm).read() if os.path.isfile(qasm) else str(qasm)
    ops = []
    for stmt in _statements(text):
        s = stmt.lower()
        if s.startswith(_BOILER):
            continue
        for pat, fn in _RULES:
            m = pat.match(s)
            if m is not None:
                ops.extend(fn(m))
                break
        else:
            raise ValueError(f"Unsupported or unrecognized statement: {stmt}")
    return ops


def qasm_num_qubits(ops):
    m = 0
    for op in ops:
        m = max(m, op.qubit, getattr(op, "target_qubit", -1), getattr(op, "control", -2))
    return m


def qasm_plan(qasm, n=None, prec="c64", ctx=None, fused=True):
    """A measurement-free QASM circuit compiled into a device plan (fused passes)."""
    ops = from_qasm(qasm)
    n = n or qasm_num_qubits(ops)
    plan = Plan(n, "sv", prec, ctx)
    for op in ops:
        if getattr(op, "type", "") == "🔬" or isinstance(op, OpQC):
            raise ValueError(f"{op!r} cannot be part of a plan (measurement or reset)")
        plan.add(op)
    return plan.compile(fused), n
