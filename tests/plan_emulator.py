"""Host emulation of compiled plans (test infrastructure).

A plan needs no device until it runs: the planner (tile bits, register phases)
and the op encoding (classes, factored forms, the folded scalar) run on the host,
and bt_plan_pass_ops reports every compiled pass as ops on global bits with their
encoded entries.  Applying those ops to a numpy state in order reproduces what
the pass kernels compute, so whole compiled plans can be checked against the
oracle on the CPU.  The GPU tests check the kernels' arithmetic for every op
type; these check everything the host decides.
"""
import ctypes

import numpy as np

from bluetangle_gpu import _lib as L
from bluetangle_gpu.engine import Plan

G1, D1, G2, D2, P2, CX, SW, X1, R1, RX1, DH, HB, RN, RXN = range(1, 15)
MAX_OPS, MAX_REALS = 192, 4096


class HostCtx:
    """Stands in for a context: errors come from the thread's last message."""
    h = None

    def check(self, rc):
        L.check(rc, None)


def host_plan(n, repr="sv", prec="c128"):
    return Plan(n, repr, prec, HostCtx())


def passes(plan):
    """[(kind, ops, mats)] of the compiled plan; kind 0: ops is (nops, 6)."""
    lib = L.lib()
    P = ctypes.c_void_p
    out = []
    ops = np.zeros(6 * MAX_OPS, dtype=np.int32)
    mats = np.zeros(MAX_REALS, dtype=np.float64)
    kind, nops = ctypes.c_int(), ctypes.c_int()
    for i in range(plan.stats()["passes"]):
        L.check(lib.bt_plan_pass_ops(plan.h, i, ctypes.byref(kind), ctypes.byref(nops), ops.ctypes.data_as(P),
                                     mats.ctypes.data_as(P), MAX_OPS, MAX_REALS))
        if kind.value == 0:
            out.append((0, ops[:6 * nops.value].reshape(-1, 6).copy(), mats.copy()))
        else:
            out.append((1, ops[:8].copy(), mats.copy()))
    return out


def _idx(nbits, fixed0=(), fixed1=()):
    i = np.arange(2 ** nbits, dtype=np.int64)
    keep = np.ones(i.size, dtype=bool)
    for b in fixed0:
        keep &= ((i >> b) & 1) == 0
    for b in fixed1:
        keep &= ((i >> b) & 1) == 1
    return i[keep]


def _op(x, nbits, r, m):
    t, b0, b1, fl, unit, off = (int(v) for v in r)
    c = lambda e: complex(m[off + 2 * e], m[off + 2 * e + 1])  # noqa: E731
    if t in (G1, D1, R1, RX1, X1, DH, HB, RN, RXN):
        a = _idx(nbits, fixed0=[b0])
        b = a | (1 << b0)
        x0, x1 = x[a].copy(), x[b].copy()
        if t == G1:
            x[a], x[b] = c(0) * x0 + c(1) * x1, c(2) * x0 + c(3) * x1
        elif t == D1:
            x[a], x[b] = c(0) * x0, c(1) * x1
        elif t == R1:
            p = m[off:off + 4]
            x[a], x[b] = p[0] * x0 + p[1] * x1, p[2] * x0 + p[3] * x1
        elif t == RX1:
            ca, cb = m[off], m[off + 1]
            x[a], x[b] = ca * x0 + 1j * cb * x1, 1j * cb * x0 + ca * x1
        elif t == X1:
            x[a], x[b] = (x1, x0) if unit else (c(0) * x1, c(1) * x0)
        elif t == DH:
            q = {2: -1, 3: 1j, 4: -1j}.get(unit, c(0) if unit == 0 else None)
            if fl & 1:
                x[a] = q * x0
            else:
                x[b] = q * x1
        elif t == HB:
            s01, s10, s11 = (-1 if fl & 1 else 1), (-1 if fl & 2 else 1), (-1 if fl & 4 else 1)
            x[a], x[b] = x0 + s01 * x1, s10 * x0 + s11 * x1
        elif t == RN:
            p, q, s = m[off], m[off + 1], (-1 if fl & 1 else 1)
            if fl & 2:
                x[a], x[b] = p * x0 + x1, s * x0 + q * x1
            else:
                x[a], x[b] = x0 + p * x1, q * x0 + s * x1
        else:  # RXN
            tt = m[off]
            if fl & 2:
                x[a], x[b] = -1j * tt * x0 + x1, x0 - 1j * tt * x1
            else:
                x[a], x[b] = x0 + 1j * tt * x1, 1j * tt * x0 + x1
        return
    # two-bit ops: matrix index r = 2 * bit(b0) + bit(b1)
    base = _idx(nbits, fixed0=[b0, b1])
    q = [base, base | (1 << b1), base | (1 << b0), base | (1 << b0) | (1 << b1)]
    X = [x[k].copy() for k in q]
    if t == G2:
        for rr in range(4):
            x[q[rr]] = sum(c(4 * rr + cc) * X[cc] for cc in range(4))
    elif t == D2:
        for rr in range(4):
            x[q[rr]] = c(rr) * X[rr]
    elif t in (P2, CX, SW):
        perm = {CX: [0, 1, 3, 2], SW: [0, 2, 1, 3]}.get(t) or [(fl >> (2 * rr)) & 3 for rr in range(4)]
        for rr in range(4):
            x[q[rr]] = X[perm[rr]] if (t != P2 or unit) else c(rr) * X[perm[rr]]
    else:
        raise ValueError(f"unknown op type {t}")


def _sweep(x, nbits, r, m):
    k = int(r[0])
    bits = [int(v) for v in r[1:1 + k]]
    cmask = (int(r[6]) & 0xFFFFFFFF) | ((int(r[7]) & 0xFFFFFFFF) << 32)
    ctrl = [b for b in range(nbits) if (cmask >> b) & 1]
    d = 1 << k
    M = (m[:2 * d * d:2] + 1j * m[1:2 * d * d:2]).reshape(d, d)
    base = _idx(nbits, fixed0=bits, fixed1=ctrl)
    cols = []
    for col in range(d):
        pat = 0
        for i, b in enumerate(bits):
            if (col >> (k - 1 - i)) & 1:
                pat |= 1 << b
        cols.append(base | pat)
    X = [x[cc].copy() for cc in cols]
    for row in range(d):
        x[cols[row]] = sum(M[row, col] * X[col] for col in range(d))


def run(plan, psi):
    """The compiled plan applied to psi (a state vector, or vec(rho) column-major)."""
    x = np.asarray(psi, dtype=np.complex128).ravel(order="F").copy()
    nbits = int(x.size).bit_length() - 1
    for kind, ops, mats in passes(plan):
        if kind:
            _sweep(x, nbits, ops, mats)
        else:
            for r in ops:
                _op(x, nbits, r, mats)
    return x
