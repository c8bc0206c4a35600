"""Variational circuits: variational_apply and the parameter-shift gradient.

The reference evaluates a variational circuit one call at a time
(variational_apply, BlueTangle.jl src/vqa.jl:420-456) and its parameter-shift
gradient (loss_and_grad_paramshift, src/vqa.jl:590-611) as 2P + 1 sequential
circuit evaluations: the loss at p, and for every parameter i the loss at
p + pi/2 e_i and p - pi/2 e_i, g_i = (l(p + pi/2 e_i) - l(p - pi/2 e_i)) / 2.

Here the 2P + 1 evaluations are one batch:
  * states of n <= 14 (complex64) / 13 (complex128) qubits: one program, one CTA
    per shifted circuit, each with its own gate matrices, all in one launch;
  * larger states: the circuit compiled once into fused passes; each evaluation
    rewrites the parametrised gates' matrices in place and runs the passes.
The loss is <H> of a Pauli sum given as (coef, xmask, zmask) terms (the
reference's loss(state) = real(expect(state, H)) for a Hamiltonian matrix H).
"""
import ctypes
import inspect
import os

import numpy as np

from . import _lib as L
from .engine import Context, GPUState, Plan, _ptr, apply, apply_matrix

__all__ = ["arg_counts", "variational_apply", "loss", "losses", "loss_and_grad_paramshift", "SHIFT"]

SHIFT = np.pi / 2  # for Pauli / Pauli-string rotations (src/vqa.jl:594)


def arg_counts(ops):
    """Parameters of each op: the argument count of a parametrised op's matrix
    function (_find_argument_number), 0 for fixed ops (src/vqa.jl:224-235)."""
    out = []
    for op in ops:
        if getattr(op, "type", "") == "f":
            out.append(len(inspect.signature(op.mat).parameters))
        else:
            out.append(0)
    return out


def _bound(ops, counts, p):
    """(op, matrix) per op with the parametrised ops evaluated at p, in order."""
    if sum(counts) != len(p):
        raise ValueError(f"the ansatz takes {sum(counts)} parameters, {len(p)} given")
    out, c = [], 0
    for op, k in zip(ops, counts):
        if k:
            out.append((op, np.asarray(op.mat(*p[c:c + k]), dtype=np.complex128)))
            c += k
        else:
            out.append((op, None))
    if c != len(p):
        raise ValueError(f"the ansatz takes {c} parameters, {len(p)} given")
    return out


def _qubits(op):
    qs = [op.qubit] if op.q == 1 else [op.qubit, op.target_qubit]
    return qs, ([op.control] if op.control != -2 else [])


def variational_apply(pars, ops, n, prec="c128", ctx=None, state=None):
    """The ansatz applied at pars to |0...0> (or `state`), as the reference's
    variational_apply (noiseless)."""
    counts = arg_counts(ops)
    st = state if state is not None else GPUState(n, prec, 1, ctx)
    for op, mat in _bound(ops, counts, np.asarray(pars, dtype=float)):
        if mat is None:
            apply(st, op)
        else:
            qs, cs = _qubits(op)
            apply_matrix(st, mat, qs, cs)
    return st


def _pauli_arrays(terms):
    xs = np.ascontiguousarray([t[1] for t in terms], dtype=np.uint64)
    zs = np.ascontiguousarray([t[2] for t in terms], dtype=np.uint64)
    cs = np.ascontiguousarray([t[0] for t in terms], dtype=np.float64)
    return xs, zs, cs


def _expect_members(st, terms):
    """<H> of every member (FP64 sums of the Pauli strings)."""
    xs, zs, cs = _pauli_arrays(terms)
    out = np.empty(st.batch * len(terms))
    st.ctx.check(L.lib().bt_expect_pauli(st.h, len(terms), _ptr(xs), _ptr(zs), _ptr(cs), -1, _ptr(out)))
    return out.reshape(st.batch, len(terms)).sum(axis=1)


def _ctrl(mat):
    d = mat.shape[0]
    M = np.eye(2 * d, dtype=np.complex128)
    M[d:, d:] = mat
    return M


def losses(ops, n, param_list, terms, prec="c128", ctx=None, executor="auto"):
    """<H> after the ansatz at each parameter vector of param_list, as one batch.
    executor: "program" (one CTA per evaluation, n <= 14 / 13), "plan" (fused
    passes, one evaluation after the other) or "auto"."""
    from . import trajectories as T
    ctx = ctx or Context.default()
    counts = arg_counts(ops)
    params = [np.asarray(p, dtype=float) for p in param_list]
    B = len(params)
    bound = [_bound(ops, counts, p) for p in params]
    fits = n <= T.SHARED_MAX_N[prec]
    if executor == "program" or (executor == "auto" and fits):
        prog = T.Program(n, B, prec, ctx)
        for i, op in enumerate(ops):
            qs, cs = _qubits(op)
            if op.q > 2 or len(qs) + len(cs) > 2:
                raise ValueError("programs take ops on at most two qubits (control included)")
            if counts[i]:
                mats = [bound[m][i][1] for m in range(B)]
            else:
                mats = op.mat
            if cs:
                mats = [_ctrl(m) for m in mats] if isinstance(mats, list) else _ctrl(np.asarray(mats))
                qs = cs + qs
            prog.add_gate(mats, qs)
        st = GPUState(n, prec, B, ctx)
        prog.run(st, records=False)
        vals = _expect_members(st, terms)
        st.free()
        return vals
    plan = Plan(n, "sv", prec, ctx)
    pidx = []
    for i, (op, mat) in enumerate(bound[0]):
        if mat is None:
            plan.add(op)
        else:
            qs, cs = _qubits(op)
            plan.add_matrix(mat, qs, cs)
            pidx.append(i)
    plan.set_variable(pidx).compile(True)  # angles are rewritten in place: no recompiles
    st = GPUState(n, prec, 1, ctx)
    vals = np.empty(B)
    for m in range(B):
        if m:
            plan.set_matrices([(i, bound[m][i][1]) for i in pidx])
        st.set_zero()
        plan.run(st)
        vals[m] = _expect_members(st, terms)[0]
    st.free()
    return vals


def loss(pars, ops, n, terms, prec="c128", ctx=None):
    return float(losses(ops, n, [pars], terms, prec, ctx)[0])


# HBM for the members of one batched plan run of parameter-shift evaluations
_MEMBER_BUDGET = 16 << 30


def paramshift_member_mats(base, var, shifted, owner, evals):
    """The matrices of the variable ops `var` (indices into base) for each
    evaluation in evals: evaluation 0 is the unshifted circuit, 2i + 1 and 2i + 2
    shift parameter i (of op owner[i]) by +/- the shift."""
    out = []
    for e in evals:
        mats = {j: base[j][1] for j in var}
        if e > 0:
            i = (e - 1) // 2
            mats[owner[i]] = shifted[i][(e - 1) % 2]
        out.append([mats[j] for j in var])
    return out


def loss_and_grad_paramshift(p, ops, n, terms, prec="c128", ctx=None, executor="auto"):
    """(l, g) of loss_and_grad_paramshift (src/vqa.jl:590-611): the loss at p and,
    for every parameter i, (l(p + pi/2 e_i) - l(p - pi/2 e_i)) / 2; all 2P + 1
    evaluations in one batch.  Evaluation 0 is at p, 2i+1 and 2i+2 at p -+ shift of
    parameter i: every op keeps its matrix at p except in the two evaluations that
    shift one of its parameters, so each op's matrix is evaluated once at p and
    twice per parameter it owns."""
    from . import trajectories as T
    ctx = ctx or Context.default()
    p = np.asarray(p, dtype=float)
    P = len(p)
    counts = arg_counts(ops)
    if sum(counts) != P:
        raise ValueError(f"the ansatz takes {sum(counts)} parameters, {P} given")
    base = _bound(ops, counts, p)
    owner, first = [], []  # op owning each parameter; each op's first parameter
    c = 0
    for i, k in enumerate(counts):
        first.append(c)
        owner += [i] * k
        c += k
    shifted = []  # per parameter: (matrix at p + shift, matrix at p - shift)
    for i in range(P):
        op = ops[owner[i]]
        f0, k = first[owner[i]], counts[owner[i]]
        pair = []
        for s in (SHIFT, -SHIFT):
            q = p[f0:f0 + k].copy()
            q[i - f0] += s
            pair.append(np.asarray(op.mat(*q), dtype=np.complex128))
        shifted.append(pair)
    B = 2 * P + 1
    fits = n <= T.SHARED_MAX_N[prec]
    if executor == "program" or (executor == "auto" and fits):
        prog = T.Program(n, B, prec, ctx)
        for j, (op, mat) in enumerate(base):
            qs, cs = _qubits(op)
            if op.q > 2 or len(qs) + len(cs) > 2:
                raise ValueError("programs take ops on at most two qubits (control included)")
            m0 = op.mat if mat is None else mat
            if counts[j]:
                stack = np.broadcast_to(m0, (B,) + m0.shape).copy()
                for i in range(first[j], first[j] + counts[j]):
                    stack[2 * i + 1], stack[2 * i + 2] = shifted[i]
                if cs:
                    stack = np.stack([_ctrl(m) for m in stack])
                prog.add_gate(stack, cs + qs)
            else:
                prog.add_gate(_ctrl(np.asarray(m0)) if cs else m0, cs + qs)
        st = GPUState(n, prec, B, ctx)
        prog.run(st, records=False)
        vals = _expect_members(st, terms)
        st.free()
    else:
        plan = Plan(n, "sv", prec, ctx)
        var = []
        for i, (op, mat) in enumerate(base):
            if mat is None:
                plan.add(op)
            else:
                qs, cs = _qubits(op)
                plan.add_matrix(mat, qs, cs)
                var.append(i)
        plan.set_variable(var).compile(True)  # shifted angles are rewritten in place: no recompiles
        if os.environ.get("BTGPU_VQA_PLAN_MEMBERS") == "1":
            # the evaluations as members of batched runs, each with its own matrices
            vals = np.empty(B)
            es = 8 if prec in ("c64", "complex64") else 16
            chunk = max(1, min(B, _MEMBER_BUDGET // ((2 ** n) * es)))
            for e0 in range(0, B, chunk):
                evals = list(range(e0, min(B, e0 + chunk)))
                st = GPUState(n, prec, len(evals), ctx)
                plan.run_members(st, var, paramshift_member_mats(base, var, shifted, owner, evals))
                vals[e0:e0 + len(evals)] = _expect_members(st, terms)
                st.free()
        else:
            st = GPUState(n, prec, 1, ctx)
            vals = np.empty(B)

            def run(m):
                st.set_zero()
                plan.run(st)
                vals[m] = _expect_members(st, terms)[0]

            run(0)
            for i in range(P):
                j = owner[i]
                plan.set_matrices([(j, shifted[i][0])])
                run(2 * i + 1)
                plan.set_matrices([(j, shifted[i][1])])
                run(2 * i + 2)
                plan.set_matrices([(j, base[j][1])])
            st.free()
    g = 0.5 * (vals[1::2] - vals[2::2])
    return float(vals[0]), g
