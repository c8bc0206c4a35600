"""Op descriptors with the reference's fields and constructor rules.

Mirrors Op (BlueTangle.jl src/struct.jl:365-453), OpQC (src/struct.jl:182-249)
and ifOp (src/struct.jl:666-696): `q`, `name`, `qubit`, `target_qubit`
(-1 for one-qubit ops), `control` (-2 = none), `mat`, `noisy` and `type`
("op", "phase", "🔬" for measurements, "f" for parametrised gates).  The engine
consumes these fields; it never re-derives matrix values.
"""
import numpy as np

from .gates import clean_name, gates, gates_with_phase, is_measurement
from .noise import is_valid_quantum_channel, noise_model1, noise_model2

__all__ = ["Op", "OpQC", "ifOp", "QuantumOps"]


class QuantumOps:
    pass


def _num_qubits(qubit, target, control):
    """_get_op_num_qubits (src/struct.jl:455-474)."""
    if target == -1:
        if qubit == control:
            raise ValueError("`qubit` must differ from `control` qubit")
        return 1
    if qubit == target:
        raise ValueError("`qubit` and `target_qubit` must differ")
    if qubit == control and target == control:
        raise ValueError("either `qubit` or `target_qubit` must differ from `control` qubit")
    return 2


class Op(QuantumOps):
    """Op(name, qubit[, target_qubit]; control, noisy) or Op(name, mat_or_f, qubit[, target])."""

    def __new__(cls, name, *args, **kw):
        # Op("RES", q) is an OpQC (src/struct.jl:419-427); Op("CCX", q, c, t) is a
        # controlled two-qubit Op (src/struct.jl:436-449)
        if isinstance(name, str) and len(args) == 1 and not kw and name.upper() in ("RES", "RESET"):
            return OpQC.reset(args[0])
        if isinstance(name, str) and len(args) == 3 and all(isinstance(a, int) for a in args):
            base = {"CCZ": "CZ", "CCX": "CX", "CCY": "CY", "CSWAP": "SWAP"}.get(name)
            if base is None:
                raise ValueError("Unsupported three-qubit operation")
            return Op(base, args[0], args[2], control=args[1])
        return super().__new__(cls)

    def __init__(self, name, *args, control=-2, noisy=True, type=None):
        if isinstance(name, str) and len(args) == 3 and all(isinstance(a, int) for a in args):
            return  # built by __new__
        if isinstance(name, (list, tuple)):  # Op([name, angle], ...) (src/struct.jl:550-551)
            name = f"{name[0]}({name[1]})"
        mat = None
        if args and (callable(args[0]) or isinstance(args[0], np.ndarray)):
            mat, args = args[0], args[1:]
        qubit = int(args[0])
        target = int(args[1]) if len(args) > 1 else -1
        if mat is None:
            mat = gates(name)
        self.name = name
        self.qubit = qubit
        self.target_qubit = target
        self.control = int(control)
        self.q = _num_qubits(qubit, target, self.control)
        if callable(mat) and not isinstance(mat, np.ndarray):
            if type is not None:
                raise ValueError("setting `type` for gates constructed from functions is not supported")
            self.mat = mat
            self.type = "f"
            self.noisy = noisy
            return
        mat = np.asarray(mat, dtype=np.complex128)
        if mat.shape != (2 ** self.q, 2 ** self.q):
            raise ValueError(f"size of matrix {mat.shape} not compatible with {self.q}-qubit operation")
        self.mat = mat
        if self.q == 1 and is_measurement(name):
            if self.control != -2:
                raise ValueError("measurement and control operations are incompatible.")
            self.type = "🔬"
            self.noisy = False
        else:
            self.type = "phase" if clean_name(name) in gates_with_phase else "op"
            self.noisy = noisy

    def __repr__(self):
        t = f",{self.target_qubit}" if self.q == 2 else ""
        c = f";control={self.control}" if self.control != -2 else ""
        return f"Op({self.name!r},{self.qubit}{t}{c})"


class OpQC(QuantumOps):
    """OpQC(name, kraus, qubit, target=-1) or OpQC(model, p, qubit, target=-1)."""

    def __init__(self, name, kraus_or_p, qubit, target_qubit=-1, type=""):
        if isinstance(kraus_or_p, (int, float)):
            p = float(kraus_or_p)
            q = 2 if target_qubit > 0 else 1
            kraus = noise_model1(name, p) if q == 1 else noise_model2(name, p)
            type = f"{p}"
        else:
            kraus = [np.asarray(K, dtype=np.complex128) for K in kraus_or_p]
        if not is_valid_quantum_channel(kraus):
            raise ValueError("not valid kraus operators: not CPTP!")
        q = int(round(np.log2(kraus[0].shape[0])))
        if q == 1 and target_qubit > 0:
            raise ValueError("for 1-qubit quantum channel, target_qubit should be -1")
        if q == 2 and target_qubit < 0:
            raise ValueError("for 2-qubit quantum channel, you must select the target_qubit")
        if q > 3:
            raise ValueError("Noise models are available only for up to 3 qubits!")
        self.q = q
        self.name = name.lower()
        self.qubit = int(qubit)
        self.target_qubit = int(target_qubit) if q != 3 else -1
        self.control = -2
        self.kraus = kraus
        self.noisy = False
        self.type = type

    @staticmethod
    def reset(qubit):
        """RES: amplitude damping with gamma = 1 (src/struct.jl:421-423)."""
        return OpQC("RES", [np.array([[1.0, 0.0], [0.0, 0.0]]), np.array([[0.0, 1.0], [0.0, 0.0]])], qubit)

    def __repr__(self):
        t = f",{self.target_qubit}" if self.q == 2 else ""
        return f"OpQC({self.name!r},{self.qubit}{t})"


class ifOp(QuantumOps):
    """Mid-circuit measurement with classically controlled op lists (src/struct.jl:666-696)."""

    def __init__(self, name, qubit, if0="I", if1="I"):
        if not is_measurement(name):
            raise ValueError("select MX or MY or MZ or MR basis.")
        self.q = 1
        self.name = name
        self.qubit = int(qubit)
        self.target_qubit = -1
        self.control = -2
        self.mat = gates(name)
        self.noisy = False
        self.type = "🔬"

        def lst(x):
            if isinstance(x, str):
                return [Op(x, qubit)]
            if isinstance(x, Op):
                return [x]
            return list(x)
        self.if01 = (lst(if0), lst(if1))

    def __repr__(self):
        return f"ifOp({self.name!r},{self.qubit})"
