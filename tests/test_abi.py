"""The C-ABI library loads and exports every symbol include/btgpu.h declares.

No compute calls: these run without a GPU.
"""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "btgpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bt_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_surface():
    syms = declared_symbols()
    for s in ("bt_ctx_create", "bt_state_alloc", "bt_apply_matrix", "bt_apply_kraus", "bt_measure_z",
              "bt_sample", "bt_expect_pauli", "bt_reduced_dm"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import bluetangle_gpu._lib as L
    lib = ctypes.CDLL(L.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes binding covers the same surface
    assert sorted(L.SIGNATURES) == declared_symbols()


def test_version_and_status_strings():
    import bluetangle_gpu._lib as L
    lib = L.lib()
    assert lib.bt_abi_version() == 1
    assert b"CPTP" in lib.bt_status_string(L.BT_ERR_NOT_CPTP)
    assert lib.bt_status_string(0) == b"ok"


def test_null_arguments_are_errors_not_crashes():
    import bluetangle_gpu._lib as L
    lib = L.lib()
    assert lib.bt_ctx_create(0, 0, None) == L.BT_ERR_BAD_ARG
    assert lib.bt_state_free(None) == 0
    assert lib.bt_apply_matrix(None, 1, None, None, 0, None, -1) == L.BT_ERR_BAD_ARG
    assert lib.bt_last_error(None)


def _prototypes():
    """name -> (return type, [parameter types]) of every function in the header."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    pat = r"^\s*((?:const\s+)?(?:int|int64_t|uint64_t|double|char\s*\*|void))\s*(bt_\w+)\s*\(([^;]*?)\)\s*;"
    for m in re.finditer(pat, src, flags=re.M | re.S):
        params = " ".join(m.group(3).split())
        types = [] if params in ("", "void") else [re.sub(r"\s*\b\w+$", "", p.strip()) for p in params.split(",")]
        out[m.group(2)] = (" ".join(m.group(1).split()), types)
    return out


def _split_top(s):
    """Comma-separated items at brace depth 0."""
    items, depth, cur = [], 0, ""
    for ch in s:
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
        if ch == "," and depth == 0:
            items.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        items.append(cur.strip())
    return items


_SCALAR = {"int": {"Cint", "Int32"}, "int64_t": {"Int64"}, "uint64_t": {"UInt64"}, "double": {"Float64", "Cdouble"}}
_POINTEE = {"double": {"Float64", "ComplexF64", "Cdouble"}, "int32_t": {"Int32", "Cint"}, "int": {"Cint", "Int32"},
            "int64_t": {"Int64"}, "uint64_t": {"UInt64"}, "uint8_t": {"UInt8"}}


def _compatible(ctype, jtype):
    c = ctype.replace("const", "").strip()
    if "*" not in c:
        return jtype in _SCALAR.get(c, set())
    m = re.fullmatch(r"(Ptr|Ref)\{(.+)\}", jtype)
    if not m:
        return False
    inner, base, stars = m.group(2), c.replace("*", "").strip(), c.count("*")
    if stars == 2 or base.startswith("bt_") and stars == 2:
        return inner == "Ptr{Cvoid}"
    if base.startswith("bt_") or base == "void":
        return inner == "Cvoid"
    return inner in _POINTEE.get(base, set())


def test_julia_binding_ccalls_match_the_header():
    """julia/BlueTangleGPU.jl binds the library with ccall: every call names a
    declared function with its parameter count and, per parameter, a Julia type
    of the C type's size and kind (scalars by width, pointers as Ptr/Ref of a
    matching element type, handles as Ptr{Cvoid})."""
    jl = open(os.path.join(ROOT, "julia", "BlueTangleGPU.jl")).read()
    protos = _prototypes()
    assert len(protos) >= 60
    calls = re.findall(r"ccall\(\(:(\w+),\s*lib\),\s*(\w+),\s*\(([^()]*)\)", jl)
    assert len(calls) >= 40
    seen = set()
    for name, ret, args in calls:
        assert name in protos, f"{name} is not declared in btgpu.h"
        cret, ctypes_ = protos[name]
        assert (ret == "Cstring") == cret.endswith("*"), (name, ret, cret)
        if ret != "Cstring":
            assert ret == "Cint" and cret == "int", (name, ret, cret)
        jtypes = _split_top(args)
        assert len(jtypes) == len(ctypes_), (name, jtypes, ctypes_)
        for ct, jt in zip(ctypes_, jtypes):
            assert _compatible(ct, jt), (name, ct, jt)
        seen.add(name)
    # the generics of the drop-in and the entry points they stand on are bound
    for need in ("bt_apply_matrix", "bt_apply_kraus", "bt_measure_z", "bt_measure_z2", "bt_state_copy",
                 "bt_sample", "bt_probabilities", "bt_expect_pauli", "bt_expect_z_all", "bt_fidelity",
                 "bt_fidelity_dm", "bt_plan_run", "bt_program_run", "bt_sample_members", "bt_serve_submit"):
        assert need in seen, need
    # apply is functional (a copy, then the in-place form) as the reference's
    assert re.search(r"apply\(s::GPUHandle, op::[^)]*\)\s*=\s*apply!\(copy\(s\)", jl)
    # OpQC("RES") resets (src/hilbert.jl:489-490); controls enter programs as 4x4
    assert re.search(r'uppercase\(op\.name\) in \("RES", "RESET"\)[^\n]*\n\s*_reset_Z!', jl)
    assert "_program_gate!(p, _ctrl_matrix(op.mat), [op.control, op.qubit])" in jl


def _julia_code(src):
    """The Julia source with strings, docstrings and comments blanked."""
    out, i, n = [], 0, len(src)
    while i < n:
        if src.startswith('"""', i):
            i = src.index('"""', i + 3) + 3
            out.append('""')
        elif src[i] == '"':
            j = i + 1
            while src[j] != '"':
                j += 2 if src[j] == "\\" else 1
            out.append('""')
            i = j + 1
        elif src[i] == "#":
            j = src.find("\n", i)
            i = n if j < 0 else j
        else:
            out.append(src[i])
            i += 1
    return "".join(out)


def _julia_blocks(src):
    """(block openers, `end`s) of the Julia source outside brackets (where `end`
    indexes and `for`/`if` are comprehension clauses); brackets must pair."""
    code = _julia_code(src)
    flat, stack = [], []
    pairs = {")": "(", "]": "[", "}": "{"}
    for ch in code:
        if ch in "([{":
            stack.append(ch)
        elif ch in ")]}":
            assert stack and stack[-1] == pairs[ch], f"unpaired {ch}"
            stack.pop()
        elif not stack:
            flat.append(ch)
    assert not stack, f"unclosed {stack}"
    flat = "".join(flat)
    opens = len(re.findall(r"\b(function|if|for|while|let|begin|do|struct|try|module|quote|macro)\b", flat))
    opens += len(re.findall(r"\b(abstract|primitive)\s+type\b", flat))
    return opens, len(re.findall(r"\bend\b", flat))


def test_julia_binding_is_well_formed():
    """Julia is not installed here: the binding's brackets pair, every block
    opener has its `end` (a dropped `end` is caught), and every exported name is
    defined in the file."""
    jl = open(os.path.join(ROOT, "julia", "BlueTangleGPU.jl")).read()
    opens, ends = _julia_blocks(jl)
    assert opens == ends, (opens, ends)
    k = jl.rindex("\nend")
    o2, e2 = _julia_blocks(jl[:k] + jl[k + 4:])
    assert o2 == e2 + 1
    code = _julia_code(jl)
    exported = set()
    for m in re.finditer(r"^export\b", code, flags=re.M):
        j, stmt = m.end(), ""
        while True:  # an export continues on the next line after a trailing comma
            k = code.find("\n", j)
            stmt += code[j:k] + " "
            j = k + 1
            if not code[:k].rstrip().endswith(","):
                break
        exported |= {x.strip() for x in stmt.split(",") if x.strip()}
    assert len(exported) >= 45 and "gpu_random_state" in exported
    for name in exported:
        nm = re.escape(name) + r"(?![\w!])"
        pat = rf"(function\s+{nm}|^{nm}\(.*\)\s*(where.*)?=|struct\s+{nm}|^const\s+{nm})"
        assert re.search(pat, code, flags=re.M), f"{name} is exported but not defined"
    # every private helper called (not the reference's BlueTangle._x) is defined here
    calls = set(re.findall(r"(?<![\w.!])(_[A-Za-z]\w*!?)\(", code))
    defined = set(re.findall(r"(?:function\s+|^\s*)(_[A-Za-z]\w*!?)\(", code, flags=re.M))
    assert calls <= defined, sorted(calls - defined)
