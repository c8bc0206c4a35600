"""Host execution of the generated fused-pass kernels (test infrastructure).

The plan compiler writes the CUDA source it generates for every fused pass
(BTGPU_JIT_DUMP).  That source is straight-line C++ apart from a few CUDA names,
so it is translated textually (thread and block indices, shared memory, barriers,
the FP32 two-lane helpers as per-lane host arithmetic), built with g++, and each
CTA is run on the host with one thread per CUDA thread and a barrier for
__syncthreads.  The outputs are compared with the oracle: this checks the code the
generator writes (direct and staged phases, shared-memory addressing, every op
emitter, scalar and two-lane forms) without a GPU.  The generated code must hold
no inline PTX, so the L2 and shared-memory prefetches are turned off
(BTGPU_JIT_L2PF=0, BTGPU_JIT_PREFETCH=0) in the process that plans, and
BTGPU_JIT_DUMP_ONLY skips building the kernels for the device.
"""
import ctypes
import os
import re
import subprocess

import numpy as np

HOST_HEADER = r"""
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
struct Dim { unsigned x = 0, y = 0, z = 0; };
static thread_local Dim threadIdx, blockIdx;
static Dim gridDim, blockDim;
static std::barrier<>* g_bar = nullptr;
alignas(16) static unsigned char g_smem[1 << 18];
#define __global__
#define __device__
#define __forceinline__ inline
#define __launch_bounds__(a, b)
#define __restrict__ __restrict
#define __align__(n) alignas(n)
#define __syncthreads() g_bar->arrive_and_wait()
static inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
static inline float __double2float_rn(double d) { return (float)d; }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
"""

LAUNCH = r"""
template <typename F>
static void grid_run(F body, int grid, int threads) {
  gridDim.x = grid;
  blockDim.x = threads;
  for (int b = 0; b < grid; ++b) {
    std::barrier<> bar(threads);
    g_bar = &bar;
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t)
      ts.emplace_back([&, t, b] {
        threadIdx.x = t;
        blockIdx.x = b;
        body();
      });
    for (auto& th : ts) th.join();
  }
}
template <typename T2, typename A>
static void launch(void (*k)(T2*, const A), void* psi, const void* args, int grid, int threads) {
  grid_run([&] { k((T2*)psi, *(const A*)args); }, grid, threads);
}
// kernels reading per-member entries: row m of mm for member m
template <typename T2, typename A, typename R>
static void launch_pm(void (*k)(T2*, const A, const R*, const i64), void* psi, const void* args, const void* mm,
                      long long mstride, int grid, int threads) {
  grid_run([&] { k((T2*)psi, *(const A*)args, (const R*)mm, (i64)mstride); }, grid, threads);
}
"""


def translate(src):
    """The generated CUDA source as host C++; returns (code, [(name, M, threads)])."""
    if re.search(r"\basm\s*(volatile)?\s*\(\s*\"(cp\.|prefetch)", src):
        raise ValueError("generated kernels hold copy/prefetch PTX: plan with BTGPU_JIT_L2PF=0 BTGPU_JIT_PREFETCH=0")
    kernels = [(f"pass_{m.group(1)}", int(m.group(2)), int(m.group(3)))
               for m in re.finditer(r"// pass (\d+): M=(\d+) threads=(\d+)", src)]
    code = src.replace("extern __shared__ __align__(16) unsigned char smem_raw[];",
                       "unsigned char* smem_raw = g_smem;")
    # the two-lane helpers: one FP32 operation per lane, rounded as the PTX forms are
    code = re.sub(r"__device__ __forceinline__ u64 ffma2\(.*\n",
                  "static inline u64 ffma2(u64 a, u64 b, u64 c) { return pk(std::fmaf(plo(a), plo(b), plo(c)), "
                  "std::fmaf(phi(a), phi(b), phi(c))); }\n", code)
    code = re.sub(r"__device__ __forceinline__ u64 fmul2\(.*\n",
                  "static inline u64 fmul2(u64 a, u64 b) { return pk(plo(a) * plo(b), phi(a) * phi(b)); }\n", code)
    if "asm" in code:
        raise ValueError("inline PTX left in the generated source")
    return HOST_HEADER + code + LAUNCH, kernels


def build(src, workdir, c64, permem=False):
    """Host library of the generated kernels with run_pass(i, psi, args, grid,
    threads), or with permem run_pass(i, psi, args, mm, mstride, grid, threads)."""
    code, kernels = translate(src)
    T2, A, R = ("cf", "JitArgsF<4096>", "float") if c64 else ("cd", "JitArgsD<2048>", "double")
    if permem:
        code += ('extern "C" int run_pass(int i, void* psi, const void* args, const void* mm, long long mstride, '
                 'int grid, int threads) {\n  switch (i) {\n')
        for name, _, _ in kernels:
            code += (f"    case {int(name[5:])}: launch_pm<{T2}, {A}, {R}>({name}, psi, args, mm, mstride, grid, "
                     "threads); return 0;\n")
    else:
        code += 'extern "C" int run_pass(int i, void* psi, const void* args, int grid, int threads) {\n  switch (i) {\n'
        for name, _, _ in kernels:
            code += f"    case {int(name[5:])}: launch<{T2}, {A}>({name}, psi, args, grid, threads); return 0;\n"
    code += "  }\n  return -1;\n}\n"
    tag = "pm" if permem else "k"
    cpp = os.path.join(workdir, f"kernels_{tag}.cpp")
    so = os.path.join(workdir, f"kernels_{tag}.so")
    with open(cpp, "w") as f:
        f.write(code)
    subprocess.run(["g++", "-std=c++20", "-O0", "-shared", "-fPIC", "-pthread", "-w", "-o", so, cpp], check=True)
    lib = ctypes.CDLL(so)
    lib.run_pass.restype = ctypes.c_int
    lib.run_pass.argtypes = ([ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                              ctypes.c_int, ctypes.c_int] if permem else
                             [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int])
    return lib, kernels


def _ff_slots(mats, nreals):
    """Each coefficient as the floats (h, l) packed in its double slot, as the
    library's launcher passes them to float-float complex128 kernels."""
    m = np.asarray(mats[:nreals], dtype=np.float64)
    packed = np.empty(2 * nreals, dtype=np.float32)
    packed[0::2] = m.astype(np.float32)
    packed[1::2] = (m - packed[0::2].astype(np.float64)).astype(np.float32)
    return packed.view(np.float64)


def run_members(plan, psis, src, src_pm, workdir, indices, member_mats):
    """Member m of psis (a (members, 2^n) array) under the plan with member_mats[m]
    for the gates of these add indices, as bt_plan_run_members runs it: passes
    without those gates by their kernels (src), the others by their per-member
    kernels (src_pm, built by bt_plan_prepare_members) reading the member table."""
    import plan_emulator as E
    from bluetangle_gpu import _lib as L
    from bluetangle_gpu.engine import _cm
    c64 = plan.prec in ("c64", "complex64")
    lib, kernels = build(src, workdir, c64)
    lpm, kpm = build(src_pm, workdir, c64, permem=True)
    R = ctypes.c_float if c64 else ctypes.c_double
    nreals = 4096 if c64 else 2048

    class Args(ctypes.Structure):
        _fields_ = [("member_lo", ctypes.c_int64), ("nmem", ctypes.c_int64), ("nbits", ctypes.c_int),
                    ("lg_tiles", ctypes.c_int), ("mat", R * nreals)]

    B = len(member_mats)
    idx = np.ascontiguousarray(list(indices), dtype=np.int64)
    buf = np.ascontiguousarray(np.concatenate([_cm(m).ravel() for mm in member_mats for m in mm]))
    x = np.asarray(psis, dtype=np.complex128).reshape(B, -1)
    nbits = int(x.shape[1]).bit_length() - 1
    state = x.ravel().astype(np.complex64 if c64 else np.complex128)
    P = ctypes.c_void_p
    fused = pm = 0
    for i, (kind, ops, mats) in enumerate(E.passes(plan)):
        if kind:
            y = state.astype(np.complex128).reshape(B, -1)
            for m in range(B):
                E._sweep(y[m], nbits, ops, mats)
            state = y.ravel().astype(state.dtype)
            continue
        used = ctypes.c_int()
        table = np.zeros(B * nreals, dtype=np.float64)
        rc = L.lib().bt_plan_member_table(plan.h, i, B, len(idx), idx.ctypes.data_as(P), buf.ctypes.data_as(P),
                                          table.ctypes.data_as(P), table.size, ctypes.byref(used))
        L.check(rc)
        a = Args()
        name, M, threads = kernels[fused]
        a.member_lo, a.nmem, a.nbits, a.lg_tiles = 0, B, nbits, nbits - M
        vals = _ff_slots(mats, nreals) if (not c64 and nbits >= 16 and os.environ.get("BTGPU_JIT_FF", "1") != "0") else mats
        for e in range(nreals):
            a.mat[e] = vals[e]
        grid = min(B << (nbits - M), 3)
        rows = table[:B * used.value].reshape(B, used.value)
        # a pass without member-dependent gates has equal rows (members here differ in
        # every such gate's matrix); the count of per-member kernels is checked below
        if np.all(rows == rows[0]):
            assert lib.run_pass(fused, state.ctypes.data_as(P), ctypes.byref(a), grid, threads) == 0
        else:
            tab = np.ascontiguousarray(rows.astype(np.float32 if c64 else np.float64))
            assert lpm.run_pass(pm, state.ctypes.data_as(P), ctypes.byref(a), tab.ctypes.data_as(P), used.value,
                                grid, threads) == 0
            pm += 1
        fused += 1
    assert pm == len(kpm), (pm, len(kpm))
    return state.astype(np.complex128).reshape(B, -1)


def run(plan, psi, dump_src, workdir, members=1):
    """The compiled plan applied to psi by its generated kernels run on the host
    (sweep passes by the numpy emulation).  members > 1: psi holds that many
    states back to back, run as the members of one batch."""
    import plan_emulator as E
    c64 = plan.prec in ("c64", "complex64")
    lib, kernels = build(dump_src, workdir, c64)
    R = ctypes.c_float if c64 else ctypes.c_double
    nreals = 4096 if c64 else 2048

    class Args(ctypes.Structure):
        _fields_ = [("member_lo", ctypes.c_int64), ("nmem", ctypes.c_int64), ("nbits", ctypes.c_int),
                    ("lg_tiles", ctypes.c_int), ("mat", R * nreals)]

    x = np.asarray(psi, dtype=np.complex128).ravel(order="F").copy()
    nbits = int(x.size // members).bit_length() - 1
    state = x.astype(np.complex64 if c64 else np.complex128)
    # float-float complex128 kernels read each coefficient as the floats (h, l)
    # packed in its slot, as the library's launcher writes them
    ffm = not c64 and nbits >= 16 and os.environ.get("BTGPU_JIT_FF", "1") != "0"
    fused = 0
    for kind, ops, mats in E.passes(plan):
        if kind:
            y = state.astype(np.complex128).reshape(members, -1)
            for m in range(members):
                E._sweep(y[m], nbits, ops, mats)
            state = y.ravel().astype(state.dtype)
            continue
        name, M, threads = kernels[fused]
        assert name == f"pass_{fused}"
        a = Args()
        a.member_lo, a.nmem, a.nbits, a.lg_tiles = 0, members, nbits, nbits - M
        vals = _ff_slots(mats, nreals) if ffm else mats
        for e in range(nreals):
            a.mat[e] = vals[e]
        grid = min(members << (nbits - M), 3)  # fewer CTAs than tiles: each loops over several
        rc = lib.run_pass(fused, state.ctypes.data_as(ctypes.c_void_p), ctypes.byref(a), grid, threads)
        assert rc == 0
        fused += 1
    return state.astype(np.complex128)
