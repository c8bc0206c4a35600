// Plan specialisation: each distinct fused-pass structure (tile bits, register
// sets of its phases, op types and register bits) becomes its own kernel with the
// whole op sequence as straight-line scalar code, compiled at plan-compile time
// with NVRTC for sm_103a.  Register indices, swaps and shared-memory offsets are
// then compile-time constants and no register is shuffled between ops (in the
// generic k_fused the runtime op switch costs several register moves per
// amplitude per gate).  Matrix entries stay in the kernel parameters at fixed
// offsets (or, for a batch whose members carry their own matrices, in one table
// row per member), so passes that differ only in angles share one kernel.  The
// first and last register phases move amplitudes straight between HBM and
// registers where coalesced, and each CTA asks L2 for its next tile ahead.
//
// The generator emits already-expanded code (no templates or loops for the
// compiler to unroll), kernels are compiled in parallel batches, and cubins are
// cached on disk by a hash of their source.  NVRTC is loaded with dlopen: without
// it plans run on the generic k_fused kernel.
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <functional>
#include <array>
#include <atomic>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "bt_fused.cuh"
#include "bt_jit.cuh"

// ------------------------------------------------------------------ NVRTC by dlopen
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram* nvrtcProgram_t;
struct Nvrtc {
  bool ok = false;
  nvrtcResult_t (*create)(nvrtcProgram_t*, const char*, const char*, int, const char* const*, const char* const*);
  nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char* const*);
  nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t*);
  nvrtcResult_t (*cubin)(nvrtcProgram_t, char*);
  nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t*);
  nvrtcResult_t (*log)(nvrtcProgram_t, char*);
  nvrtcResult_t (*destroy)(nvrtcProgram_t*);
  nvrtcResult_t (*version)(int*, int*) = nullptr;  // optional: part of the cubin cache key
};

static Nvrtc* nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libnvrtc.so", "libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"};
    void* h = nullptr;
    for (const char* nm : names)
      if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return;
    n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
    n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
    n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
    n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
    n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
    n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
    n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
    n.version = (decltype(n.version))dlsym(h, "nvrtcVersion");
    n.ok = n.create && n.compile && n.cubin_size && n.cubin && n.log_size && n.log && n.destroy;
  });
  return n.ok ? &n : nullptr;
}

bool bt_jit_available() { return nvrtc() != nullptr && getenv("BTGPU_NO_JIT") == nullptr; }

// Tuning knobs of the specialised passes (read once): resident CTAs per SM the
// kernels are compiled for (register budget 65536 / (threads * blocks)), and the
// most gates a specialised pass takes.
static int env_int(const char* name, int dflt, int lo, int hi) {
  const char* v = getenv(name);
  if (!v || !*v) return dflt;
  const int x = atoi(v);
  return x < lo ? lo : (x > hi ? hi : x);
}
int bt_jit_min_blocks() {
  static const int v = env_int("BTGPU_JIT_MINB", 2, 1, 4);
  return v;
}
int bt_jit_max_ops() {
  static const int v = env_int("BTGPU_PLAN_MAX_OPS", 96, 8, BT_FUSED_MAX_OPS);
  return v;
}
int bt_tile_rb(bool c64) {
  static const int v = env_int("BTGPU_TILE_RB", BT_TILE_RB_C64, 4, 6);
  return c64 ? v : BT_TILE_RB_C128;
}

// ------------------------------------------------------------------ generated source
static const char* kPrelude = R"PRELUDE(
typedef long long i64;
typedef unsigned long long u64;
struct __align__(8) cf { float x, y; };
struct __align__(16) cd { double x, y; };
struct __align__(16) f4 { float x, y, z, w; };
struct __align__(16) pu { u64 x, y; };  // a shared-memory pair unit of the pair-lane form
__device__ __forceinline__ float fm(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fm(double a, double b, double c) { return __fma_rn(a, b, c); }
template <int NM> struct JitArgsF { i64 member_lo, nmem; int nbits, lg_tiles; float mat[NM]; };
template <int NM> struct JitArgsD { i64 member_lo, nmem; int nbits, lg_tiles; double mat[NM]; };
// packed pairs of FP32 values (two amplitudes' real or imaginary parts) and the
// two-lane FMA / multiply of sm_100-family GPUs
// (pack / unpack as plain bit operations: register-pair moves the compiler can coalesce)
__device__ __forceinline__ u64 pk(float a, float b) { return (u64)__float_as_uint(a) | ((u64)__float_as_uint(b) << 32); }
__device__ __forceinline__ float plo(u64 r) { return __uint_as_float((unsigned)r); }
__device__ __forceinline__ float phi(u64 r) { return __uint_as_float((unsigned)(r >> 32)); }
__device__ __forceinline__ u64 ffma2(u64 a, u64 b, u64 c) { u64 d; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c)); return d; }
__device__ __forceinline__ u64 fmul2(u64 a, u64 b) { u64 d; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
__device__ __forceinline__ u64 bc(float a) { return pk(a, a); }
// float-float numbers (complex128 passes in FP32 arithmetic, BTGPU_JIT_FF): a
// value is h + l with |l| <= ulp(h) / 2, 48 significant bits; sums by TwoSum and
// products by FMA-exact TwoProduct (Dekker, Knuth; Joldes, Muller and Popescu's
// accurate double-word algorithms), each renormalised by FastTwoSum
struct ff {
  float h, l;
  __device__ __forceinline__ ff() {}
  __device__ __forceinline__ ff(float a, float b) : h(a), l(b) {}
  __device__ __forceinline__ ff(double d) {
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
  }
  __device__ __forceinline__ operator double() const { return (double)h + (double)l; }
};
struct __align__(16) ffc2 { ff x, y; };
__device__ __forceinline__ ff ff_fast(float s, float e) { const float t = s + e; return ff(t, e - (t - s)); }
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const float s = a.h + b.h, bb = s - a.h, e = (a.h - (s - bb)) + (b.h - bb);
  return ff_fast(s, e + (a.l + b.l));
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.h, -a.l); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = a.h * b.h;
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  return ff_fast(p, e);
}
__device__ __forceinline__ ff fm(ff a, ff b, ff c) { return a * b + c; }
// coefficients arrive split on the host: each double slot holds the floats (h, l)
__device__ __forceinline__ const ff* ffp(const double* p) { return reinterpret_cast<const ff*>(p); }
)PRELUDE";

static std::string fmt_u64(uint64_t v) {
  char b[32];
  snprintf(b, sizeof b, "%lluULL", (unsigned long long)v);
  return b;
}

static int swz_host(bool f, int l) { return f ? (l ^ ((l >> 4) & 15)) : (l ^ ((l >> 3) & 7)); }

// Complex-pair arithmetic (complex64, BTGPU_JIT_CPAIR=1; off by default): an op
// with real coefficients applies the same real map to the real and the imaginary
// part of its amplitudes, so (x_j, y_j) -- one amplitude, as it lies in memory and
// in registers after a 64-bit load -- goes through one two-lane FP32 instruction
// (fma.rn.f32x2 / mul.rn.f32x2) instead of two: the add/sub butterflies (H), the
// factored real rotations (RY) and real 2x2 matrices.  Ops with complex
// coefficients (phases, RX) mix the two parts and stay scalar.  Measured on the
// 28- and 33-qubit brickwork: 8.5% fewer instructions, FMA pipe busier by as
// much, pass times unchanged (the passes are bound by neither issue nor FMA).
// complex128 fused passes in float-float arithmetic (on unless BTGPU_JIT_FF=0):
// GB300 issues FP64 at a small share of its FP32 rate, so the passes' complex128
// arithmetic runs as float-float on the FP32 pipe (48-bit significands: relative
// error ~2^-48 per operation, far inside the 1e-12 the complex128 results are held
// to); the tile keeps float-float pairs (16 bytes per amplitude, as a complex128
// value), HBM keeps complex128, and coefficients are split on the host.  32-qubit
// brickwork of depth 30: 12.17 -> 5.99 s per circuit on a GB300.
bool bt_jit_ff_on() {
  static const bool v = env_int("BTGPU_JIT_FF", 1, 0, 1) != 0;
  return v;
}

// a pass in float-float form: complex128, not a per-member kernel, and on a state
// of at least 2^16 entries (smaller ones are latency-bound, where the longer
// float-float chains cost more than the FP64 issue rate: 12-qubit plans ran 5%
// slower in it)
template <typename R>
static bool ff_pass(const FusedArgs<R>& a) {
  return sizeof(R) == 8 && !a.permem && a.nbits >= 16 && bt_jit_ff_on();
}

static bool cpair_on() {
  static const bool v = env_int("BTGPU_JIT_CPAIR", 0, 0, 1) != 0;
  return v;
}

// emits one op on the scalar registers x<j> (real) / y<j> (imaginary), j < 2^NB
// mref: where the op's entries are read (the kernel parameters, or a per-member table)
// cp: complex-pair form of the real-coefficient ops (complex64 only)
static void emit_op(std::ostringstream& o, const FOp& op, int NB, const char* mref = "a.mat", bool cp = false) {
  const int D = 1 << NB;
  auto M = [&](int e) {
    std::ostringstream s;
    s << mref << "[" << (op.moff + e) << "]";
    return s.str();
  };
  auto pairs = [&](int B, auto&& body) {
    for (int j = 0; j < D; ++j)
      if (!(j & (1 << B))) body(j, j | (1 << B));
  };
  auto quads = [&](int B0, int B1, auto&& body) {
    for (int j = 0; j < D; ++j)
      if (!(j & ((1 << B0) | (1 << B1)))) {
        const int q[4] = {j, j | (1 << B1), j | (1 << B0), j | (1 << B0) | (1 << B1)};
        body(q);
      }
  };
  const int b0 = op.b0, b1 = op.b1;
  switch (op.type) {
    case FOP_G1:
      o << "    { const R m0=" << M(0) << ",m1=" << M(1) << ",m2=" << M(2) << ",m3=" << M(3) << ",m4=" << M(4)
        << ",m5=" << M(5) << ",m6=" << M(6) << ",m7=" << M(7) << ";\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << ";"
          << " x" << j << "=fm(m0,ar,fm(-m1,ai,fm(m2,br,-m3*bi)));"
          << " y" << j << "=fm(m0,ai,fm(m1,ar,fm(m2,bi,m3*br)));"
          << " x" << k << "=fm(m4,ar,fm(-m5,ai,fm(m6,br,-m7*bi)));"
          << " y" << k << "=fm(m4,ai,fm(m5,ar,fm(m6,bi,m7*br))); }\n";
      });
      o << "    }\n";
      break;
    case FOP_D1:
      o << "    { const R d0r=" << M(0) << ",d0i=" << M(1) << ",d1r=" << M(2) << ",d1i=" << M(3) << ";\n";
      for (int j = 0; j < D; ++j) {
        const char* s = (j & (1 << b0)) ? "d1" : "d0";
        o << "      { const R ar=x" << j << ",ai=y" << j << "; x" << j << "=fm(" << s << "r,ar,-" << s << "i*ai); y" << j
          << "=fm(" << s << "r,ai," << s << "i*ar); }\n";
      }
      o << "    }\n";
      break;
    case FOP_R1:
      if (cp) {
        o << "    { const u64 A0=bc(" << M(0) << "),A1=bc(" << M(1) << "),A2=bc(" << M(2) << "),A3=bc(" << M(3) << ");\n";
        pairs(b0, [&](int j, int k) {
          o << "      { const u64 A=pk(x" << j << ",y" << j << "), B=pk(x" << k << ",y" << k
            << "); const u64 C=ffma2(A0,A,fmul2(A1,B)), E=ffma2(A2,A,fmul2(A3,B)); x" << j << "=plo(C); y" << j
            << "=phi(C); x" << k << "=plo(E); y" << k << "=phi(E); }\n";
        });
        o << "    }\n";
        break;
      }
      o << "    { const R a0=" << M(0) << ",a1=" << M(1) << ",a2=" << M(2) << ",a3=" << M(3) << ";\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << "; x" << j
          << "=fm(a0,ar,a1*br); y" << j << "=fm(a0,ai,a1*bi); x" << k << "=fm(a2,ar,a3*br); y" << k
          << "=fm(a2,ai,a3*bi); }\n";
      });
      o << "    }\n";
      break;
    case FOP_DH:  // diag(1, q) (diag(q, 1) with flags bit 0): one half only
      if (op.unit == 0) o << "    { const R qr=" << M(0) << ",qi=" << M(1) << ";\n";
      for (int j = 0; j < D; ++j) {
        if (((j >> b0) & 1) == (op.flags & 1)) continue;
        o << "      { const R ar=x" << j << ",ai=y" << j << ";";
        if (op.unit == 2) o << " x" << j << "=-ar; y" << j << "=-ai; }\n";
        else if (op.unit == 3) o << " x" << j << "=-ai; y" << j << "=ar; }\n";
        else if (op.unit == 4) o << " x" << j << "=ai; y" << j << "=-ar; }\n";
        else o << " x" << j << "=fm(qr,ar,-qi*ai); y" << j << "=fm(qr,ai,qi*ar); }\n";
      }
      if (op.unit == 0) o << "    }\n";
      break;
    case FOP_HB: {  // [[1, s01], [s10, s11]]: adds and subtracts
      const char* s01 = (op.flags & 1) ? "-" : "+";
      const char* s10 = (op.flags & 2) ? "-" : "";
      const char* s11 = (op.flags & 4) ? "-" : "+";
      if (cp && !((op.flags & 2) && (op.flags & 4))) {
        // a + s01 b, then s10 a + s11 b as b + s10 a (s11 = +) or a + s11 b (s10 = +)
        o << "    { const u64 S01=bc(" << ((op.flags & 1) ? "-1.0f" : "1.0f") << "), S2=bc("
          << (((op.flags & 2) || (op.flags & 4)) ? "-1.0f" : "1.0f") << ");\n";
        pairs(b0, [&](int j, int k) {
          o << "      { const u64 A=pk(x" << j << ",y" << j << "), B=pk(x" << k << ",y" << k << "); const u64 C=ffma2(S01,B,A), E="
            << ((op.flags & 2) ? "ffma2(S2,A,B)" : "ffma2(S2,B,A)") << "; x" << j << "=plo(C); y" << j << "=phi(C); x" << k
            << "=plo(E); y" << k << "=phi(E); }\n";
        });
        o << "    }\n";
        break;
      }
      pairs(b0, [&](int j, int k) {
        o << "    { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << "; x" << j << "=ar" << s01
          << "br; y" << j << "=ai" << s01 << "bi; x" << k << "=" << s10 << "ar" << s11 << "br; y" << k << "=" << s10
          << "ai" << s11 << "bi; }\n";
      });
      break;
    }
    case FOP_RN: {  // [[1, p], [q, s]] or [[p, 1], [s, q]]: one FMA per component
      const bool B = op.flags & 2;
      const char* sg = (op.flags & 1) ? "-" : "";
      if (cp) {
        // (x_j, y_j) = p b + a; (x_k, y_k) = q a + s b, with s = -1 as q a + (-1) b
        o << "    { const u64 P=bc(" << M(0) << "),Q=bc(" << M(1) << ")" << ((op.flags & 1) ? ",N=bc(-1.0f)" : "")
          << ";\n";
        pairs(b0, [&](int j, int k) {
          o << "      { const u64 A=pk(x" << j << ",y" << j << "), B=pk(x" << k << ",y" << k << ");";
          o << " const u64 C=ffma2(P," << (B ? "A" : "B") << "," << (B ? "B" : "A") << ");";
          if (op.flags & 1)
            o << " const u64 E=ffma2(Q," << (B ? "B" : "A") << ",fmul2(N," << (B ? "A" : "B") << "));";
          else
            o << " const u64 E=ffma2(Q," << (B ? "B" : "A") << "," << (B ? "A" : "B") << ");";
          o << " x" << j << "=plo(C); y" << j << "=phi(C); x" << k << "=plo(E); y" << k << "=phi(E); }\n";
        });
        o << "    }\n";
        break;
      }
      o << "    { const R p=" << M(0) << ",q=" << M(1) << ";\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << ";";
        if (!B)
          o << " x" << j << "=fm(p,br,ar); y" << j << "=fm(p,bi,ai); x" << k << "=fm(q,ar," << sg << "br); y" << k
            << "=fm(q,ai," << sg << "bi); }\n";
        else
          o << " x" << j << "=fm(p,ar,br); y" << j << "=fm(p,ai,bi); x" << k << "=fm(q,br," << sg << "ar); y" << k
            << "=fm(q,bi," << sg << "ai); }\n";
      });
      o << "    }\n";
      break;
    }
    case FOP_RXN:  // [[1, it], [it, 1]] or [[-it, 1], [1, -it]]
      o << "    { const R t=" << M(0) << ";\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << ";";
        if (!(op.flags & 2))
          o << " x" << j << "=fm(-t,bi,ar); y" << j << "=fm(t,br,ai); x" << k << "=fm(-t,ai,br); y" << k
            << "=fm(t,ar,bi); }\n";
        else
          o << " x" << j << "=fm(t,ai,br); y" << j << "=fm(-t,ar,bi); x" << k << "=fm(t,bi,ar); y" << k
            << "=fm(-t,br,ai); }\n";
      });
      o << "    }\n";
      break;
    case FOP_RX1:
      o << "    { const R ca=" << M(0) << ",cb=" << M(1) << ";\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << "; x" << j
          << "=fm(ca,ar,-cb*bi); y" << j << "=fm(ca,ai,cb*br); x" << k << "=fm(ca,br,-cb*ai); y" << k
          << "=fm(ca,bi,cb*ar); }\n";
      });
      o << "    }\n";
      break;
    case FOP_X1:
      if (op.unit) {
        pairs(b0, [&](int j, int k) {
          o << "    { const R tr=x" << j << ",ti=y" << j << "; x" << j << "=x" << k << "; y" << j << "=y" << k << "; x" << k
            << "=tr; y" << k << "=ti; }\n";
        });
      } else {
        o << "    { const R p0r=" << M(0) << ",p0i=" << M(1) << ",p1r=" << M(2) << ",p1i=" << M(3) << ";\n";
        pairs(b0, [&](int j, int k) {
          o << "      { const R ar=x" << j << ",ai=y" << j << ",br=x" << k << ",bi=y" << k << "; x" << j
            << "=fm(p0r,br,-p0i*bi); y" << j << "=fm(p0r,bi,p0i*br); x" << k << "=fm(p1r,ar,-p1i*ai); y" << k
            << "=fm(p1r,ai,p1i*ar); }\n";
        });
        o << "    }\n";
      }
      break;
    case FOP_D2:
      o << "    { const R e0r=" << M(0) << ",e0i=" << M(1) << ",e1r=" << M(2) << ",e1i=" << M(3) << ",e2r=" << M(4)
        << ",e2i=" << M(5) << ",e3r=" << M(6) << ",e3i=" << M(7) << ";\n";
      for (int j = 0; j < D; ++j) {
        const int r = ((j >> b0) & 1) * 2 + ((j >> b1) & 1);
        o << "      { const R ar=x" << j << ",ai=y" << j << "; x" << j << "=fm(e" << r << "r,ar,-e" << r << "i*ai); y" << j
          << "=fm(e" << r << "r,ai,e" << r << "i*ar); }\n";
      }
      o << "    }\n";
      break;
    case FOP_G2:
      o << "    {";
      for (int e = 0; e < 32; ++e) o << (e ? "," : " const R ") << "g" << e << "=" << M(e);
      o << ";\n";
      quads(b0, b1, [&](const int* q) {
        o << "      { const R ";
        for (int c = 0; c < 4; ++c) o << (c ? "," : "") << "r" << c << "=x" << q[c] << ",i" << c << "=y" << q[c];
        o << ";";
        for (int r = 0; r < 4; ++r) {
          std::ostringstream re, im;
          re << "(R)0";  // a zero of the arithmetic's type (float, double or float-float)
          im << "(R)0";
          for (int c = 0; c < 4; ++c) {
            re.str("fm(g" + std::to_string(8 * r + 2 * c) + ",r" + std::to_string(c) + ",fm(-g" +
                   std::to_string(8 * r + 2 * c + 1) + ",i" + std::to_string(c) + "," + re.str() + "))");
            im.str("fm(g" + std::to_string(8 * r + 2 * c) + ",i" + std::to_string(c) + ",fm(g" +
                   std::to_string(8 * r + 2 * c + 1) + ",r" + std::to_string(c) + "," + im.str() + "))");
          }
          o << " x" << q[r] << "=" << re.str() << "; y" << q[r] << "=" << im.str() << ";";
        }
        o << " }\n";
      });
      o << "    }\n";
      break;
    case FOP_P2:
    case FOP_CX:
    case FOP_SW: {
      int P[4];
      bool unit = true;
      if (op.type == FOP_CX) {  // control b0, target b1: rows 2 and 3 swap
        P[0] = 0, P[1] = 1, P[2] = 3, P[3] = 2;
      } else if (op.type == FOP_SW) {
        P[0] = 0, P[1] = 2, P[2] = 1, P[3] = 3;
      } else {
        for (int r = 0; r < 4; ++r) P[r] = (op.flags >> (2 * r)) & 3;
        unit = op.unit != 0;
      }
      o << "    {";
      if (!unit)
        for (int e = 0; e < 8; ++e) o << (e ? "," : " const R ") << "h" << e << "=" << M(e);
      o << (unit ? "\n" : ";\n");
      quads(b0, b1, [&](const int* q) {
        o << "      { const R ";
        for (int c = 0; c < 4; ++c) o << (c ? "," : "") << "r" << c << "=x" << q[c] << ",i" << c << "=y" << q[c];
        o << ";";
        for (int r = 0; r < 4; ++r) {
          if (unit) {
            o << " x" << q[r] << "=r" << P[r] << "; y" << q[r] << "=i" << P[r] << ";";
          } else {
            o << " x" << q[r] << "=fm(h" << 2 * r << ",r" << P[r] << ",-h" << 2 * r + 1 << "*i" << P[r] << "); y" << q[r]
              << "=fm(h" << 2 * r << ",i" << P[r] << ",h" << 2 * r + 1 << "*r" << P[r] << ");";
          }
        }
        o << " }\n";
      });
      o << "    }\n";
      break;
    }
  }
}

// ------------------------------------------------------------------ packed (complex64)
// In a packed phase the 2^NB register amplitudes are held as pairs that differ in
// register bit P: X<j> = (x_j, x_{j|P}), Y<j> = (y_j, y_{j|P}) for j with bit P
// clear.  An op that does not touch bit P applies the same arithmetic to both
// lanes, so it runs on the pairs with two-lane FMAs: half the instructions of the
// scalar code.  Diagonal ops on bit P take per-lane coefficients.  Other ops on
// bit P fall back to the scalar code (unpack, op, repack).

static bool touches(const FOp& op, int P) {
  const bool two = op.type == FOP_G2 || op.type == FOP_D2 || op.type == FOP_P2 || op.type == FOP_CX ||
                   op.type == FOP_SW;
  return op.b0 == P || (two && op.b1 == P);
}

// pack bit of a phase: the register bit that the fewest non-diagonal ops touch
static int choose_pack_bit(const FusedArgs<float>& a, const FPhase& ph, int NB) {
  int best = NB - 1, bestc = 1 << 30;
  for (int b = NB - 1; b >= 0; --b) {
    int cnt = 0;
    for (int oi = ph.op0; oi < ph.op0 + ph.nop; ++oi) {
      const FOp& op = a.op[oi];
      if (op.type != FOP_D1 && op.type != FOP_D2 && op.type != FOP_DH && touches(op, b)) ++cnt;
    }
    if (cnt < bestc) best = b, bestc = cnt;
  }
  return best;
}

// emits op on the pairs; false: the op needs the scalar fallback
static bool emit_op_packed(std::ostringstream& o, const FOp& op, int NB, int P, const char* mref = "a.mat") {
  const int D = 1 << NB;
  auto M = [&](int e) {
    std::ostringstream s;
    s << mref << "[" << (op.moff + e) << "]";
    return s.str();
  };
  auto bcs = [&](const char* name, int e, bool neg) {  // broadcast coefficient pair
    o << " const u64 " << name << "=bc(" << (neg ? "-" : "") << M(e) << ");";
  };
  auto k0 = [&](int j) { return !(j & (1 << P)); };
  auto pairs = [&](int B, auto&& body) {
    for (int j = 0; j < D; ++j)
      if (k0(j) && !(j & (1 << B))) body(j, j | (1 << B));
  };
  auto quads = [&](int B0, int B1, auto&& body) {
    for (int j = 0; j < D; ++j)
      if (k0(j) && !(j & ((1 << B0) | (1 << B1)))) {
        const int q[4] = {j, j | (1 << B1), j | (1 << B0), j | (1 << B0) | (1 << B1)};
        body(q);
      }
  };
  const int b0 = op.b0, b1 = op.b1;
  if (op.type == FOP_D1 || op.type == FOP_D2) {
    // diagonal: coefficient index of each lane; per-lane pairs when the index
    // depends on bit P
    o << "    {";
    for (int j = 0; j < D; ++j) {
      if (!k0(j)) continue;
      int r[2];
      for (int l = 0; l < 2; ++l) {
        const int jj = l ? (j | (1 << P)) : j;
        r[l] = op.type == FOP_D1 ? ((jj >> b0) & 1) : ((jj >> b0) & 1) * 2 + ((jj >> b1) & 1);
      }
      const int base = 0;
      (void)base;
      o << "\n      { const u64 er=pk(" << M(2 * r[0]) << "," << M(2 * r[1]) << "), ei=pk(" << M(2 * r[0] + 1) << ","
        << M(2 * r[1] + 1) << "), nei=pk(-" << M(2 * r[0] + 1) << ",-" << M(2 * r[1] + 1) << "); const u64 ar=X" << j
        << ", ai=Y" << j << "; X" << j << "=ffma2(er,ar,fmul2(nei,ai)); Y" << j << "=ffma2(er,ai,fmul2(ei,ar)); }";
    }
    o << "\n    }\n";
    return true;
  }
  if (op.type == FOP_DH) {
    // diag(1, q) (diag(q, 1) with flags bit 0) on bit b0: on the pack bit only the
    // lanes of the multiplied half change (high lanes for diag(1, q))
    const bool onp = b0 == P, lo = op.flags & 1;
    const char* SG = !onp ? "0x8000000080000000ULL" : (lo ? "0x80000000ULL" : "0x8000000000000000ULL");
    const char* HIT = lo ? "0xFFFFFFFFULL" : "0xFFFFFFFF00000000ULL";   // lane changed on the pack bit
    const char* KEEP = lo ? "0xFFFFFFFF00000000ULL" : "0xFFFFFFFFULL";
    if (op.unit == 0) {
      o << "    { const float qr=" << M(0) << ", qi=" << M(1) << ";";
      if (onp && !lo)
        o << " const u64 er=pk(1.0f,qr), ei=pk(0.0f,qi), nei=pk(-0.0f,-qi);";
      else if (onp)
        o << " const u64 er=pk(qr,1.0f), ei=pk(qi,0.0f), nei=pk(-qi,-0.0f);";
      else
        o << " const u64 er=bc(qr), ei=bc(qi), nei=bc(-qi);";
      o << "\n";
    }
    for (int j = 0; j < D; ++j) {
      if (!k0(j) || (!onp && ((j >> b0) & 1) == (int)lo)) continue;
      const std::string X = "X" + std::to_string(j), Y = "Y" + std::to_string(j);
      if (op.unit == 0)
        o << "      { const u64 ar=" << X << ", ai=" << Y << "; " << X << "=ffma2(er,ar,fmul2(nei,ai)); " << Y
          << "=ffma2(er,ai,fmul2(ei,ar)); }\n";
      else if (op.unit == 2)
        o << "    " << X << "^=" << SG << "; " << Y << "^=" << SG << ";\n";
      else if (!onp && op.unit == 3)
        o << "    { const u64 ar=" << X << "; " << X << "=" << Y << "^" << SG << "; " << Y << "=ar; }\n";
      else if (!onp)  // unit 4
        o << "    { const u64 ar=" << X << "; " << X << "=" << Y << "; " << Y << "=ar^" << SG << "; }\n";
      else if (op.unit == 3)  // hit lane (x, y) -> (-y, x)
        o << "    { const u64 ar=" << X << ", ai=" << Y << "; " << X << "=(ar&" << KEEP << ")|((ai^" << SG << ")&" << HIT
          << "); " << Y << "=(ai&" << KEEP << ")|(ar&" << HIT << "); }\n";
      else  // hit lane (x, y) -> (y, -x)
        o << "    { const u64 ar=" << X << ", ai=" << Y << "; " << X << "=(ar&" << KEEP << ")|(ai&" << HIT << "); " << Y
          << "=(ai&" << KEEP << ")|((ar^" << SG << ")&" << HIT << "); }\n";
    }
    if (op.unit == 0) o << "    }\n";
    return true;
  }
  if (touches(op, P)) return false;
  switch (op.type) {
    case FOP_HB: {  // [[1, s01], [s10, s11]] as two-lane fma(+-1, a, b): one rounding, = add / subtract
      const bool n01 = op.flags & 1, n10 = op.flags & 2, n11 = op.flags & 4;
      o << "    { const u64 P1=bc(1.0f), N1=bc(-1.0f);\n";
      pairs(b0, [&](int j, int k) {
        for (int c = 0; c < 2; ++c) {
          const std::string A = (c ? "Y" : "X") + std::to_string(j), B = (c ? "Y" : "X") + std::to_string(k);
          o << "      { const u64 ua=" << A << ", ub=" << B << "; " << A << "=ffma2(" << (n01 ? "N1" : "P1") << ",ub,ua); "
            << B << "=";
          if (!n11) o << "ffma2(" << (n10 ? "N1" : "P1") << ",ua,ub); }\n";
          else if (!n10) o << "ffma2(N1,ub,ua); }\n";
          else o << "ffma2(N1,ua,ub^0x8000000080000000ULL); }\n";
        }
      });
      o << "    }\n";
      return true;
    }
    case FOP_RN: {  // one two-lane FMA per register; s = -1 flips the addend's signs
      const bool B = op.flags & 2, neg = op.flags & 1;
      o << "    { const u64 pp=bc(" << M(0) << "), qq=bc(" << M(1) << ");\n";
      pairs(b0, [&](int j, int k) {
        for (int c = 0; c < 2; ++c) {
          const std::string A = (c ? "Y" : "X") + std::to_string(j), Bk = (c ? "Y" : "X") + std::to_string(k);
          const std::string sa = neg ? "ua^0x8000000080000000ULL" : "ua", sb = neg ? "ub^0x8000000080000000ULL" : "ub";
          o << "      { const u64 ua=" << A << ", ub=" << Bk << "; ";
          if (!B) o << A << "=ffma2(pp,ub,ua); " << Bk << "=ffma2(qq,ua," << sb << "); }\n";
          else o << A << "=ffma2(pp,ua,ub); " << Bk << "=ffma2(qq,ub," << sa << "); }\n";
        }
      });
      o << "    }\n";
      return true;
    }
    case FOP_RXN:
      o << "    { const u64 tt=bc(" << M(0) << "), nt=bc(-" << M(0) << ");\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const u64 ar=X" << j << ",ai=Y" << j << ",br=X" << k << ",bi=Y" << k << ";";
        if (!(op.flags & 2))
          o << " X" << j << "=ffma2(nt,bi,ar); Y" << j << "=ffma2(tt,br,ai); X" << k << "=ffma2(nt,ai,br); Y" << k
            << "=ffma2(tt,ar,bi); }\n";
        else
          o << " X" << j << "=ffma2(tt,ai,br); Y" << j << "=ffma2(nt,ar,bi); X" << k << "=ffma2(tt,bi,ar); Y" << k
            << "=ffma2(nt,br,ai); }\n";
      });
      o << "    }\n";
      return true;
    case FOP_G1:
      o << "    {";
      bcs("m0", 0, false), bcs("m1", 1, false), bcs("n1", 1, true), bcs("m2", 2, false), bcs("m3", 3, false);
      bcs("n3", 3, true), bcs("m4", 4, false), bcs("m5", 5, false), bcs("n5", 5, true), bcs("m6", 6, false);
      bcs("m7", 7, false), bcs("n7", 7, true);
      o << "\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const u64 ar=X" << j << ",ai=Y" << j << ",br=X" << k << ",bi=Y" << k << ";"
          << " X" << j << "=ffma2(m0,ar,ffma2(n1,ai,ffma2(m2,br,fmul2(n3,bi))));"
          << " Y" << j << "=ffma2(m0,ai,ffma2(m1,ar,ffma2(m2,bi,fmul2(m3,br))));"
          << " X" << k << "=ffma2(m4,ar,ffma2(n5,ai,ffma2(m6,br,fmul2(n7,bi))));"
          << " Y" << k << "=ffma2(m4,ai,ffma2(m5,ar,ffma2(m6,bi,fmul2(m7,br)))); }\n";
      });
      o << "    }\n";
      return true;
    case FOP_R1:
      o << "    {";
      bcs("a0", 0, false), bcs("a1", 1, false), bcs("a2", 2, false), bcs("a3", 3, false);
      o << "\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const u64 ar=X" << j << ",ai=Y" << j << ",br=X" << k << ",bi=Y" << k << "; X" << j
          << "=ffma2(a0,ar,fmul2(a1,br)); Y" << j << "=ffma2(a0,ai,fmul2(a1,bi)); X" << k << "=ffma2(a2,ar,fmul2(a3,br)); Y" << k
          << "=ffma2(a2,ai,fmul2(a3,bi)); }\n";
      });
      o << "    }\n";
      return true;
    case FOP_RX1:
      o << "    {";
      bcs("ca", 0, false), bcs("cb", 1, false), bcs("nb", 1, true);
      o << "\n";
      pairs(b0, [&](int j, int k) {
        o << "      { const u64 ar=X" << j << ",ai=Y" << j << ",br=X" << k << ",bi=Y" << k << "; X" << j
          << "=ffma2(ca,ar,fmul2(nb,bi)); Y" << j << "=ffma2(ca,ai,fmul2(cb,br)); X" << k << "=ffma2(ca,br,fmul2(nb,ai)); Y" << k
          << "=ffma2(ca,bi,fmul2(cb,ar)); }\n";
      });
      o << "    }\n";
      return true;
    case FOP_X1:
      if (op.unit) {
        pairs(b0, [&](int j, int k) {
          o << "    { const u64 tr=X" << j << ",ti=Y" << j << "; X" << j << "=X" << k << "; Y" << j << "=Y" << k << "; X" << k
            << "=tr; Y" << k << "=ti; }\n";
        });
      } else {
        o << "    {";
        bcs("p0r", 0, false), bcs("p0i", 1, false), bcs("n0i", 1, true);
        bcs("p1r", 2, false), bcs("p1i", 3, false), bcs("n1i", 3, true);
        o << "\n";
        pairs(b0, [&](int j, int k) {
          o << "      { const u64 ar=X" << j << ",ai=Y" << j << ",br=X" << k << ",bi=Y" << k << "; X" << j
            << "=ffma2(p0r,br,fmul2(n0i,bi)); Y" << j << "=ffma2(p0r,bi,fmul2(p0i,br)); X" << k << "=ffma2(p1r,ar,fmul2(n1i,ai)); Y" << k
            << "=ffma2(p1r,ai,fmul2(p1i,ar)); }\n";
        });
        o << "    }\n";
      }
      return true;
    case FOP_G2:
      o << "    {";
      for (int e = 0; e < 32; ++e) {
        o << " const u64 g" << e << "=bc(" << M(e) << ");";
        if (e & 1) o << " const u64 ng" << e << "=bc(-" << M(e) << ");";
      }
      o << "\n";
      quads(b0, b1, [&](const int* q) {
        o << "      { const u64 ";
        for (int c = 0; c < 4; ++c) o << (c ? "," : "") << "r" << c << "=X" << q[c] << ",i" << c << "=Y" << q[c];
        o << ";";
        for (int r = 0; r < 4; ++r) {
          std::string re = "fmul2(g" + std::to_string(8 * r) + ",r0)", im = "fmul2(g" + std::to_string(8 * r) + ",i0)";
          re = "ffma2(ng" + std::to_string(8 * r + 1) + ",i0," + re + ")";
          im = "ffma2(g" + std::to_string(8 * r + 1) + ",r0," + im + ")";
          for (int c = 1; c < 4; ++c) {
            const std::string gr = std::to_string(8 * r + 2 * c), gi = std::to_string(8 * r + 2 * c + 1);
            const std::string cs = std::to_string(c);
            re = "ffma2(g" + gr + ",r" + cs + ",ffma2(ng" + gi + ",i" + cs + "," + re + "))";
            im = "ffma2(g" + gr + ",i" + cs + ",ffma2(g" + gi + ",r" + cs + "," + im + "))";
          }
          o << " X" << q[r] << "=" << re << "; Y" << q[r] << "=" << im << ";";
        }
        o << " }\n";
      });
      o << "    }\n";
      return true;
    case FOP_P2:
    case FOP_CX:
    case FOP_SW: {
      int Pm[4];
      bool unit = true;
      if (op.type == FOP_CX) {
        Pm[0] = 0, Pm[1] = 1, Pm[2] = 3, Pm[3] = 2;
      } else if (op.type == FOP_SW) {
        Pm[0] = 0, Pm[1] = 2, Pm[2] = 1, Pm[3] = 3;
      } else {
        for (int r = 0; r < 4; ++r) Pm[r] = (op.flags >> (2 * r)) & 3;
        unit = op.unit != 0;
      }
      o << "    {";
      if (!unit)
        for (int e = 0; e < 8; ++e) {
          o << " const u64 h" << e << "=bc(" << M(e) << ");";
          if (e & 1) o << " const u64 nh" << e << "=bc(-" << M(e) << ");";
        }
      o << "\n";
      quads(b0, b1, [&](const int* q) {
        o << "      { const u64 ";
        for (int c = 0; c < 4; ++c) o << (c ? "," : "") << "r" << c << "=X" << q[c] << ",i" << c << "=Y" << q[c];
        o << ";";
        for (int r = 0; r < 4; ++r) {
          if (unit)
            o << " X" << q[r] << "=r" << Pm[r] << "; Y" << q[r] << "=i" << Pm[r] << ";";
          else
            o << " X" << q[r] << "=ffma2(h" << 2 * r << ",r" << Pm[r] << ",fmul2(nh" << 2 * r + 1 << ",i" << Pm[r] << ")); Y"
              << q[r] << "=ffma2(h" << 2 * r << ",i" << Pm[r] << ",fmul2(h" << 2 * r + 1 << ",r" << Pm[r] << "));";
        }
        o << " }\n";
      });
      o << "    }\n";
      return true;
    }
  }
  return false;
}

// complex64 specialised passes run scalar FP32 code unless a plan says otherwise
// (BTGPU_JIT_PACKED=1: two-lane code by default).  With the factored ops (one
// FMA per component for rotations) the moves that repack amplitude pairs for the
// two-lane form at every phase boundary cost more than the halved FMA issue saves:
// 33-qubit brickwork 0.884 s per circuit scalar, 0.963 s two-lane.
bool bt_jit_packed_default() {
  static const bool v = env_int("BTGPU_JIT_PACKED", 0, 0, 1) != 0;
  return v;
}

// Whether a phase may read (first phase) or write (last phase) its register
// amplitudes straight from / to global memory: a warp's access for one register
// index spans the lanes' tile bits (the lowest non-register bits), and it is
// taken when it touches at most twice the 128-byte lines its bytes need.
// BTGPU_JIT_DIRECT: 0 never, 1 by that rule (default), 2 always.
static bool direct_ok(const FPhase& ph, int NB, int M, bool f) {
  static const int mode = env_int("BTGPU_JIT_DIRECT", 1, 0, 2);
  if (mode != 1) return mode == 2;
  uint32_t regmask = 0;
  for (int b = 0; b < NB; ++b) regmask |= 1u << ph.reg[b];
  const bool pair = f && (regmask & 1);
  const int bytes = pair ? 16 : (f ? 8 : 16);  // per lane and access
  const int linebits = f ? 4 : 3;              // tile bits inside a 128-byte line
  int lanes = 0, outside = 0;
  for (int bit = 0; bit < M && lanes < 5; ++bit)
    if (!((regmask >> bit) & 1)) {
      outside += bit >= linebits;
      ++lanes;
    }
  const int lines = 1 << outside, need = std::max(1, 32 * bytes / 128);
  return lines <= 2 * need;
}

// next-tile prefetch into shared memory during a direct last phase
// (BTGPU_JIT_PREFETCH=1; off by default: on the 28- and 33-qubit brickwork the
// extra shared-memory copies cost more than the hidden load latency saves)
// L2 prefetch of each CTA's next tile during the current one (BTGPU_JIT_L2PF)
static bool l2_prefetch_on() {
  static const bool v = env_int("BTGPU_JIT_L2PF", 1, 0, 1) != 0;
  return v;
}

static bool prefetch_on() {
  static const bool v = env_int("BTGPU_JIT_PREFETCH", 0, 0, 1) != 0;
  return v;
}

template <typename R>
static void gen_kernel(std::ostringstream& o, const FusedArgs<R>& a, int NB, const std::string& name) {
  const bool f = sizeof(R) == 4;
  const int M = a.M, c = a.c, D = 1 << NB;
  const int NM = f ? BT_FUSED_MAX_REALS_F : BT_FUSED_MAX_REALS_D;
  const int V = f ? 2 : 1;
  const int T = 1 << (M - NB);
  const int NPT = (1 << M) / V / T;
  const char* T2 = f ? "cf" : "cd";
  // float-float form of a complex128 pass (not the per-member kernels)
  const bool ffm = ff_pass(a);
  const char* TT = ffm ? "ffc2" : T2;  // the shared-memory tile's element
  // per-member entries (a.permem): member m of the launch reads its ops' entries from
  // row m of the table mm (mstride reals per row) instead of the kernel parameters
  const char* mref = a.permem ? "cm" : (ffm ? "ffp(a.mat)" : "a.mat");
  // six register bits: 128 threads of up to 170 registers, three CTAs per SM
  // (BTGPU_JIT_MINB6 sets another count)
  static const int minb6 = env_int("BTGPU_JIT_MINB6", 3, 1, 4);
  const int minb = NB >= 6 ? minb6 : bt_jit_min_blocks();
  o << "extern \"C\" __global__ void __launch_bounds__(" << T << ", " << minb << ") " << name << "("
    << T2 << "* __restrict__ psi, const "
    << (f ? "JitArgsF<" : "JitArgsD<") << NM << "> a";
  if (a.permem) o << ", const " << (f ? "float" : "double") << "* __restrict__ mm, const i64 mstride";
  o << ") {\n";
  o << "  typedef " << (f ? "float" : (ffm ? "ff" : "double")) << " R;\n";
  const int NP = a.nphase;
  if (NP == 0) {  // nothing to apply
    o << "}\n";
    return;
  }
  // The first phase loads its register amplitudes straight from global memory and
  // the last one stores them straight back, where a warp's accesses stay nearly
  // coalesced; otherwise the tile is staged through shared memory with 16-byte
  // accesses.  A one-phase pass with both direct needs no shared memory at all.
  // With prefetch (the last phase direct), the next tile is instead copied into
  // the shared-memory tile with cp.async as soon as the last phase has read the
  // current one, so its load latency hides behind that phase's arithmetic and
  // stores.
  const bool dlast = direct_ok(a.ph[NP - 1], NB, M, f);
  const bool pf = dlast && prefetch_on() && !ffm;
  const bool dfirst = !pf && direct_ok(a.ph[0], NB, M, f);
  const bool staged = pf || !dfirst || !dlast;
  const bool use_smem = staged || NP > 1;
  auto thread_off = [&](const FPhase& ph) {  // global offset of the thread's non-register tile bits
    uint32_t regmask = 0;
    for (int b = 0; b < NB; ++b) regmask |= 1u << ph.reg[b];
    std::ostringstream e;
    e << "(i64)0";
    int nb = 0;
    for (int bit = 0; bit < M; ++bit)
      if (!((regmask >> bit) & 1)) e << " | ((i64)((threadIdx.x >> " << nb++ << ") & 1) << " << a.tbits[bit] << ")";
    return e.str();
  };
  auto reg_off = [&](const FPhase& ph, int j) {  // global offset of register amplitude j
    int64_t v = 0;
    for (int b = 0; b < NB; ++b)
      if ((j >> b) & 1) v |= (int64_t)1 << a.tbits[ph.reg[b]];
    return v;
  };
  if (use_smem) {
    o << "  extern __shared__ __align__(16) unsigned char smem_raw[];\n";
    o << "  " << TT << "* tile = reinterpret_cast<" << TT << "*>(smem_raw);\n";
  }
  if (staged) {
    o << "  i64* runoff = reinterpret_cast<i64*>(smem_raw + " << ((f ? 8 : 16) << M) << ");\n";
    o << "  for (int r = threadIdx.x; r < " << (1 << (M - c)) << "; r += " << T << ") { i64 v = 0;";
    for (int b = 0; b < M - c; ++b) o << " v |= (i64)((r >> " << b << ") & 1) << " << a.tbits[c + b] << ";";
    o << " runoff[r] = v; }\n  __syncthreads();\n";
  }
  if (dfirst) o << "  const i64 tf = " << thread_off(a.ph[0]) << ";\n";
  if (dlast) o << "  const i64 tl = " << thread_off(a.ph[NP - 1]) << ";\n";
  o << "  const i64 per = 1LL << a.lg_tiles, total = per * a.nmem;\n";
  // first amplitude of tile `tid`: the tile bits inserted as zeros into the tile index
  o << "  auto tile_ptr = [&](i64 tid) -> " << T2 << "* {\n";
  o << "    const i64 mem = a.member_lo + (tid >> a.lg_tiles);\n    u64 base = (u64)(tid & (per - 1));\n";
  for (int i = 0; i < M; ++i) {
    const int p = a.tbits[i];
    o << "    base = ((base >> " << p << ") << " << (p + 1) << ") | (base & " << fmt_u64((1ULL << p) - 1) << ");\n";
  }
  o << "    return psi + (mem << a.nbits) + base;\n  };\n";
  if (pf) {
    // one amplitude per copy, straight into its swizzled slot; one commit group
    // per tile (empty past the end)
    o << "  auto fetch = [&](i64 tid) {\n    if (tid < total) {\n      const " << T2 << "* g = tile_ptr(tid);\n";
    o << "      const unsigned sb = (unsigned)__cvta_generic_to_shared(tile);\n";
    for (int i = 0; i < (1 << M) / T; ++i) {
      o << "      { const int l = threadIdx.x + " << i * T << "; const " << T2 << "* src = g + runoff[l >> " << c
        << "] + (l & " << ((1 << c) - 1) << "); const unsigned dst = sb + "
        << (f ? "8u * (unsigned)(l ^ ((l >> 4) & 15))" : "16u * (unsigned)(l ^ ((l >> 3) & 7))") << ";";
      o << (f ? " asm volatile(\"cp.async.ca.shared.global [%0], [%1], 8;\" :: \"r\"(dst), \"l\"(src) : \"memory\"); }\n"
              : " asm volatile(\"cp.async.cg.shared.global [%0], [%1], 16;\" :: \"r\"(dst), \"l\"(src) : \"memory\"); }\n");
    }
    o << "    }\n    asm volatile(\"cp.async.commit_group;\" ::: \"memory\");\n  };\n";
    o << "  fetch(blockIdx.x);\n";
  }
  // L2 prefetch of the CTA's next tile while this one computes: each thread asks
  // for whole contiguous runs (2^c amplitudes) of it
  const int nruns = 1 << (M - c), run_bytes = (f ? 8 : 16) << c;
  const bool l2pf = l2_prefetch_on() && pf == false;
  if (l2pf) {
    o << "  const int pr = threadIdx.x;\n  i64 roff = 0;\n";
    for (int b = 0; b < M - c; ++b) o << "  roff |= (i64)((pr >> " << b << ") & 1) << " << a.tbits[c + b] << ";\n";
  }
  o << "  for (i64 tid = blockIdx.x; tid < total; tid += gridDim.x) {\n";
  o << "    " << T2 << "* g = tile_ptr(tid);\n";
  if (a.permem) o << "    const R* cm = mm + (tid >> a.lg_tiles) * mstride;\n";
  if (l2pf) {
    o << "    if (tid + gridDim.x < total" << (T > nruns ? " && threadIdx.x < " + std::to_string(nruns) : std::string())
      << ") { const " << T2 << "* gn = tile_ptr(tid + gridDim.x) + roff;";
    o << " asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], " << run_bytes << ";\" :: \"l\"(gn) : \"memory\");";
    if (T < nruns) {  // fewer threads than runs: the rest by stride
      o << " for (int q = " << T << "; q < " << nruns << "; q += " << T << ") { i64 ro = 0;";
      for (int b = 0; b < M - c; ++b) o << " ro |= (i64)(((threadIdx.x + q) >> " << b << ") & 1) << " << a.tbits[c + b] << ";";
      o << " const " << T2 << "* gq = tile_ptr(tid + gridDim.x) + ro; asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], "
        << run_bytes << ";\" :: \"l\"(gq) : \"memory\"); }";
    }
    o << " }\n";
  }
  if (pf) o << "    asm volatile(\"cp.async.wait_group 0;\" ::: \"memory\");\n    __syncthreads();\n";
  if (!dfirst && !pf) {
    // tile load: every 16-byte load in flight, then into the swizzled tile
    o << "    {\n";
    for (int i = 0; i < NPT; ++i)
      o << "      const int l" << i << " = (threadIdx.x + " << i * T << ") * " << V << "; const f4 b" << i
        << " = *reinterpret_cast<const f4*>(g + runoff[l" << i << " >> " << c << "] + (l" << i << " & "
        << ((1 << c) - 1) << "));\n";
    for (int i = 0; i < NPT; ++i) {
      if (f)
        o << "      { const int s0 = l" << i << " ^ ((l" << i << " >> 4) & 15), s1 = (l" << i << " + 1) ^ (((l" << i
          << " + 1) >> 4) & 15); tile[s0] = cf{b" << i << ".x, b" << i << ".y}; tile[s1] = cf{b" << i << ".z, b" << i
          << ".w}; }\n";
      else if (ffm)
        o << "      { const cd d = *reinterpret_cast<const cd*>(&b" << i << "); tile[l" << i << " ^ ((l" << i
          << " >> 3) & 7)] = ffc2{ff(d.x), ff(d.y)}; }\n";
      else
        o << "      *reinterpret_cast<f4*>(&tile[l" << i << " ^ ((l" << i << " >> 3) & 7)]) = b" << i << ";\n";
    }
    o << "    }\n    __syncthreads();\n";
  }
  for (int p = 0; p < NP; ++p) {
    const FPhase& ph = a.ph[p];
    const bool rd_direct = p == 0 && dfirst, wr_direct = p == NP - 1 && dlast;
    // complex64 amplitude pairs that differ in tile bit 0 (register bit 0) move as 16 bytes
    const bool pair = f && ph.reg[0] == 0;
    uint32_t regmask = 0;
    for (int b = 0; b < NB; ++b) regmask |= 1u << ph.reg[b];
    o << "    { // phase " << p << "\n";
    if (!rd_direct || !wr_direct) {
      o << "    const int t = threadIdx.x; const int lb = 0";
      int nb = 0;
      for (int bit = 0; bit < M; ++bit)
        if (!((regmask >> bit) & 1)) {
          o << " | (((t >> " << nb << ") & 1) << " << bit << ")";
          ++nb;
        }
      o << ";\n    const int sb = " << (f ? "lb ^ ((lb >> 4) & 15)" : "lb ^ ((lb >> 3) & 7)") << ";\n";
    }
    o << "    R ";
    for (int j = 0; j < D; ++j) o << (j ? ", " : "") << "x" << j << ", y" << j;
    o << ";\n";
    std::vector<int> offs(D);
    for (int j = 0; j < D; ++j) {
      int l = 0;
      for (int b = 0; b < NB; ++b)
        if ((j >> b) & 1) l |= 1 << ph.reg[b];
      offs[j] = swz_host(f, l);  // the swizzle is XOR-linear: swz(lb | l) = swz(lb) ^ swz(l)
    }
    // Only the swizzled low bits (0-3 complex64, 0-2 complex128) of an offset can
    // meet the thread's bits: above them offs[j] holds register bits, where sb is
    // zero, so sb ^ offs[j] = (sb ^ low) + high.  One XOR per distinct low part;
    // the high part becomes a constant offset of the access.
    const int lowmask = f ? 15 : 7;
    std::vector<int> lows;
    auto saddr = [&](int j) {
      const int lo = offs[j] & lowmask, hi = offs[j] & ~lowmask;
      const int k = (int)(std::find(lows.begin(), lows.end(), lo) - lows.begin());
      return "s" + std::to_string(k) + (hi ? " + " + std::to_string(hi) : std::string());
    };
    if (!rd_direct || !wr_direct) {
      for (int j = 0; j < D; ++j)
        if (std::find(lows.begin(), lows.end(), offs[j] & lowmask) == lows.end()) lows.push_back(offs[j] & lowmask);
      for (size_t k = 0; k < lows.size(); ++k) o << "    const int s" << k << " = sb ^ " << lows[k] << ";\n";
    }
    if (rd_direct) {
      o << "    { const " << T2 << "* gp = g + tf;\n";
      for (int j = 0; j < D; ++j) {
        if (pair && (j & 1)) continue;
        if (pair)
          o << "    { const f4 v = *reinterpret_cast<const f4*>(gp + " << reg_off(ph, j) << "LL); x" << j << " = v.x; y"
            << j << " = v.y; x" << (j | 1) << " = v.z; y" << (j | 1) << " = v.w; }\n";
        else
          o << "    { const " << T2 << " v = gp[" << reg_off(ph, j) << "LL]; x" << j << " = v.x; y" << j << " = v.y; }\n";
      }
      o << "    }\n";
    } else {
      for (int j = 0; j < D; ++j)
        o << "    { const " << TT << " v = tile[" << saddr(j) << "]; x" << j << " = v.x; y" << j << " = v.y; }\n";
      // the tile's last shared-memory reads: the next tile may overwrite it once every warp is past them
      if (wr_direct) o << "    __syncthreads();\n";
      if (wr_direct && pf) o << "    fetch(tid + gridDim.x);\n";
    }
    if (f && a.packed) {
      const int P = choose_pack_bit(*reinterpret_cast<const FusedArgs<float>*>(&a), ph, NB);
      auto pack = [&]() {
        for (int j = 0; j < D; ++j)
          if (!(j & (1 << P)))
            o << "    X" << j << "=pk(x" << j << ",x" << (j | (1 << P)) << "); Y" << j << "=pk(y" << j << ",y"
              << (j | (1 << P)) << ");\n";
      };
      auto unpack = [&]() {
        for (int j = 0; j < D; ++j)
          if (!(j & (1 << P)))
            o << "    x" << j << "=plo(X" << j << "); x" << (j | (1 << P)) << "=phi(X" << j << "); y" << j << "=plo(Y" << j
              << "); y" << (j | (1 << P)) << "=phi(Y" << j << ");\n";
      };
      o << "    u64 ";
      bool first = true;
      for (int j = 0; j < D; ++j)
        if (!(j & (1 << P))) {
          o << (first ? "" : ", ") << "X" << j << ", Y" << j;
          first = false;
        }
      o << ";\n";
      pack();
      for (int oi = ph.op0; oi < ph.op0 + ph.nop; ++oi) {
        std::ostringstream po;
        if (emit_op_packed(po, a.op[oi], NB, P, mref)) {
          o << po.str();
        } else {  // scalar fallback for an op on the pack bit
          unpack();
          emit_op(o, a.op[oi], NB, mref);
          pack();
        }
      }
      unpack();
    } else {
      for (int oi = ph.op0; oi < ph.op0 + ph.nop; ++oi) emit_op(o, a.op[oi], NB, mref, f && cpair_on());
    }
    if (wr_direct) {
      o << "    { " << T2 << "* gp = g + tl;\n";
      for (int j = 0; j < D; ++j) {
        if (pair && (j & 1)) continue;
        if (pair)
          o << "    *reinterpret_cast<f4*>(gp + " << reg_off(ph, j) << "LL) = f4{x" << j << ", y" << j << ", x"
            << (j | 1) << ", y" << (j | 1) << "};\n";
        else
          o << "    gp[" << reg_off(ph, j) << "LL] = " << T2 << "{x" << j << ", y" << j << "};\n";
      }
      o << "    }\n    }\n";
    } else {
      for (int j = 0; j < D; ++j) o << "    tile[" << saddr(j) << "] = " << TT << "{x" << j << ", y" << j << "};\n";
      o << "    __syncthreads();\n    }\n";
    }
  }
  if (!dlast) {
    o << "    {\n";
    for (int i = 0; i < NPT; ++i) {
      o << "      const int l" << i << " = (threadIdx.x + " << i * T << ") * " << V << ";";
      if (f)
        o << " const cf u" << i << " = tile[l" << i << " ^ ((l" << i << " >> 4) & 15)], v" << i << " = tile[(l" << i
          << " + 1) ^ (((l" << i << " + 1) >> 4) & 15)]; const f4 b" << i << " = f4{u" << i << ".x, u" << i << ".y, v"
          << i << ".x, v" << i << ".y};\n";
      else if (ffm)
        o << " f4 b" << i << "; { const ffc2 e = tile[l" << i << " ^ ((l" << i << " >> 3) & 7)]; const cd d = cd{(double)e.x, "
          << "(double)e.y}; b" << i << " = *reinterpret_cast<const f4*>(&d); }\n";
      else
        o << " const f4 b" << i << " = *reinterpret_cast<const f4*>(&tile[l" << i << " ^ ((l" << i << " >> 3) & 7)]);\n";
    }
    for (int i = 0; i < NPT; ++i)
      o << "      *reinterpret_cast<f4*>(g + runoff[l" << i << " >> " << c << "] + (l" << i << " & " << ((1 << c) - 1)
        << ")) = b" << i << ";\n";
    o << "    }\n    __syncthreads();\n";
  }
  o << "  }\n";
  if (pf) o << "  asm volatile(\"cp.async.wait_group 0;\" ::: \"memory\");\n";
  o << "}\n";
}

// ------------------------------------------------------------------ pair-lane form (complex64)
// A pass planned with a lane bit P (FusedArgs::pbit, chosen by the planner as the
// tile bit the fewest non-diagonal gates touch) holds P as register bit 4 of
// every phase.  A thread's 32 amplitudes are then 16 pairs that differ only in P:
// X<j> = (x_j, x_{j|16}) and Y<j> = (y_j, y_{j|16}) in 64-bit registers, j < 16,
// and every op that does not mix the two halves of a pair (all ops not on P, and
// diagonal ops on P with per-lane coefficients) runs as two-lane FP32 code
// (fma.rn.f32x2 / mul.rn.f32x2): one instruction for two amplitudes.  The pairs
// never change between phases: the shared-memory tile holds one 16-byte unit per
// pair, (re_a, re_b | im_a, im_b) for the amplitudes a (P = 0) and b (P = 1),
// indexed by the tile index without P, so a phase boundary is one 16-byte store
// and load per pair.  The remaining ops (non-diagonal ops on P, dense two-qubit
// matrices) run as the scalar code on the unpacked halves.  Global memory keeps
// its interleaved layout: the direct first/last phase and the staged tile copies
// regroup the 16-byte accesses into pairs.
//
// Bank conflicts: a 16-byte access is served a quarter warp (8 lanes) per
// wavefront, which is conflict-free when the 8 lanes' units lie in 8 different
// 16-byte bank groups (unit index mod 8).  Lanes 0..7 vary the three lowest
// thread bits of the phase, so each phase boundary gets its own swizzle: unit u
// is stored at u ^ sum_k u_k v_k over the unit-index bits k >= 3, with the bank
// vectors v_k (3 bits) chosen so that the three lane bits of both the writing and
// the reading phase map to independent bank vectors.  The map is XOR-linear and
// leaves bits >= 3 unchanged, so a thread's address is its base XOR a constant.
struct PairSwz {
  int v[32] = {0};  // bank vector of unit-index bit k (k >= 3; bits 0..2 map to themselves)
  int vec(int k) const { return k < 3 ? (1 << k) : v[k]; }
  int apply(int u) const {
    int s = u;
    for (int k = 3; k < 31; ++k)
      if ((u >> k) & 1) s ^= v[k];
    return s;
  }
};

static bool indep3(int a, int b, int c) { return a && b && c && a != b && a != c && b != c && (a ^ b) != c; }

// bank vectors for the unit-index bits >= 3 satisfying every lane triple (each
// three bit positions whose bank vectors must be independent): the XOR-fold of the
// 3-bit digits (v_k = 1 << (k mod 3)) when it already does, else a backtracking
// search over the positions the triples use; the fold if nothing satisfies them
static PairSwz choose_swz(const std::vector<std::array<int, 3>>& triples, int nq) {
  PairSwz S;
  for (int k = 3; k < nq; ++k) S.v[k] = 1 << (k % 3);
  auto ok = [&](const PairSwz& T) {
    for (auto& t : triples)
      if (!indep3(T.vec(t[0]), T.vec(t[1]), T.vec(t[2]))) return false;
    return true;
  };
  if (ok(S)) return S;
  std::vector<int> pos;  // the positions >= 3 that a triple uses
  for (auto& t : triples)
    for (int k : t)
      if (k >= 3 && std::find(pos.begin(), pos.end(), k) == pos.end()) pos.push_back(k);
  std::sort(pos.begin(), pos.end());
  PairSwz T = S;
  std::vector<char> set(32, 0);
  for (int k = 0; k < 3; ++k) set[k] = 1;
  for (int k = 0; k < 32; ++k)
    if (std::find(pos.begin(), pos.end(), k) == pos.end()) set[k] = 1;
  // a triple is checked once all its positions are assigned
  auto consistent = [&]() {
    for (auto& t : triples)
      if (set[t[0]] && set[t[1]] && set[t[2]] && !indep3(T.vec(t[0]), T.vec(t[1]), T.vec(t[2]))) return false;
    return true;
  };
  long long budget = 2000000;
  std::function<bool(size_t)> rec = [&](size_t i) -> bool {
    if (i == pos.size()) return true;
    for (int v = 1; v < 8 && budget > 0; ++v, --budget) {
      T.v[pos[i]] = v;
      set[pos[i]] = 1;
      if (consistent() && rec(i + 1)) return true;
      set[pos[i]] = 0;
    }
    return false;
  };
  if (rec(0)) return T;
  return S;  // unsatisfiable (not expected): the fold, with bank conflicts
}

static void gen_kernel_pl(std::ostringstream& o, const FusedArgs<float>& a, const std::string& name) {
  const int M = a.M, c = a.c, NB = 5, P = a.pbit;
  const int T = 1 << (M - NB);
  const int NM = BT_FUSED_MAX_REALS_F;
  const int NP = a.nphase;
  const int NQ = M - 1;  // unit-index bits
  const char* mref = a.permem ? "cm" : "a.mat";
  o << "extern \"C\" __global__ void __launch_bounds__(" << T << ", " << bt_jit_min_blocks() << ") " << name
    << "(cf* __restrict__ psi, const JitArgsF<" << NM << "> a";
  if (a.permem) o << ", const float* __restrict__ mm, const i64 mstride";
  o << ") {\n  typedef float R;\n";
  if (NP == 0) {
    o << "}\n";
    return;
  }
  auto qpos = [&](int bit) { return bit < P ? bit : bit - 1; };
  const int cmask = (1 << c) - 1;
  const bool dfirst = direct_ok(a.ph[0], NB, M, true);
  const bool dlast = direct_ok(a.ph[NP - 1], NB, M, true);
  const bool staged_in = !dfirst, staged_out = !dlast;
  const bool use_smem = staged_in || staged_out || NP > 1;
  auto regmask_of = [&](const FPhase& ph) {
    uint32_t m = 0;
    for (int b = 0; b < NB; ++b) m |= 1u << ph.reg[b];
    return m;
  };
  // unit-index positions of a phase's thread bits, in threadIdx order
  auto tpos = [&](const FPhase& ph) {
    const uint32_t rm = regmask_of(ph);
    std::vector<int> v;
    for (int bit = 0; bit < M; ++bit)
      if (!((rm >> bit) & 1)) v.push_back(qpos(bit));
    return v;
  };
  // one swizzle for the whole pass, so that a phase writes its results to exactly
  // the units it read (in place, no barrier between its reads and its writes):
  // the lane bits of every phase that touches shared memory, and of the staged
  // copies, must have independent bank vectors under it
  std::vector<std::array<int, 3>> tr;
  for (int p = 0; p < NP; ++p) {
    const bool rd_direct = p == 0 && dfirst, wr_direct = p == NP - 1 && dlast;
    if (rd_direct && wr_direct) continue;
    auto t = tpos(a.ph[p]);
    tr.push_back({t[0], t[1], t[2]});
  }
  if ((staged_in || staged_out) && P != 0) tr.push_back({1, 2, 3});  // staged copies: lanes on unit bits 1..3
  const PairSwz swz1 = choose_swz(tr, NQ);
  std::vector<PairSwz> swz(NP + 1, swz1);
  auto thread_off = [&](const FPhase& ph) {  // global offset of the thread's non-register tile bits
    const uint32_t rm = regmask_of(ph);
    std::ostringstream e;
    e << "(i64)0";
    int nb = 0;
    for (int bit = 0; bit < M; ++bit)
      if (!((rm >> bit) & 1)) e << " | ((i64)((threadIdx.x >> " << nb++ << ") & 1) << " << a.tbits[bit] << ")";
    return e.str();
  };
  auto reg_off = [&](const FPhase& ph, int j) {  // global offset of register amplitude j (bit 4: the lane)
    int64_t v = 0;
    for (int b = 0; b < NB; ++b)
      if ((j >> b) & 1) v |= (int64_t)1 << a.tbits[ph.reg[b]];
    return v;
  };
  // swizzled unit index of a thread's bits at unit-index positions tp (threadIdx
  // order): the unit index itself with its bank bits (0..2) XORed by the parity of
  // its bits under each bank bit's mask; computed where a phase starts
  auto base_expr = [&](const std::vector<int>& tp, const PairSwz& S) {
    std::ostringstream q;
    q << "0";
    for (size_t i = 0; i < tp.size(); ++i) q << " | (((int)(threadIdx.x >> " << i << ") & 1) << " << tp[i] << ")";
    unsigned mask[3] = {0, 0, 0};
    for (int k = 3; k < 31; ++k)
      for (int r = 0; r < 3; ++r)
        if ((S.v[k] >> r) & 1) mask[r] |= 1u << k;
    std::ostringstream e;
    e << "[&]() { const int q = " << q.str() << "; return q";
    for (int r = 0; r < 3; ++r)
      if (mask[r]) e << " ^ ((__popc((unsigned)q & " << mask[r] << "u) & 1) << " << r << ")";
    e << "; }()";
    return e.str();
  };
  const int64_t pofs = (int64_t)1 << a.tbits[P];
  if (use_smem) o << "  extern __shared__ __align__(16) unsigned char smem_raw[];\n  pu* tile2 = reinterpret_cast<pu*>(smem_raw);\n";
  if (staged_in || staged_out) {
    o << "  i64* runoff = reinterpret_cast<i64*>(smem_raw + " << (8 << M) << ");\n";
    o << "  for (int r = threadIdx.x; r < " << (1 << (M - c)) << "; r += " << T << ") { i64 v = 0;";
    for (int b = 0; b < M - c; ++b) o << " v |= (i64)((r >> " << b << ") & 1) << " << a.tbits[c + b] << ";";
    o << " runoff[r] = v; }\n  __syncthreads();\n";
  }
  // per-thread swizzled bases of the staged copies (unit u = threadIdx.x + i T, or
  // twice that for a lane bit above 0) and of every phase's reads and writes
  const int csh = P == 0 ? 0 : 1;
  std::vector<int> tcopy;
  for (int i = 0; (1 << i) < T; ++i) tcopy.push_back(i + csh);
  if (dfirst) o << "  const i64 tf = " << thread_off(a.ph[0]) << ";\n";
  if (dlast) o << "  const i64 tl = " << thread_off(a.ph[NP - 1]) << ";\n";
  o << "  const i64 per = 1LL << a.lg_tiles, total = per * a.nmem;\n";
  o << "  auto tile_ptr = [&](i64 tid) -> cf* {\n";
  o << "    const i64 mem = a.member_lo + (tid >> a.lg_tiles);\n    u64 base = (u64)(tid & (per - 1));\n";
  for (int i = 0; i < M; ++i) {
    const int p = a.tbits[i];
    o << "    base = ((base >> " << p << ") << " << (p + 1) << ") | (base & " << fmt_u64((1ULL << p) - 1) << ");\n";
  }
  o << "    return psi + (mem << a.nbits) + base;\n  };\n";
  // global offset (from the tile's first amplitude) of tile index l
  auto goff = [&](const std::string& l) {
    return "runoff[(" + l + ") >> " + std::to_string(c) + "] + ((" + l + ") & " + std::to_string(cmask) + ")";
  };
  const int nruns = 1 << (M - c), run_bytes = 8 << c;
  const bool l2pf = l2_prefetch_on();
  if (l2pf) {
    o << "  const int pr = threadIdx.x;\n  i64 roff = 0;\n";
    for (int b = 0; b < M - c; ++b) o << "  roff |= (i64)((pr >> " << b << ") & 1) << " << a.tbits[c + b] << ";\n";
  }
  o << "  for (i64 tid = blockIdx.x; tid < total; tid += gridDim.x) {\n";
  o << "    cf* g = tile_ptr(tid);\n";
  if (a.permem) o << "    const R* cm = mm + (tid >> a.lg_tiles) * mstride;\n";
  if (l2pf) {
    o << "    if (tid + gridDim.x < total" << (T > nruns ? " && threadIdx.x < " + std::to_string(nruns) : std::string())
      << ") { const cf* gn = tile_ptr(tid + gridDim.x) + roff;";
    o << " asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], " << run_bytes << ";\" :: \"l\"(gn) : \"memory\");";
    if (T < nruns) {
      o << " for (int q = " << T << "; q < " << nruns << "; q += " << T << ") { i64 ro = 0;";
      for (int b = 0; b < M - c; ++b) o << " ro |= (i64)(((threadIdx.x + q) >> " << b << ") & 1) << " << a.tbits[c + b] << ";";
      o << " const cf* gq = tile_ptr(tid + gridDim.x) + ro; asm volatile(\"cp.async.bulk.prefetch.L2.global [%0], "
        << run_bytes << ";\" :: \"l\"(gq) : \"memory\"); }";
    }
    o << " }\n";
  }
  const int NU = 1 << NQ;  // pair units of the tile
  // tile index of pair unit u: u with a zero inserted at bit P
  auto expand = [&](const std::string& u) {
    return "(((" + u + ") >> " + std::to_string(P) + ") << " + std::to_string(P + 1) + ") | ((" + u + ") & " +
           std::to_string((1 << P) - 1) + ")";
  };
  if (staged_in) {
    const PairSwz& S = swz[0];
    o << "    {\n      const int cin = " << base_expr(tcopy, S) << ";\n";
    if (P == 0) {  // one 16-byte load is one pair (a, a+1)
      const int UPT = NU / T;
      for (int i = 0; i < UPT; ++i)
        o << "      const int u" << i << " = threadIdx.x + " << i * T << "; const f4 b" << i
          << " = *reinterpret_cast<const f4*>(g + " << goff("u" + std::to_string(i) + " << 1") << ");\n";
      for (int i = 0; i < UPT; ++i)
        o << "      tile2[cin ^ " << S.apply(i * T) << "] = pu{pk(b" << i << ".x, b" << i << ".z), pk(b" << i << ".y, b" << i
          << ".w)};\n";
    } else {  // two 16-byte loads (a, a+1) and (a|P, a|P+1) are two pairs
      const int H = NU / 2 / T;
      for (int i = 0; i < H; ++i) {
        o << "      const int u" << i << " = (threadIdx.x + " << i * T << ") << 1; const int l" << i << " = "
          << expand("u" + std::to_string(i)) << ";\n";
        o << "      const f4 va" << i << " = *reinterpret_cast<const f4*>(g + " << goff("l" + std::to_string(i))
          << "), vb" << i << " = *reinterpret_cast<const f4*>(g + "
          << goff("l" + std::to_string(i) + " | " + std::to_string(1 << P)) << ");\n";
      }
      for (int i = 0; i < H; ++i)
        o << "      tile2[cin ^ " << S.apply(2 * i * T) << "] = pu{pk(va" << i << ".x, vb" << i << ".x), pk(va" << i
          << ".y, vb" << i << ".y)}; tile2[cin ^ " << S.apply(2 * i * T + 1) << "] = pu{pk(va" << i << ".z, vb" << i
          << ".z), pk(va" << i << ".w, vb" << i << ".w)};\n";
    }
    o << "    }\n    __syncthreads();\n";
  }
  for (int p = 0; p < NP; ++p) {
    const FPhase& ph = a.ph[p];
    const bool rd_direct = p == 0 && dfirst, wr_direct = p == NP - 1 && dlast;
    // 16-byte global accesses: along the lane bit when it is tile bit 0, else along
    // tile bit 0 when it is a register bit (reg[0], the register bits ascend)
    const int gcase = P == 0 ? 0 : (ph.reg[0] == 0 ? 1 : 2);
    o << "    { // phase " << p << "\n";
    // the register units' offsets under a boundary's swizzle: XOR with the thread's
    // base in bits 0..2, an addition above them (the base has no register bits)
    auto uaddr = [&](const char* base, const PairSwz& S, int j) {
      int q = 0;
      for (int b = 0; b < 4; ++b)
        if ((j >> b) & 1) q |= 1 << qpos(ph.reg[b]);
      const int sw = S.apply(q), lo = sw & 7, hi = sw & ~7;
      std::string e = std::string("(") + base + (lo ? " ^ " + std::to_string(lo) : std::string()) + ")";
      return hi ? e + " + " + std::to_string(hi) : e;
    };
    if (!rd_direct || !wr_direct) o << "    const int sb = " << base_expr(tpos(ph), swz[p]) << ";\n";
    // ops that run as scalar code on the unpacked halves
    bool scalar = false;
    std::vector<std::string> packed_src(ph.nop);
    std::vector<char> is_packed(ph.nop, 0);
    for (int k = 0; k < ph.nop; ++k) {
      const FOp& op = a.op[ph.op0 + k];
      std::ostringstream po;
      if (op.type != FOP_G2 && emit_op_packed(po, op, NB, 4, mref)) {
        packed_src[k] = po.str();
        is_packed[k] = 1;
      } else {
        scalar = true;
      }
    }
    o << "    u64 ";
    for (int j = 0; j < 16; ++j) o << (j ? ", " : "") << "X" << j << ", Y" << j;
    o << ";\n";
    if (scalar) {
      o << "    R ";
      for (int j = 0; j < 32; ++j) o << (j ? ", " : "") << "x" << j << ", y" << j;
      o << ";\n";
    }
    if (rd_direct) {
      o << "    { const cf* gp = g + tf;\n";
      for (int j = 0; j < 16; ++j) {
        const int64_t r0 = reg_off(ph, j);
        if (gcase == 0)
          o << "    { const f4 v = *reinterpret_cast<const f4*>(gp + " << r0 << "LL); X" << j << " = pk(v.x, v.z); Y" << j
            << " = pk(v.y, v.w); }\n";
        else if (gcase == 1) {
          if (j & 1) continue;
          o << "    { const f4 v0 = *reinterpret_cast<const f4*>(gp + " << r0 << "LL), v1 = *reinterpret_cast<const f4*>(gp + "
            << (r0 + pofs) << "LL); X" << j << " = pk(v0.x, v1.x); Y" << j << " = pk(v0.y, v1.y); X" << (j | 1)
            << " = pk(v0.z, v1.z); Y" << (j | 1) << " = pk(v0.w, v1.w); }\n";
        } else
          o << "    { const cf va = gp[" << r0 << "LL], vb = gp[" << (r0 + pofs) << "LL]; X" << j << " = pk(va.x, vb.x); Y"
            << j << " = pk(va.y, vb.y); }\n";
      }
      o << "    }\n";
    } else {
      for (int j = 0; j < 16; ++j)
        o << "    { const pu v = tile2[" << uaddr("sb", swz[p], j) << "]; X" << j << " = v.x; Y" << j << " = v.y; }\n";
      // the tile's last shared-memory reads: the next tile may overwrite it once every warp is past them
      if (wr_direct) o << "    __syncthreads();\n";
    }
    auto unpack = [&]() {
      for (int j = 0; j < 16; ++j)
        o << "    x" << j << "=plo(X" << j << "); x" << (j | 16) << "=phi(X" << j << "); y" << j << "=plo(Y" << j << "); y"
          << (j | 16) << "=phi(Y" << j << ");\n";
    };
    auto pack = [&]() {
      for (int j = 0; j < 16; ++j)
        o << "    X" << j << "=pk(x" << j << ",x" << (j | 16) << "); Y" << j << "=pk(y" << j << ",y" << (j | 16) << ");\n";
    };
    for (int k = 0; k < ph.nop; ++k) {
      if (is_packed[k]) {
        o << packed_src[k];
        continue;
      }
      unpack();
      emit_op(o, a.op[ph.op0 + k], NB, mref);
      pack();
    }
    if (wr_direct) {
      o << "    { cf* gp = g + tl;\n";
      for (int j = 0; j < 16; ++j) {
        const int64_t r0 = reg_off(ph, j);
        if (gcase == 0)
          o << "    *reinterpret_cast<f4*>(gp + " << r0 << "LL) = f4{plo(X" << j << "), plo(Y" << j << "), phi(X" << j
            << "), phi(Y" << j << ")};\n";
        else if (gcase == 1) {
          if (j & 1) continue;
          o << "    *reinterpret_cast<f4*>(gp + " << r0 << "LL) = f4{plo(X" << j << "), plo(Y" << j << "), plo(X"
            << (j | 1) << "), plo(Y" << (j | 1) << ")};\n";
          o << "    *reinterpret_cast<f4*>(gp + " << (r0 + pofs) << "LL) = f4{phi(X" << j << "), phi(Y" << j << "), phi(X"
            << (j | 1) << "), phi(Y" << (j | 1) << ")};\n";
        } else
          o << "    gp[" << r0 << "LL] = cf{plo(X" << j << "), plo(Y" << j << ")}; gp[" << (r0 + pofs) << "LL] = cf{phi(X"
            << j << "), phi(Y" << j << ")};\n";
      }
      o << "    }\n    }\n";
    } else {
      for (int j = 0; j < 16; ++j)
        o << "    tile2[" << uaddr("sb", swz[p + 1], j) << "] = pu{X" << j << ", Y" << j << "};\n";
      o << "    __syncthreads();\n    }\n";
    }
  }
  if (staged_out) {
    const PairSwz& S = swz[NP];
    o << "    {\n      const int cout = " << base_expr(tcopy, S) << ";\n";
    if (P == 0) {
      const int UPT = NU / T;
      for (int i = 0; i < UPT; ++i)
        o << "      const int u" << i << " = threadIdx.x + " << i * T << "; const pu b" << i << " = tile2[cout ^ "
          << S.apply(i * T) << "];\n";
      for (int i = 0; i < UPT; ++i)
        o << "      *reinterpret_cast<f4*>(g + " << goff("u" + std::to_string(i) + " << 1") << ") = f4{plo(b" << i
          << ".x), plo(b" << i << ".y), phi(b" << i << ".x), phi(b" << i << ".y)};\n";
    } else {
      const int H = NU / 2 / T;
      for (int i = 0; i < H; ++i)
        o << "      const int u" << i << " = (threadIdx.x + " << i * T << ") << 1; const int l" << i << " = "
          << expand("u" + std::to_string(i)) << "; const pu va" << i << " = tile2[cout ^ " << S.apply(2 * i * T)
          << "], vb" << i << " = tile2[cout ^ " << S.apply(2 * i * T + 1) << "];\n";
      for (int i = 0; i < H; ++i) {
        o << "      *reinterpret_cast<f4*>(g + " << goff("l" + std::to_string(i)) << ") = f4{plo(va" << i << ".x), plo(va"
          << i << ".y), plo(vb" << i << ".x), plo(vb" << i << ".y)};\n";
        o << "      *reinterpret_cast<f4*>(g + " << goff("l" + std::to_string(i) + " | " + std::to_string(1 << P))
          << ") = f4{phi(va" << i << ".x), phi(va" << i << ".y), phi(vb" << i << ".x), phi(vb" << i << ".y)};\n";
      }
    }
    o << "    }\n    __syncthreads();\n";
  }
  o << "  }\n}\n";
}

// the kernel of one fused pass: the pair-lane form where the pass was planned with
// a lane bit (complex64), else the scalar / two-lane-per-phase form
template <typename R>
static void gen_pass(std::ostringstream& o, const FusedArgs<R>& a, int NB, const std::string& name) {
  if constexpr (sizeof(R) == 4) {
    if (a.pbit >= 0 && NB == 5) {
      gen_kernel_pl(o, a, name);
      return;
    }
  }
  gen_kernel<R>(o, a, NB, name);
}

// structure key: everything that shapes the code (not the matrix values)
template <typename R>
static std::string structure_key(const FusedArgs<R>& a) {
  std::ostringstream k;
  k << (sizeof(R) == 4 ? 'f' : 'd') << a.M << ':' << a.c << ':' << bt_jit_min_blocks() << ':'
    << (a.nphase ? (int)a.ph[0].nreg : 0) << ':' << (sizeof(R) == 4 && a.packed ? 'p' : 's') << ':'
    << (a.permem ? 'm' : 'k') << ':' << a.pbit << ':' << (ff_pass(a) ? 'F' : 'N') << ':';
  for (int i = 0; i < a.M; ++i) k << a.tbits[i] << ',';
  for (int p = 0; p < a.nphase; ++p) {
    const FPhase& ph = a.ph[p];
    k << '|';
    for (int b = 0; b < ph.nreg; ++b) k << (int)ph.reg[b] << '.';
    for (int oi = ph.op0; oi < ph.op0 + ph.nop; ++oi) {
      const FOp& op = a.op[oi];
      k << (int)op.type << (int)op.b0 << (int)op.b1 << '_' << (int)op.flags << (int)op.unit << '@' << op.moff << ';';
    }
  }
  return k.str();
}

// one NVRTC program (cubin) per compile batch; loaded as a CUDA library on first use
struct JitModule {
  std::vector<char> cubin;
  cudaLibrary_t lib = nullptr;
};
struct JitEntry {
  JitModule* mod = nullptr;
  std::string name;
  std::atomic<cudaKernel_t> kernel{nullptr};  // resolved at the first launch
  std::atomic<bool> attr_set[64] = {};         // shared-memory attribute set, per device
};
static std::mutex g_jit_mu;
static std::map<std::string, JitEntry*> g_jit_cache;

static uint64_t fnv1a(const std::string& s) {
  uint64_t h = 1469598103934665603ULL;
  for (unsigned char ch : s) h = (h ^ ch) * 1099511628211ULL;
  return h;
}

static std::string cache_dir() {
  const char* d = getenv("BTGPU_JIT_CACHE");
  std::string dir;
  if (d && *d) dir = d;
  else {
    const char* home = getenv("HOME");
    dir = std::string(home && *home ? home : "/tmp") + "/.cache/btgpu_jit";
  }
  std::string acc;
  for (size_t i = 0; i < dir.size(); ++i) {  // mkdir -p
    acc += dir[i];
    if (dir[i] == '/' || i + 1 == dir.size()) mkdir(acc.c_str(), 0755);
  }
  return dir;
}

static const char* kOpts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-default-device"};

// what besides the source decides a cubin: the compile options, the NVRTC and the
// driver versions (a cubin built by an older toolkit is not reused after an upgrade)
static const std::string& cache_salt() {
  static const std::string salt = [] {
    std::string k = "btk-cache-v2";
    for (const char* o : kOpts) k += std::string("|") + o;
    int ma = 0, mi = 0, drv = 0;
    if (Nvrtc* nv = nvrtc())
      if (nv->version) nv->version(&ma, &mi);
    cudaDriverGetVersion(&drv);
    k += "|nvrtc" + std::to_string(ma) + "." + std::to_string(mi) + "|driver" + std::to_string(drv);
    return k;
  }();
  return salt;
}

// compiles one source to a cubin (disk cache keyed by the source, the options and
// the NVRTC / driver versions); "" on success
static std::string compile_cubin(const std::string& code, std::vector<char>& cubin) {
  const std::string path = cache_dir() + "/btk_" + std::to_string(fnv1a(cache_salt() + "\n" + code)) + ".cubin";
  if (FILE* fd = fopen(path.c_str(), "rb")) {
    fseek(fd, 0, SEEK_END);
    long sz = ftell(fd);
    fseek(fd, 0, SEEK_SET);
    cubin.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = sz > 0 ? fread(cubin.data(), 1, (size_t)sz, fd) : 0;
    fclose(fd);
    if (sz > 0 && got == (size_t)sz) return "";
  }
  Nvrtc* nv = nvrtc();
  nvrtcProgram_t prog = nullptr;
  if (nv->create(&prog, code.c_str(), "bt_plan_jit.cu", 0, nullptr, nullptr)) return "nvrtcCreateProgram failed";
  if (nv->compile(prog, 3, kOpts)) {
    size_t ls = 0;
    nv->log_size(prog, &ls);
    std::string log(ls, '\0');
    nv->log(prog, &log[0]);
    nv->destroy(&prog);
    return "NVRTC compile of a plan failed: " + log.substr(0, 2000);
  }
  size_t cs = 0;
  nv->cubin_size(prog, &cs);
  cubin.resize(cs);
  nv->cubin(prog, cubin.data());
  nv->destroy(&prog);
  // a name no other process or thread writes: the pid and the thread's id
  const std::string tmp = path + ".tmp" + std::to_string((long long)getpid()) + "_" +
                          std::to_string(std::hash<std::thread::id>()(std::this_thread::get_id()));
  if (FILE* fd = fopen(tmp.c_str(), "wb")) {  // write-then-rename: concurrent processes never read a partial file
    fwrite(cubin.data(), 1, cubin.size(), fd);
    fclose(fd);
    rename(tmp.c_str(), path.c_str());
  }
  return "";
}

template <typename R>
static int jit_prepare_t(bt_ctx* ctx, std::vector<const FusedArgs<R>*>& passes, std::vector<void*>& out) {
  out.assign(passes.size(), nullptr);
  if (!nvrtc()) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "NVRTC is not available");
  std::vector<std::string> keys(passes.size());
  std::vector<std::string> order;                     // new structures in first-seen order
  std::map<std::string, const FusedArgs<R>*> first;
  for (size_t i = 0; i < passes.size(); ++i) keys[i] = structure_key(*passes[i]);
  if (const char* dump = getenv("BTGPU_JIT_DUMP")) {
    // inspection aid: the generated source of every fused pass of this compile,
    // kernel pass_<i> for the i-th fused pass (whether compiled now or cached)
    std::ostringstream src;
    src << kPrelude;
    for (size_t i = 0; i < passes.size(); ++i) {
      const FusedArgs<R>& pa = *passes[i];
      const int nreg = pa.nphase ? pa.ph[0].nreg : (sizeof(R) == 4 ? BT_TILE_RB_C64 : BT_TILE_RB_C128);
      src << "// pass " << i << ": M=" << pa.M << " threads=" << (1 << (pa.M - nreg)) << "\n";
      gen_pass<R>(src, pa, nreg, "pass_" + std::to_string(i));
    }
    if (FILE* fd = fopen(dump, "w")) {
      const std::string t = src.str();
      fwrite(t.data(), 1, t.size(), fd);
      fclose(fd);
    }
    // BTGPU_JIT_DUMP_ONLY: write the source without building it (the passes keep
    // the generic kernel)
    if (getenv("BTGPU_JIT_DUMP_ONLY")) return BT_OK;
  }
  {
    std::lock_guard<std::mutex> lk(g_jit_mu);  // held for lookups and inserts, not for compiling
    for (size_t i = 0; i < passes.size(); ++i)
      if (!g_jit_cache.count(keys[i]) && !first.count(keys[i])) {
        first[keys[i]] = passes[i];
        order.push_back(keys[i]);
      }
  }
  if (!order.empty()) {
    // batches of kernels compiled concurrently (NVRTC programs are independent)
    int hw = (int)std::thread::hardware_concurrency();
    if (hw < 1) hw = 1;
    const int nb = (int)std::min<size_t>(order.size(), (size_t)std::min(hw, 32));
    std::vector<std::string> srcs(nb), errs(nb);
    std::vector<std::vector<std::string>> names(nb), bkeys(nb);
    for (int b = 0; b < nb; ++b) {
      std::ostringstream src;
      src << kPrelude;
      for (size_t i = b; i < order.size(); i += nb) {
        const std::string nm = "btk_" + std::to_string(i);
        const FusedArgs<R>& pa = *first[order[i]];
        gen_pass<R>(src, pa, pa.nphase ? pa.ph[0].nreg : (sizeof(R) == 4 ? BT_TILE_RB_C64 : BT_TILE_RB_C128), nm);
        names[b].push_back(nm);
        bkeys[b].push_back(order[i]);
      }
      srcs[b] = src.str();
    }
    std::vector<JitModule*> mods(nb);
    std::vector<std::thread> th;
    for (int b = 0; b < nb; ++b) {
      mods[b] = new JitModule();
      th.emplace_back([&, b] { errs[b] = compile_cubin(srcs[b], mods[b]->cubin); });
    }
    for (auto& t : th) t.join();
    for (int b = 0; b < nb; ++b)
      if (!errs[b].empty()) {
        for (auto* m : mods) delete m;
        return bt_fail(ctx, BT_ERR_DEVICE, errs[b]);
      }
    std::lock_guard<std::mutex> lk(g_jit_mu);
    for (int b = 0; b < nb; ++b)
      for (size_t i = 0; i < names[b].size(); ++i) {
        if (g_jit_cache.count(bkeys[b][i])) continue;  // compiled meanwhile by another plan
        JitEntry* je = new JitEntry();
        je->mod = mods[b];
        je->name = names[b][i];
        g_jit_cache[bkeys[b][i]] = je;
      }
  }
  std::lock_guard<std::mutex> lk(g_jit_mu);
  for (size_t i = 0; i < passes.size(); ++i) out[i] = g_jit_cache[keys[i]];
  return BT_OK;
}

int bt_jit_prepare_f(bt_ctx* ctx, std::vector<const FusedArgs<float>*>& passes, std::vector<void*>& out) {
  return jit_prepare_t<float>(ctx, passes, out);
}
int bt_jit_prepare_d(bt_ctx* ctx, std::vector<const FusedArgs<double>*>& passes, std::vector<void*>& out) {
  return jit_prepare_t<double>(ctx, passes, out);
}

// the generated kernels take (psi, JitArgs{member_lo, nmem, nbits, lg_tiles, mat[]})
template <typename R>
struct JitArgsHost {
  int64_t member_lo, nmem;
  int nbits, lg_tiles;
  R mat[sizeof(R) == 4 ? BT_FUSED_MAX_REALS_F : BT_FUSED_MAX_REALS_D];
};

// mm / mstride: the per-member table of a kernel compiled with a.permem (row m for
// member member_lo + m), else unused
template <typename R>
static int jit_launch_t(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<R>& a, const void* mm = nullptr,
                        int64_t mstride = 0) {
  JitEntry* je = (JitEntry*)entry;
  typedef typename CT<R>::T C2;
  const int M = a.M;
  const size_t smem = (sizeof(C2) << M) + sizeof(int64_t) * (1 << (M - a.c));
  cudaKernel_t kern = je->kernel.load(std::memory_order_acquire);
  if (!kern) {  // first launch: load the batch's cubin and resolve the kernel
    std::lock_guard<std::mutex> lk(g_jit_mu);
    kern = je->kernel.load(std::memory_order_acquire);
    if (!kern) {
      if (!je->mod->lib) {
        cudaError_t e = cudaLibraryLoadData(&je->mod->lib, je->mod->cubin.data(), nullptr, nullptr, 0, nullptr,
                                            nullptr, 0);
        if (e != cudaSuccess) return bt_cuda_check(ctx, e, "cudaLibraryLoadData of a plan");
      }
      cudaError_t e = cudaLibraryGetKernel(&kern, je->mod->lib, je->name.c_str());
      if (e != cudaSuccess) return bt_cuda_check(ctx, e, "cudaLibraryGetKernel");
      je->kernel.store(kern, std::memory_order_release);
    }
  }
  if (ctx->device < 64 && !je->attr_set[ctx->device].load(std::memory_order_acquire)) {
    cudaError_t e = cudaKernelSetAttributeForDevice(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem,
                                                    ctx->device);
    if (e != cudaSuccess) return bt_cuda_check(ctx, e, "jit kernel smem attribute");
    je->attr_set[ctx->device].store(true, std::memory_order_release);
  }
  static thread_local JitArgsHost<R> h;
  h.member_lo = a.member_lo;
  h.nmem = a.nmem;
  h.nbits = a.nbits;
  h.lg_tiles = a.lg_tiles;
  memcpy(h.mat, a.mat, sizeof(h.mat));
  if (ff_pass(a)) {
    // float-float kernels read each coefficient as the floats (h, l) packed in its slot
    for (size_t i = 0; i < sizeof(h.mat) / sizeof(R); ++i) {
      const double d = (double)a.mat[i];
      const float hi = (float)d, lo = (float)(d - (double)hi);
      float pair[2] = {hi, lo};
      memcpy(reinterpret_cast<char*>(h.mat) + i * 8, pair, 8);
    }
  }
  void* args[] = {&psi, &h, &mm, &mstride};
  int64_t total = (1LL << a.lg_tiles) * a.nmem;
  int64_t grid = (int64_t)ctx->sm_count * bt_jit_min_blocks() * 4;
  if (grid > total) grid = total;
  const unsigned threads = 1u << (a.M - (a.nphase ? a.ph[0].nreg : (sizeof(R) == 4 ? BT_TILE_RB_C64 : BT_TILE_RB_C128)));
  cudaError_t e = cudaLaunchKernel((const void*)kern, dim3((unsigned)grid), dim3(threads), args, smem,
                                   ctx->stream);
  ctx->launches++;
  return bt_cuda_check(ctx, e, "jit pass launch");
}

int bt_jit_launch_f(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<float>& a) {
  return jit_launch_t<float>(ctx, entry, psi, a);
}
int bt_jit_launch_members_f(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<float>& a, const float* mm,
                            int64_t mstride) {
  return jit_launch_t<float>(ctx, entry, psi, a, mm, mstride);
}
int bt_jit_launch_members_d(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<double>& a, const double* mm,
                            int64_t mstride) {
  return jit_launch_t<double>(ctx, entry, psi, a, mm, mstride);
}
int bt_jit_launch_d(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<double>& a) {
  return jit_launch_t<double>(ctx, entry, psi, a);
}
