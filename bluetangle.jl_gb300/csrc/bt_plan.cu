// Circuit plans: the gate-fusion pass of the circuit compiler (the role of the
// reference's compile/get_layers, BlueTangle.jl src/ops.jl:278-329, :421-445) and
// their execution.
//
// A plan is a list of dense gates over the bits of a state (n bits for a state
// vector; 2n for a density matrix, where a gate U on qubit q becomes U on row bit
// n-q and conj(U) on column bit 2n-q, and a Kraus sum becomes one superoperator
// on both).  compile() groups the gates into passes:
//   * fused passes: a set of at most M bits (always containing the lowest c
//     bits) and every gate that acts inside it and is not ordered behind a gate
//     left out; gates inside a pass are grouped into register phases of at most
//     RB bits.  Each fused pass is one launch of its specialised kernel (bt_jit.cu)
//     or of the generic k_fused (bt_fused_impl.cuh).
//   * sweep passes: gates of more than two bits, or with controls that do not fit
//     a two-bit matrix, run as one k_gate sweep (bt_gate.cu).
// Gates are only reordered past gates on disjoint bits, so the plan applies the
// same linear map as the gates in their given order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "bt_fused.cuh"
#include "bt_jit.cuh"
#include "bt_tc.cuh"

struct PGate {
  int k = 0;
  int bits[2 * BT_MAX_K] = {0};  // bits[0] = most significant bit of the matrix index
  uint64_t cmask = 0;
  std::vector<double> m;  // row-major interleaved 2^k x 2^k
  int ku = 0, fold_nc = 0;  // the caller's gate size and the controls folded into m
  // updated in place (bt_plan_set_matrices / bt_plan_set_variable): encoded in
  // forms whose structure does not depend on the entries, so later updates never
  // force a recompile
  bool var = false;
  uint64_t allbits() const {
    uint64_t b = cmask;
    for (int i = 0; i < k; ++i) b |= 1ULL << bits[i];
    return b;
  }
};

struct PPass {
  int kind = 0;  // 0 fused, 1 sweep
  int gate = -1;
  int ngates = 0;
  std::vector<unsigned char> args;  // FusedArgs<float> or <double>, bytes
  std::vector<int> op_gate;         // gate of each op, and its register bits before encoding
  std::vector<uint8_t> op_b0, op_b1;
  // per-member form (bt_plan_run_members): the pass compiled to read its entries
  // from a per-member table, and its specialised kernel
  std::vector<unsigned char> pm_args;
  void* pm_jit = nullptr;
  // tensor-core form (compile mode 3): index of the pass's first phase block in
  // the plan's device table of block images, or -1
  int tc_block = -1;
};

struct bt_plan {
  bt_ctx* ctx = nullptr;
  int n = 0, repr = 0, prec = 0, nbits = 0;
  std::vector<PGate> gates;
  std::vector<PPass> passes;
  std::vector<std::pair<int, int>> adds;  // per bt_plan_add_*: first gate and count (0: not updatable)
  bool compiled = false;
  int compile_mode = 0;
  int64_t nphases = 0;
  // tuning (bt_plan_set_tuning; 0 / -1: the library defaults)
  int tune_max_ops = 0, tune_rb = 0, tune_packed = -1, tune_m = 0;
  // specialised kernel of each pass (bt_jit.cu), published when compiled; the
  // background compiler of a tiered plan writes them while runs read them
  std::unique_ptr<std::atomic<void*>[]> jit;
  std::atomic<int64_t> njit{0};
  std::thread jit_thread;
  // device table of per-member entries (bt_plan_run_members), reused pass by pass
  void* d_pm = nullptr;
  size_t d_pm_bytes = 0;
  int d_pm_device = -1;
  // device table of the tensor-core phase blocks (compile mode 3)
  float* d_tc = nullptr;
  int d_tc_device = -1;
};

// reals of the matrices that bt_plan_set_matrices reads for these add indices
int bt_plan_gate_dims(const bt_plan* p, const int64_t* idx, int count, size_t* reals);

static void join_jit(bt_plan* p) {
  if (p->jit_thread.joinable()) p->jit_thread.join();
}

// compiles the fused passes' kernels and publishes them pass by pass
static void specialise(bt_plan* p) {
  const bool c64 = p->prec == BT_PREC_C64;
  std::vector<size_t> idx;
  std::vector<void*> ent;
  int rc;
  if (c64) {
    std::vector<const FusedArgs<float>*> v;
    for (size_t i = 0; i < p->passes.size(); ++i)
      if (p->passes[i].kind == 0) {
        v.push_back(reinterpret_cast<const FusedArgs<float>*>(p->passes[i].args.data()));
        idx.push_back(i);
      }
    rc = bt_jit_prepare_f(p->ctx, v, ent);
  } else {
    std::vector<const FusedArgs<double>*> v;
    for (size_t i = 0; i < p->passes.size(); ++i)
      if (p->passes[i].kind == 0) {
        v.push_back(reinterpret_cast<const FusedArgs<double>*>(p->passes[i].args.data()));
        idx.push_back(i);
      }
    rc = bt_jit_prepare_d(p->ctx, v, ent);
  }
  if (rc != BT_OK) return;
  int64_t n = 0;
  for (size_t j = 0; j < idx.size(); ++j) {
    p->jit[idx[j]].store(ent[j], std::memory_order_release);
    n += ent[j] != nullptr;
  }
  p->njit.store(n);
}

static int popc(uint64_t x) { return __builtin_popcountll(x); }

static void kron_ctrl(int k, const double* u_rm, int nc, std::vector<double>& out) {
  // controlled-U on (controls..., targets...): identity except the block where all controls are 1
  const int d = 1 << k, D = 1 << (k + nc);
  out.assign(2 * D * D, 0.0);
  for (int i = 0; i < D; ++i) out[2 * (i * D + i)] = 1.0;
  const int off = D - d;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      out[2 * ((off + r) * D + off + c)] = u_rm[2 * (r * d + c)];
      out[2 * ((off + r) * D + off + c) + 1] = u_rm[2 * (r * d + c) + 1];
    }
}

static void add_gate(bt_plan* p, int k, const int* bits, const double* rm, int nc, const int* cbits) {
  PGate g;
  g.ku = k;
  if (nc > 0 && k + nc <= 2) {
    g.fold_nc = nc;
    // fold the control into a dense two-bit matrix so the gate can join a tile
    kron_ctrl(k, rm, nc, g.m);
    g.k = k + nc;
    for (int i = 0; i < nc; ++i) g.bits[i] = cbits[i];
    for (int i = 0; i < k; ++i) g.bits[nc + i] = bits[i];
  } else {
    g.k = k;
    for (int i = 0; i < k; ++i) g.bits[i] = bits[i];
    for (int i = 0; i < nc; ++i) g.cmask |= 1ULL << cbits[i];
    g.m.assign(rm, rm + 2 * (1 << k) * (1 << k));
  }
  p->gates.push_back(std::move(g));
  p->compiled = false;
}

static bool eligible(const PGate& g) { return g.cmask == 0 && g.k <= 2; }

// classify a 2^k x 2^k matrix: 2 diagonal, 1 monomial (one non-zero per row and
// column), 0 general
static int classify(const PGate& g, int* perm) {
  const int d = 1 << g.k;
  bool diag = true, mono = true;
  for (int r = 0; r < d; ++r) {
    int nz = 0;
    for (int c = 0; c < d; ++c) {
      bool z = g.m[2 * (r * d + c)] == 0.0 && g.m[2 * (r * d + c) + 1] == 0.0;
      if (!z) {
        ++nz;
        if (c != r) diag = false;
        perm[r] = c;
      }
    }
    if (nz != 1) mono = false;
  }
  if (mono) {
    int seen = 0;
    for (int r = 0; r < d; ++r) seen |= 1 << perm[r];
    if (seen != (1 << d) - 1) mono = false;
  }
  return diag ? 2 : (mono ? 1 : 0);
}

// a monomial matrix whose non-zero entries are all exactly 1
static bool classify_unit(const PGate& g) {
  const int d = 1 << g.k;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const double re = g.m[2 * (r * d + c)], im = g.m[2 * (r * d + c) + 1];
      if (!(re == 0 && im == 0) && !(re == 1 && im == 0)) return false;
    }
  return true;
}

// Scalar factors taken out of one-qubit ops (BTGPU_PLAN_FACTOR=0 turns it off):
// diag(d0, d1) = d0 diag(1, d1/d0) touches half the amplitudes, and a real
// matrix with entries of one magnitude (H) is that magnitude times an add/sub
// butterfly.  The factors of a pass multiply into one scalar that is folded
// back into one op of the pass (encode_pass), so the pass applies the same map.
static bool factor_on() {
  static const bool v = [] {
    const char* e = getenv("BTGPU_PLAN_FACTOR");
    return !(e && *e == '0');
  }();
  return v;
}

// classifies gate g and writes its op type and matrix entries at mat[0..nre)
// in double; fac receives the complex scalar taken out of the op (1 if none).
// (o.b0/o.b1 hold the register bits of the gate's first/second bit on entry)
static void encode_op(const PGate& g, FOp& o, double* mat, int& nre, double* fac, bool factor) {
  factor = factor && !g.var;
  int perm[4] = {0, 1, 2, 3};
  const int cls = classify(g, perm);
  const double* m = g.m.data();
  int w = 0;
  fac[0] = 1.0, fac[1] = 0.0;
  if (g.k == 1) {
    // m = [m00r m00i m01r m01i m10r m10i m11r m11i]
    const bool real = m[1] == 0 && m[3] == 0 && m[5] == 0 && m[7] == 0;
    const double a0 = fabs(m[0]);
    const double n0 = m[0] * m[0] + m[1] * m[1], n1 = m[6] * m[6] + m[7] * m[7];
    if (cls == 2 && factor && (n0 != 0 || n1 != 0)) {
      // the larger entry factored out: d1 / d0 on the bit-1 half (or d0 / d1 on
      // the bit-0 half); exact -1, i, -i become sign flips and swaps
      const bool lo = n1 > 4 * n0;  // clearly larger only: unitary diagonals always factor d0
      const double* f = lo ? m + 6 : m;   // factored entry
      const double* e = lo ? m : m + 6;   // the other
      const double n = lo ? n1 : n0;
      const double qr = (e[0] * f[0] + e[1] * f[1]) / n, qi = (e[1] * f[0] - e[0] * f[1]) / n;
      o.type = FOP_DH;
      o.flags = lo ? 1 : 0;
      o.unit = (qr == -1 && qi == 0) ? 2 : (qr == 0 && qi == 1) ? 3 : (qr == 0 && qi == -1) ? 4 : 0;
      mat[w++] = qr;
      mat[w++] = qi;
      fac[0] = f[0], fac[1] = f[1];
    } else if (cls == 2) {
      o.type = FOP_D1;
      mat[w++] = m[0];
      mat[w++] = m[1];
      mat[w++] = m[6];
      mat[w++] = m[7];
    } else if (cls == 1) {  // anti-diagonal
      o.type = FOP_X1;
      o.unit = (m[2] == 1 && m[3] == 0 && m[4] == 1 && m[5] == 0) ? 1 : 0;
      mat[w++] = m[2];
      mat[w++] = m[3];
      mat[w++] = m[4];
      mat[w++] = m[5];
    } else if (real && factor && a0 != 0 && fabs(m[2]) == a0 && fabs(m[4]) == a0 && fabs(m[6]) == a0) {
      // m00 * [[1, s01], [s10, s11]], signs relative to m00
      o.type = FOP_HB;
      o.flags = (uint8_t)(((m[2] < 0) != (m[0] < 0)) | (((m[4] < 0) != (m[0] < 0)) << 1) |
                          (((m[6] < 0) != (m[0] < 0)) << 2));
      fac[0] = m[0];
    } else if (real && factor && m[0] != 0 && fabs(m[6]) == a0 && a0 >= fabs(m[2]) && a0 >= fabs(m[4])) {
      // [[a, b], [c, d]] with |d| = |a| >= |b|: a [[1, b/a], [c/a, d/a = +-1]]
      o.type = FOP_RN;
      o.flags = (uint8_t)((m[6] < 0) != (m[0] < 0));
      mat[w++] = m[2] / m[0];
      mat[w++] = m[4] / m[0];
      fac[0] = m[0];
    } else if (real && factor && m[2] != 0 && fabs(m[4]) == fabs(m[2]) && fabs(m[2]) >= a0 &&
               fabs(m[2]) >= fabs(m[6])) {
      // |c| = |b| >= |a|: b [[a/b, 1], [c/b = +-1, d/b]]
      o.type = FOP_RN;
      o.flags = (uint8_t)(2 | ((m[4] < 0) != (m[2] < 0)));
      mat[w++] = m[0] / m[2];
      mat[w++] = m[6] / m[2];
      fac[0] = m[2];
    } else if (real) {
      o.type = FOP_R1;
      mat[w++] = m[0];
      mat[w++] = m[2];
      mat[w++] = m[4];
      mat[w++] = m[6];
    } else if (m[0] == m[6] && m[1] == 0 && m[7] == 0 && m[2] == 0 && m[4] == 0 && m[3] == m[5]) {
      // [[a, ib], [ib, a]]
      if (factor && (m[0] != 0 || m[3] != 0)) {
        o.type = FOP_RXN;
        if (fabs(m[0]) >= fabs(m[3])) {  // a [[1, i b/a], [i b/a, 1]]
          mat[w++] = m[3] / m[0];
          fac[0] = m[0];
        } else {  // ib [[-i a/b, 1], [1, -i a/b]]
          o.flags = 2;
          mat[w++] = m[0] / m[3];
          fac[0] = 0, fac[1] = m[3];
        }
      } else {
        o.type = FOP_RX1;
        mat[w++] = m[0];
        mat[w++] = m[3];
      }
    } else {
      o.type = FOP_G1;
      for (int e = 0; e < 8; ++e) mat[w++] = m[e];
    }
  } else if (cls == 1 && classify_unit(g) && perm[0] == 0 && perm[1] == 1 && perm[2] == 3 && perm[3] == 2) {
    o.type = FOP_CX;  // control = matrix MSB (register b0), target = LSB (b1)
  } else if (cls == 1 && classify_unit(g) && perm[0] == 0 && perm[1] == 3 && perm[2] == 2 && perm[3] == 1) {
    o.type = FOP_CX;  // control = matrix LSB, target = MSB
    const uint8_t t = o.b0;
    o.b0 = o.b1;
    o.b1 = t;
  } else if (cls == 1 && classify_unit(g) && perm[0] == 0 && perm[1] == 2 && perm[2] == 1 && perm[3] == 3) {
    o.type = FOP_SW;
  } else if (cls == 2) {
    o.type = FOP_D2;
    for (int r = 0; r < 4; ++r) {
      mat[w++] = g.m[2 * (r * 4 + r)];
      mat[w++] = g.m[2 * (r * 4 + r) + 1];
    }
  } else if (cls == 1) {
    o.type = FOP_P2;
    o.flags = (uint8_t)(perm[0] | (perm[1] << 2) | (perm[2] << 4) | (perm[3] << 6));
    bool unit = true;
    for (int r = 0; r < 4; ++r) {
      double pr = g.m[2 * (r * 4 + perm[r])], pi = g.m[2 * (r * 4 + perm[r]) + 1];
      if (pr != 1.0 || pi != 0.0) unit = false;
      mat[w++] = pr;
      mat[w++] = pi;
    }
    o.unit = unit ? 1 : 0;
  } else {
    o.type = FOP_G2;
    for (int e = 0; e < 32; ++e) mat[w++] = g.m[e];
  }
  nre = w;
}

// Encodes the ops of a fused pass (kept: their gates; ob0/ob1: their register
// bits) with the scalar factors folded into one op: a general op (complex
// entries scaled), a real op when the scalar is real, else one factored
// diagonal / butterfly turned back into its full form.  update: the pass
// exists and only its matrices are rewritten; false when an op's structure
// (type, bits, flags) would change, which needs a recompile.
template <typename R>
static bool encode_pass(bt_plan* p, const std::vector<int>& kept, const std::vector<uint8_t>& ob0,
                        const std::vector<uint8_t>& ob1, FusedArgs<R>& a, bool update, bool factor = true) {
  const int nop = (int)kept.size();
  std::vector<FOp> ops(nop);
  std::vector<double> mats((size_t)nop * 32);
  std::vector<int> nre(nop);
  factor = factor && factor_on();
  double tr = 1.0, ti = 0.0;  // product of the factors
  for (int i = 0; i < nop; ++i) {
    FOp& o = ops[i];
    memset(&o, 0, sizeof(o));
    o.b0 = ob0[i];
    o.b1 = ob1[i];
    double f[2];
    encode_op(p->gates[kept[i]], o, &mats[(size_t)i * 32], nre[i], f, factor);
    const double r = tr * f[0] - ti * f[1];
    ti = tr * f[1] + ti * f[0];
    tr = r;
  }
  // the factored ops grow amplitudes by at most the inverse of the scalar: keep
  // it well inside the complex64 range, else encode the pass without factors
  const double mag = sqrt(tr * tr + ti * ti);
  if (factor && !(mag > 1e-18 && mag < 1e18)) return encode_pass<R>(p, kept, ob0, ob1, a, update, false);
  if (tr != 1.0 || ti != 0.0) {
    const bool real = ti == 0;
    int t = -1, mode = 0;
    auto pick = [&](int m, auto&& ok) {
      for (int i = 0; i < nop && t < 0; ++i)
        if (ok(ops[i])) t = i, mode = m;
    };
    // in order of the arithmetic the fold adds: none, then the cheapest expansion
    pick(1, [](const FOp& o) {
      return o.type == FOP_G1 || o.type == FOP_G2 || o.type == FOP_D1 || o.type == FOP_D2 ||
             ((o.type == FOP_P2 || o.type == FOP_X1) && !o.unit);
    });
    if (real) pick(2, [](const FOp& o) { return o.type == FOP_R1; });
    pick(3, [](const FOp& o) { return o.type == FOP_DH; });
    if (real) pick(4, [](const FOp& o) { return o.type == FOP_RN || o.type == FOP_HB; });
    pick(5, [](const FOp& o) { return o.type == FOP_RXN || o.type == FOP_RN || o.type == FOP_HB; });
    if (t < 0) return encode_pass<R>(p, kept, ob0, ob1, a, update, false);
    double* m = &mats[(size_t)t * 32];
    FOp& o = ops[t];
    // the factored op as a real or complex 2x2 [[e00, e01], [e10, e11]] (RN, HB, RXN)
    auto full = [&](double (&e)[8]) {
      for (double& x : e) x = 0;
      if (o.type == FOP_HB) {
        e[0] = 1, e[2] = (o.flags & 1) ? -1 : 1, e[4] = (o.flags & 2) ? -1 : 1, e[6] = (o.flags & 4) ? -1 : 1;
      } else if (o.type == FOP_RN) {
        const double sg = (o.flags & 1) ? -1 : 1;
        if (o.flags & 2) e[0] = m[0], e[2] = 1, e[4] = sg, e[6] = m[1];
        else e[0] = 1, e[2] = m[0], e[4] = m[1], e[6] = sg;
      } else {  // RXN
        if (o.flags & 2) e[1] = -m[0], e[2] = 1, e[4] = 1, e[7] = -m[0];
        else e[0] = 1, e[3] = m[0], e[5] = m[0], e[6] = 1;
      }
    };
    if (mode == 1) {
      for (int e = 0; e + 1 < nre[t]; e += 2) {
        const double r = m[e] * tr - m[e + 1] * ti;
        m[e + 1] = m[e] * ti + m[e + 1] * tr;
        m[e] = r;
      }
    } else if (mode == 2) {
      for (int e = 0; e < nre[t]; ++e) m[e] *= tr;
    } else if (mode == 3) {  // diag(s, s q) or diag(s q, s)
      const double qr = m[0], qi = m[1], sr = tr * qr - ti * qi, si = tr * qi + ti * qr;
      const bool lo = o.flags & 1;
      o.type = FOP_D1;
      o.unit = 0;
      o.flags = 0;
      m[0] = lo ? sr : tr, m[1] = lo ? si : ti, m[2] = lo ? tr : sr, m[3] = lo ? ti : si;
      nre[t] = 4;
    } else {
      double e[8];
      full(e);
      o.flags = 0;
      o.unit = 0;
      if (mode == 4) {  // real scalar: R1
        o.type = FOP_R1;
        m[0] = e[0] * tr, m[1] = e[2] * tr, m[2] = e[4] * tr, m[3] = e[6] * tr;
        nre[t] = 4;
      } else {  // G1
        o.type = FOP_G1;
        for (int k = 0; k < 8; k += 2) m[k] = e[k] * tr - e[k + 1] * ti, m[k + 1] = e[k] * ti + e[k + 1] * tr;
        nre[t] = 8;
      }
    }
  }
  if (update) {
    // a structure that changed needs a recompile; its gates take the
    // value-independent forms from then on
    bool same = true;
    for (int i = 0; i < nop; ++i) {
      const FOp& o = a.op[i];
      if (ops[i].type != o.type || ops[i].b0 != o.b0 || ops[i].b1 != o.b1 || ops[i].flags != o.flags ||
          ops[i].unit != o.unit) {
        p->gates[kept[i]].var = true;
        same = false;
      }
    }
    if (!same) return false;
  }
  int w = 0;
  for (int i = 0; i < nop; ++i) {
    if (update) {
      w = a.op[i].moff;
    } else {
      ops[i].moff = (uint16_t)w;
      a.op[i] = ops[i];
    }
    for (int e = 0; e < nre[i]; ++e) a.mat[w++] = (R)mats[(size_t)i * 32 + e];
  }
  return true;
}

// register-phase windows (on unless BTGPU_PLAN_PHASE_WINDOWS=0): each register
// phase of a pass may also take NB consecutive tile bits where they hold more gates
// than the set grown in gate order (33-qubit brickwork: 90 phases instead of 117,
// 0.844 -> 0.786 s per circuit on a GB300)
static bool phase_windows_on() {
  static const bool v = [] {
    const char* e = getenv("BTGPU_PLAN_PHASE_WINDOWS");
    return !(e && *e == '0');
  }();
  return v;
}

// width of the beam search over register-phase sequences (BTGPU_PLAN_PHASE_BEAM;
// 1: the greedy choice).  Ranked by phases plus staged first/last phases, width 8
// plans the 33-qubit brickwork into 92 phases with one staged end instead of 96
// with six: 0.787 -> 0.744 s per circuit on a GB300.
static int phase_beam() {
  static const int v = [] {
    const char* e = getenv("BTGPU_PLAN_PHASE_BEAM");
    const int x = e && *e ? atoi(e) : 8;
    return x < 1 ? 1 : (x > 64 ? 64 : x);
  }();
  return v;
}

// Pair-lane form (complex64 specialised passes, bt_jit.cu): one tile bit of the
// pass, the lane bit, is a register bit of every phase, so each thread holds its
// amplitudes as pairs that differ only in that bit and applies every op that
// does not mix the two halves with two-lane FP32 instructions (fma.rn.f32x2) on
// the pair.  The lane bit is the tile bit the fewest non-diagonal gates of the
// pass touch (on the window planner's passes usually one of the low bits that no
// gate of the pass acts on); a phase then chooses NB - 1 register bits.  Off
// unless BTGPU_JIT_LANES=1: on a GB300 the form cuts the instructions of a dense
// 28-qubit pass by 26% (911M -> 673M: the FP32 instructions halve) but is slower
// on 21 of the 23 passes of the 28-qubit brickwork (23.3 vs 21.8 ms per circuit;
// 33 qubits: 0.828 vs 0.787 s): the FMA pipe time stays the same, each op's
// coefficients must be broadcast into register pairs, and at 16 warps per SM and
// the 128-register cap the halved instruction-level parallelism of a phase shows
// as dependency and scoreboard stalls (issue 48% active against 70%).
static bool lanes_on() {
  static const bool v = [] {
    const char* e = getenv("BTGPU_JIT_LANES");
    return e && *e == '1';
  }();
  return v;
}

template <typename R>
static bool build_fused(bt_plan* p, const std::vector<int>& take, uint64_t tilemask, int M, int NB, int c,
                        std::vector<int>& kept, FusedArgs<R>& a, int64_t* nph, std::vector<uint8_t>& ob0,
                        std::vector<uint8_t>& ob1, bool lanes = false) {
  memset(&a, 0, sizeof(a));
  a.nbits = p->nbits;
  a.M = M;
  a.c = c;
  a.pbit = -1;
  int nb = 0, local[64];
  for (int b = 0; b < p->nbits; ++b) {
    local[b] = -1;
    if ((tilemask >> b) & 1) {
      a.tbits[nb] = b;
      local[b] = nb++;
    }
  }
  a.lg_tiles = p->nbits - M;
  int pbit = -1;
  if (lanes && NB == 5 && M >= NB + 1) {
    int cnt[32] = {0};
    for (int gi : take) {
      const PGate& g = p->gates[gi];
      int perm[4] = {0, 1, 2, 3};
      if (!g.var && classify(g, perm) == 2) continue;  // diagonal: per-lane coefficients
      for (int i = 0; i < g.k; ++i) cnt[local[g.bits[i]]]++;
    }
    pbit = 0;
    for (int b = 1; b < M; ++b)
      if (cnt[b] < cnt[pbit]) pbit = b;
    a.pbit = pbit;
  }
  const uint32_t pmask = pbit >= 0 ? 1u << pbit : 0u;
  const int NF = NB - (pbit >= 0 ? 1 : 0);  // register bits a phase chooses
  const int maxreals = sizeof(R) == 4 ? BT_FUSED_MAX_REALS_F : BT_FUSED_MAX_REALS_D;
  // register phases over the pass's gates with blocking, in order.  A phase with
  // register set rs takes the gates it can in order (a gate left out blocks its
  // bits): rs grown gate by gate up to NF bits, or a window of NF consecutive free
  // tile bits.  The sequence of phases is chosen by a beam search over those
  // candidates that keeps the `beam` partial sequences with the fewest gates left
  // (width 1: the greedy choice of the candidate taking the most gates).
  auto scan = [&](const std::vector<int>& rem, int nop0, int nreal0, uint32_t rs, bool fixed, std::vector<int>& ph,
                  std::vector<int>& rest, uint32_t& regs, int& nr) {
    regs = fixed ? rs : 0;
    nr = nreal0;
    uint32_t blocked = 0;
    ph.clear();
    rest.clear();
    for (int gi : rem) {
      const PGate& g = p->gates[gi];
      uint32_t lb = 0;
      for (int i = 0; i < g.k; ++i) lb |= 1u << local[g.bits[i]];
      const uint32_t lf = lb & ~pmask;  // the lane bit is in every phase
      const int need = g.k == 1 ? 8 : 32;
      if ((lb & blocked) || (fixed ? (lf & ~rs) != 0 : popc(regs | lf) > NF) ||
          nop0 + (int)ph.size() + 1 > BT_FUSED_MAX_OPS || nr + need > maxreals) {
        blocked |= lb;
        rest.push_back(gi);
        continue;
      }
      if (!fixed) regs |= lf;
      ph.push_back(gi);
      nr += need;
    }
  };
  // the tile bits a phase may choose, ascending (all but the lane bit)
  std::vector<int> free_bits;
  for (int b = 0; b < M; ++b)
    if (b != pbit) free_bits.push_back(b);
  struct Seq {
    std::vector<int> rem;
    std::vector<uint32_t> regs;             // per phase
    std::vector<std::vector<int>> gates;    // per phase
    int nop = 0, nreal = 0;
  };
  // whether the specialised kernel can move a phase with register set regs
  // straight between HBM and registers (as bt_jit.cu decides it: the warp's lanes
  // on the lowest non-register tile bits touch at most twice the 128-byte lines
  // their bytes need); a first or last phase that cannot is staged through shared
  // memory, which costs about one more phase
  const bool f32 = sizeof(R) == 4;
  auto direct = [&](uint32_t regs) {
    const uint32_t all = pbit >= 0 ? (regs | pmask) : regs;
    const bool pair = f32 && (all & 1);
    const int bytes = pair ? 16 : (f32 ? 8 : 16), linebits = f32 ? 4 : 3;
    int lanes = 0, outside = 0;
    for (int b = 0; b < M && lanes < 5; ++b)
      if (!((all >> b) & 1)) {
        outside += b >= linebits;
        ++lanes;
      }
    return (1 << outside) <= 2 * std::max(1, 32 * bytes / 128);
  };
  auto cost = [&](const Seq& q) {
    if (q.regs.empty()) return 0;
    return (int)q.regs.size() + (direct(q.regs.front()) ? 0 : 1) + (direct(q.regs.back()) ? 0 : 1);
  };
  const int beam = phase_beam();
  std::vector<Seq> cur(1), complete;
  cur[0].rem = take;
  Seq best;
  for (int depth = 0; depth < BT_FUSED_MAX_PHASES && !cur.empty(); ++depth) {
    // a sequence still open needs at least one more phase
    if (!complete.empty()) {
      int bc = 1 << 30;
      for (const Seq& q : complete) bc = std::min(bc, cost(q));
      if (bc <= depth + 1) break;
    }
    std::vector<Seq> next;
    for (const Seq& sq : cur) {
      std::vector<uint32_t> cands = {0u};
      std::vector<char> fixed = {0};
      if (phase_windows_on())
        for (int s0 = 0; s0 + NF <= (int)free_bits.size(); ++s0) {
          uint32_t w = 0;
          for (int i = 0; i < NF; ++i) w |= 1u << free_bits[s0 + i];
          cands.push_back(w);
          fixed.push_back(1);
        }
      // candidates in order, the one taking the most gates first (ties: earlier)
      std::vector<Seq> kids;
      std::vector<uint32_t> seen;
      for (size_t ci = 0; ci < cands.size(); ++ci) {
        Seq k;
        std::vector<int> ph;
        uint32_t regs = 0;
        int nr = 0;
        scan(sq.rem, sq.nop, sq.nreal, cands[ci], fixed[ci] != 0, ph, k.rem, regs, nr);
        if (ph.empty()) continue;
        // pad the register set to NF bits with the highest unused free tile bits
        for (int i = (int)free_bits.size() - 1; i >= 0 && popc(regs) < NF; --i) regs |= 1u << free_bits[i];
        if (std::find(seen.begin(), seen.end(), regs) != seen.end()) continue;
        seen.push_back(regs);
        k.regs = sq.regs;
        k.regs.push_back(regs);
        k.gates = sq.gates;
        k.gates.push_back(ph);
        k.nop = sq.nop + (int)ph.size();
        k.nreal = nr;
        kids.push_back(std::move(k));
      }
      std::stable_sort(kids.begin(), kids.end(),
                       [](const Seq& x, const Seq& y) { return x.rem.size() < y.rem.size(); });
      for (size_t i = 0; i < kids.size() && (int)i < beam; ++i) next.push_back(std::move(kids[i]));
    }
    if (next.empty()) break;
    std::stable_sort(next.begin(), next.end(), [&](const Seq& x, const Seq& y) {
      if (x.rem.size() != y.rem.size()) return x.rem.size() < y.rem.size();
      return direct(x.regs.front()) && !direct(y.regs.front());
    });
    if ((int)next.size() > beam) next.resize(beam);
    cur.clear();
    for (Seq& q : next) {
      if (q.rem.empty()) complete.push_back(std::move(q));
      else cur.push_back(std::move(q));
    }
    if (beam == 1 && !complete.empty()) break;  // the greedy sequence
  }
  if (complete.empty() && !cur.empty()) complete.push_back(cur[0]);  // phase cap reached
  if (!complete.empty()) {
    best = complete[0];
    for (const Seq& q : complete)
      if (cost(q) < cost(best)) best = q;
  }
  int nop = 0, nreal = 0;
  kept.clear();
  for (size_t q = 0; q < best.regs.size(); ++q) {
    const uint32_t regs = best.regs[q];
    const std::vector<int>& ph = best.gates[q];
    for (int gi : ph) nreal += p->gates[gi].k == 1 ? 8 : 32;
    FPhase& P = a.ph[a.nphase++];
    int rb = 0, regidx[32];
    for (int b = 0; b < M; ++b)
      if ((regs >> b) & 1) {
        regidx[b] = rb;
        P.reg[rb++] = (uint8_t)b;
      }
    if (pbit >= 0) {  // the lane: register bit NB - 1
      regidx[pbit] = rb;
      P.reg[rb++] = (uint8_t)pbit;
    }
    P.nreg = (uint8_t)NB;
    P.op0 = (uint16_t)nop;
    P.nop = (uint16_t)ph.size();
    for (int gi : ph) {
      const PGate& g = p->gates[gi];
      FOp& o = a.op[nop++];
      o.moff = (uint16_t)(nreal - (g.k == 1 ? 8 : 32));  // provisional; rewritten below
      o.b0 = (uint8_t)regidx[local[g.bits[0]]];
      o.b1 = g.k == 2 ? (uint8_t)regidx[local[g.bits[1]]] : 0;
      kept.push_back(gi);
    }
  }
  // write matrices compactly in op order
  ob0.clear();
  ob1.clear();
  for (int i = 0; i < nop; ++i) {
    ob0.push_back(a.op[i].b0);
    ob1.push_back(a.op[i].b1);
  }
  encode_pass<R>(p, kept, ob0, ob1, a, false);
  *nph = a.nphase;
  return !kept.empty();
}

extern "C" {

int bt_plan_create(bt_ctx* ctx, int n, int repr, int prec, bt_plan** out) {
  // ctx may be NULL: planning and specialisation need no device (errors then go to
  // the thread's bt_last_error(NULL)); running needs a state, which carries a ctx
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "NULL argument");
  if (repr != BT_REPR_SV && repr != BT_REPR_DM) return bt_fail(ctx, BT_ERR_BAD_ARG, "repr must be SV or DM");
  if (prec != BT_PREC_C128 && prec != BT_PREC_C64) return bt_fail(ctx, BT_ERR_BAD_ARG, "prec must be C128 or C64");
  if (n < 1 || n > (repr == BT_REPR_DM ? 17 : 34)) return bt_fail(ctx, BT_ERR_BAD_ARG, "qubit count out of range");
  bt_plan* p = new bt_plan();
  p->ctx = ctx;
  p->n = n;
  p->repr = repr;
  p->prec = prec;
  p->nbits = repr == BT_REPR_DM ? 2 * n : n;
  *out = p;
  return BT_OK;
}

int bt_plan_free(bt_plan* p) {
  if (p) join_jit(p);
  if (p && p->d_pm) {
    cudaSetDevice(p->d_pm_device);
    cudaFree(p->d_pm);
  }
  if (p && p->d_tc) {
    cudaSetDevice(p->d_tc_device);
    cudaFree(p->d_tc);
  }
  delete p;
  return BT_OK;
}

int bt_plan_add_matrix(bt_plan* p, int k, const int32_t* qubits, const double* mat, int nctrl, const int32_t* ctrls) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  bt_ctx* ctx = p->ctx;
  if (k < 1 || k > BT_MAX_K || !qubits || !mat) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad gate (1 <= k <= 5)");
  if (nctrl < 0 || (nctrl && !ctrls)) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad control list");
  uint64_t seen = 0;
  for (int i = 0; i < k + nctrl; ++i) {
    int q = i < k ? qubits[i] : ctrls[i - k];
    if (q < 1 || q > p->n) return bt_fail(ctx, BT_ERR_BAD_ARG, "N must be larger than qubits");
    if (seen & (1ULL << q)) return bt_fail(ctx, BT_ERR_BAD_ARG, "qubits and controls must differ");
    seen |= 1ULL << q;
  }
  const int d = 1 << k;
  std::vector<double> rm(2 * d * d);
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      rm[2 * (r * d + c)] = mat[2 * (r + c * d)];
      rm[2 * (r * d + c) + 1] = mat[2 * (r + c * d) + 1];
    }
  int bits[BT_MAX_K], cb[64];
  const int n = p->n;
  for (int i = 0; i < k; ++i) bits[i] = n - qubits[i];
  for (int i = 0; i < nctrl; ++i) cb[i] = n - ctrls[i];
  const int first = (int)p->gates.size();
  add_gate(p, k, bits, rm.data(), nctrl, cb);
  if (p->repr == BT_REPR_DM) {
    for (int i = 0; i < d * d; ++i) rm[2 * i + 1] = -rm[2 * i + 1];
    for (int i = 0; i < k; ++i) bits[i] = 2 * n - qubits[i];
    for (int i = 0; i < nctrl; ++i) cb[i] = 2 * n - ctrls[i];
    add_gate(p, k, bits, rm.data(), nctrl, cb);
  }
  p->adds.push_back({first, (int)p->gates.size() - first});
  return BT_OK;
}

}  // extern "C"

// rho <- sum_i K_i rho K_i^dagger as one 2k-bit superoperator gate on (row bits,
// column bits); K column-major interleaved
static void add_superop(bt_plan* p, int k, const int32_t* qubits, int nk, const double* kraus) {
  const int n = p->n, d = 1 << k, dd = d * d;
  std::vector<double> sup(2 * dd * dd, 0.0);
  for (int i = 0; i < nk; ++i) {
    const double* K = kraus + (size_t)i * 2 * dd;  // column-major
    for (int ir = 0; ir < d; ++ir)
      for (int ic = 0; ic < d; ++ic)
        for (int jr = 0; jr < d; ++jr)
          for (int jc = 0; jc < d; ++jc) {
            double ar = K[2 * (ir + jr * d)], ai = K[2 * (ir + jr * d) + 1];
            double br = K[2 * (ic + jc * d)], bi = -K[2 * (ic + jc * d) + 1];
            int r = ir * d + ic, c = jr * d + jc;
            sup[2 * (r * dd + c)] += ar * br - ai * bi;
            sup[2 * (r * dd + c) + 1] += ar * bi + ai * br;
          }
  }
  int bits[4];
  for (int i = 0; i < k; ++i) {
    bits[i] = n - qubits[i];
    bits[k + i] = 2 * n - qubits[i];
  }
  add_gate(p, 2 * k, bits, sup.data(), 0, nullptr);
}

// K_{i*m + j} = A_i (x) B_j for nk = m*m two-qubit operators (column-major
// interleaved 4x4)?  Recovers A (first qubit) and B (second qubit) as
// column-major 2x2 sets; false unless every product matches within 1e-14
// relative.  The split of a common scale between A and B does not change the
// channel.
static bool factor_kron_pairs(int nk, const double* kraus, std::vector<double>& A, int& na, std::vector<double>& B,
                              int& nb) {
  int m = 1;
  while (m * m < nk) ++m;
  if (m * m != nk || m < 2) return false;
  auto get = [&](int i, int r, int c, double& re, double& im) {
    re = kraus[(size_t)i * 32 + 2 * (r + 4 * c)];
    im = kraus[(size_t)i * 32 + 2 * (r + 4 * c) + 1];
  };
  // the largest entry of K_0 = A_0 (x) B_0 fixes A_0[a*, b*] = 1
  int p = 0, q = 0;
  double best = -1, mx = 0;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double re, im;
      get(0, r, c, re, im);
      const double v = re * re + im * im;
      if (v > best) best = v, p = r, q = c;
    }
  for (int i = 0; i < nk; ++i)
    for (int e = 0; e < 32; ++e) mx = std::max(mx, std::fabs(kraus[(size_t)i * 32 + e]));
  if (!(best > 0)) return false;
  const int as = p >> 1, rs = p & 1, bs = q >> 1, cs = q & 1;
  double b00r, b00i;
  get(0, p, q, b00r, b00i);  // B_0[r*, c*]
  const double den = b00r * b00r + b00i * b00i;
  A.assign((size_t)m * 8, 0.0);
  B.assign((size_t)m * 8, 0.0);
  for (int j = 0; j < m; ++j)  // B_j = block (a*, b*) of K_j
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) {
        double re, im;
        get(j, 2 * as + r, 2 * bs + c, re, im);
        B[(size_t)j * 8 + 2 * (r + 2 * c)] = re;
        B[(size_t)j * 8 + 2 * (r + 2 * c) + 1] = im;
      }
  for (int i = 0; i < m; ++i)  // A_i[a, b] = K_{i*m}[2a + r*, 2b + c*] / B_0[r*, c*]
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        double re, im;
        get(i * m, 2 * a + rs, 2 * b + cs, re, im);
        A[(size_t)i * 8 + 2 * (a + 2 * b)] = (re * b00r + im * b00i) / den;
        A[(size_t)i * 8 + 2 * (a + 2 * b) + 1] = (im * b00r - re * b00i) / den;
      }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j)
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
          const double* a = &A[(size_t)i * 8 + 2 * ((r >> 1) + 2 * (c >> 1))];
          const double* bb = &B[(size_t)j * 8 + 2 * ((r & 1) + 2 * (c & 1))];
          const double pr = a[0] * bb[0] - a[1] * bb[1], pi = a[0] * bb[1] + a[1] * bb[0];
          double re, im;
          get(i * m + j, r, c, re, im);
          if (std::fabs(pr - re) > 1e-14 * mx || std::fabs(pi - im) > 1e-14 * mx) return false;
        }
  na = nb = m;
  return true;
}

extern "C" {

int bt_plan_add_kraus_sum(bt_plan* p, int k, const int32_t* qubits, int nk, const double* kraus) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  bt_ctx* ctx = p->ctx;
  if (p->repr != BT_REPR_DM) return bt_fail(ctx, BT_ERR_BAD_ARG, "a Kraus sum needs a density-matrix plan");
  if (k < 1 || k > 2 || !qubits || nk < 1 || !kraus) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad channel (k <= 2)");
  const int n = p->n, d = 1 << k, dd = d * d;
  for (int i = 0; i < k; ++i)
    if (qubits[i] < 1 || qubits[i] > n) return bt_fail(ctx, BT_ERR_BAD_ARG, "N must be larger than qubits");
  if (k == 2 && qubits[0] == qubits[1]) return bt_fail(ctx, BT_ERR_BAD_ARG, "qubits must differ");
  p->adds.push_back({(int)p->gates.size(), 0});  // a channel's matrices are not updatable
  // a two-qubit set of products A_i (x) B_j over every (i, j) -- the reference's
  // two-qubit named channels (src/noise.jl:126) -- is the channel A on the first
  // qubit after B on the second: two one-qubit superoperators, which fused passes
  // hold, instead of one 4-bit superoperator applied as its own sweep
  std::vector<double> A, B;
  int na = 0, nb = 0;
  if (k == 2 && factor_kron_pairs(nk, kraus, A, na, B, nb)) {
    add_superop(p, 1, &qubits[1], nb, B.data());
    add_superop(p, 1, &qubits[0], na, A.data());
    return BT_OK;
  }
  add_superop(p, k, qubits, nk, kraus);
  (void)dd;
  return BT_OK;
}

}  // extern "C"

template <typename R>
static bool update_pass(bt_plan* p, PPass& ps, const std::vector<char>& touched) {
  FusedArgs<R>& a = *reinterpret_cast<FusedArgs<R>*>(ps.args.data());
  bool any = false;
  for (int gi : ps.op_gate) any |= touched[gi] != 0;
  // the whole pass is re-encoded: the folded scalar depends on every op's factor
  return !any || encode_pass<R>(p, ps.op_gate, ps.op_b0, ps.op_b1, a, true);
}

extern "C" {

}  // extern "C"

// Writes the matrices of these adds (column-major, back to back, in the size each
// was added with) into their gates: the column pass of a density-matrix gate takes
// conj(U), folded controls are re-folded.  The gates become variable; touched
// marks them.
static int assign_matrices(bt_plan* p, int count, const int64_t* add_index, const double* mats,
                           std::vector<char>& touched) {
  bt_ctx* ctx = p->ctx;
  if (count < 0 || (count > 0 && (!add_index || !mats))) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad update arrays");
  touched.assign(p->gates.size(), 0);
  size_t off = 0;
  for (int i = 0; i < count; ++i) {
    const int64_t ai = add_index[i];
    if (ai < 0 || ai >= (int64_t)p->adds.size()) return bt_fail(ctx, BT_ERR_BAD_ARG, "add index out of range");
    const int first = p->adds[ai].first, cnt = p->adds[ai].second;
    if (cnt == 0) return bt_fail(ctx, BT_ERR_BAD_ARG, "a Kraus sum cannot be updated");
    const int ku = p->gates[first].ku, d = 1 << ku;
    std::vector<double> rm(2 * d * d);
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        rm[2 * (r * d + c)] = mats[off + 2 * (r + c * d)];
        rm[2 * (r * d + c) + 1] = mats[off + 2 * (r + c * d) + 1];
      }
    off += 2 * (size_t)d * d;
    for (int j = 0; j < cnt; ++j) {
      PGate& g = p->gates[first + j];
      if (j == 1)  // the column pass of a density-matrix gate applies conj(U)
        for (int e = 0; e < d * d; ++e) rm[2 * e + 1] = -rm[2 * e + 1];
      if (g.fold_nc > 0) kron_ctrl(ku, rm.data(), g.fold_nc, g.m);
      else g.m = rm;
      g.var = true;
      touched[first + j] = 1;
    }
  }
  return BT_OK;
}

extern "C" {

int bt_plan_set_matrices(bt_plan* p, int count, const int64_t* add_index, const double* mats) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  std::vector<char> touched;
  int rc = assign_matrices(p, count, add_index, mats, touched);
  if (rc) return rc;
  if (!p->compiled) return BT_OK;
  if (p->compile_mode == 3) {  // the phase blocks are products of the gates: rebuilt at the next run
    p->compiled = false;
    return BT_OK;
  }
  for (auto& ps : p->passes) {
    if (ps.kind != 0) continue;
    const bool ok = p->prec == BT_PREC_C64 ? update_pass<float>(p, ps, touched) : update_pass<double>(p, ps, touched);
    if (!ok) {  // a gate changed its structural class: recompile at the next run
      p->compiled = false;
      break;
    }
  }
  return BT_OK;
}

int bt_plan_set_variable(bt_plan* p, int count, const int64_t* add_index) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  if (count < 0 || (count > 0 && !add_index)) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "bad index array");
  for (int i = 0; i < count; ++i) {
    const int64_t ai = add_index[i];
    if (ai < 0 || ai >= (int64_t)p->adds.size()) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "add index out of range");
    const int first = p->adds[ai].first, cnt = p->adds[ai].second;
    for (int j = 0; j < cnt; ++j) {
      if (!p->gates[first + j].var) p->compiled = false;
      p->gates[first + j].var = true;
    }
  }
  return BT_OK;
}

// Gates a fused pass with tile bit set Q takes from the remaining ones, in order;
// a gate left out blocks its bits for the gates after it (the plan applies the
// same map as the gates in their given order).  Q grows gate by gate up to M bits
// (fixed = false) or is given (fixed = true).
static void absorb(const bt_plan* p, const std::vector<int>& rem, uint64_t& Q, int M, int max_ops, bool fixed,
                   std::vector<int>& take) {
  uint64_t blocked = 0;
  take.clear();
  for (int gi : rem) {
    const PGate& g = p->gates[gi];
    const uint64_t b = g.allbits();
    if (!eligible(g) || (b & blocked) || (fixed ? (b & ~Q) != 0 : popc(Q | b) > M)) {
      blocked |= b;
      // nothing more fits once every bit of a full set is blocked
      if ((fixed || popc(Q) == M) && (Q & ~blocked) == 0) break;
      continue;
    }
    Q |= b;
    take.push_back(gi);
    if ((int)take.size() >= max_ops) break;
  }
}

// window candidates for the tile bits (BTGPU_PLAN_WINDOWS=0 turns them off)
static bool windows_on() {
  static const bool v = [] {
    const char* e = getenv("BTGPU_PLAN_WINDOWS");
    return !(e && *e == '0');
  }();
  return v;
}

// Tile bits of the next fused pass: the set grown in gate order, or, where it
// takes more gates, the lowest c bits with a window of M - c consecutive bits.
// On nearest-neighbour circuits a window follows the light cone of its qubits
// through many layers, where the grown set stops at the first layer's gate that
// does not fit (33-qubit brickwork of depth 30: 29 passes instead of 63).
static void select_bits(const bt_plan* p, const std::vector<int>& rem, uint64_t lowmask, int M, int c, int max_ops,
                        uint64_t& Q, std::vector<int>& take) {
  Q = lowmask;
  absorb(p, rem, Q, M, max_ops, false, take);
  const int w = M - c;
  if (!windows_on() || w <= 0 || p->nbits <= M) return;
  std::vector<int> t;
  for (int s = c; s + w <= p->nbits; ++s) {
    uint64_t W = lowmask | (((1ULL << w) - 1) << s);
    absorb(p, rem, W, M, max_ops, true, t);
    if (t.size() > take.size()) {
      take.swap(t);
      Q = W;
    }
  }
}

// Tensor-core form (compile mode 3): each register phase of a fused pass of
// 2^13-amplitude tiles becomes one dense 32 x 32 block, the product of the phase's
// gates on its 5 register bits (complex128, in order), stored as its TF32 MMA
// operand image (bt_tc.cu) in a device table of the plan
static void phase_block(const bt_plan* p, const FusedArgs<float>& a, const std::vector<int>& op_gate, int ph,
                        std::vector<double>& u) {
  const FPhase& P = a.ph[ph];
  int regidx[64];
  for (int b = 0; b < 64; ++b) regidx[b] = -1;
  for (int b = 0; b < 5; ++b) regidx[a.tbits[P.reg[b]]] = b;  // global bit -> register bit
  u.assign(2 * 32 * 32, 0.0);
  for (int j = 0; j < 32; ++j) u[2 * (j * 32 + j)] = 1.0;
  std::vector<double> nu(u.size());
  for (int oi = P.op0; oi < P.op0 + P.nop; ++oi) {
    const PGate& g = p->gates[op_gate[oi]];
    const int k = g.k, d = 1 << k;
    int rb[2];
    uint32_t gm = 0;
    for (int i = 0; i < k; ++i) {
      rb[i] = regidx[g.bits[i]];
      gm |= 1u << rb[i];
    }
    nu = u;
    for (int col = 0; col < 32; ++col)
      for (int x = 0; x < 32; ++x) {
        if (x & gm) continue;
        int idx[4];
        for (int sidx = 0; sidx < d; ++sidx) {
          int y = x;
          for (int i = 0; i < k; ++i)
            if ((sidx >> (k - 1 - i)) & 1) y |= 1 << rb[i];
          idx[sidx] = y;
        }
        for (int r = 0; r < d; ++r) {
          double re = 0, im = 0;
          for (int sidx = 0; sidx < d; ++sidx) {
            const double mr = g.m[2 * (r * d + sidx)], mi = g.m[2 * (r * d + sidx) + 1];
            const double vr = u[2 * (idx[sidx] * 32 + col)], vi = u[2 * (idx[sidx] * 32 + col) + 1];
            re += mr * vr - mi * vi;
            im += mr * vi + mi * vr;
          }
          nu[2 * (idx[r] * 32 + col)] = re;
          nu[2 * (idx[r] * 32 + col) + 1] = im;
        }
      }
    u.swap(nu);
  }
}

static int build_tc_blocks(bt_plan* p) {
  std::vector<float> img;
  std::vector<double> u;
  int nblk = 0;
  for (auto& ps : p->passes) {
    ps.tc_block = -1;
    if (ps.kind != 0) continue;
    const FusedArgs<float>& a = *reinterpret_cast<const FusedArgs<float>*>(ps.args.data());
    if (a.M != 13 || a.c != BT_TILE_LOW_C64 || a.nphase < 1 || a.ph[0].nreg != 5) continue;
    ps.tc_block = nblk;
    for (int ph = 0; ph < a.nphase; ++ph) {
      phase_block(p, a, ps.op_gate, ph, u);
      img.resize((size_t)(nblk + 1) * 8192);
      bt_tc_block_image(u.data(), img.data() + (size_t)nblk * 8192);
      ++nblk;
    }
  }
  if (p->d_tc) {
    cudaSetDevice(p->d_tc_device);
    cudaFree(p->d_tc);
    p->d_tc = nullptr;
  }
  if (!nblk) return BT_OK;
  if (!p->ctx) return bt_fail(nullptr, BT_ERR_BAD_ARG, "tensor-core plans need a context (device memory)");
  bt_ctx* ctx = p->ctx;
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!rc) rc = bt_cuda_check(ctx, cudaMalloc((void**)&p->d_tc, img.size() * sizeof(float)), "tensor-core block table");
  if (!rc)
    rc = bt_cuda_check(ctx, cudaMemcpy(p->d_tc, img.data(), img.size() * sizeof(float), cudaMemcpyHostToDevice),
                       "tensor-core block table upload");
  p->d_tc_device = ctx->device;
  return rc;
}

int bt_plan_compile(bt_plan* p, int mode) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  if (mode < 0 || mode > 3) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "compile mode must be 0, 1, 2 or 3");
  if (mode == 3 && (p->prec != BT_PREC_C64 || p->repr != BT_REPR_SV))
    return bt_fail(p->ctx, BT_ERR_UNSUPPORTED, "tensor-core plans (mode 3) are complex64 state-vector plans");
  join_jit(p);  // a background compile reads the passes about to be rebuilt
  p->compile_mode = mode;
  p->passes.clear();
  p->nphases = 0;
  const bool c64 = p->prec == BT_PREC_C64;
  // register bits per thread: a tuned width only where every pass gets its
  // specialised kernel before the first run (the generic kernel has one width)
  const int rb_tuned = c64 ? (p->tune_rb ? p->tune_rb : bt_tile_rb(true)) : BT_TILE_RB_C128;
  const int NB = mode == 3 ? BT_TILE_RB_C64
                           : ((mode == 0 && bt_jit_available()) ? rb_tuned : (c64 ? BT_TILE_RB_C64 : BT_TILE_RB_C128));
  const int packed = p->tune_packed >= 0 ? p->tune_packed : (int)bt_jit_packed_default();
  // the tile covers the whole state when the state is smaller than the default
  // tile, down to 2^(M - NB) = 32 threads per CTA; a tuned smaller tile spreads a
  // small state over more CTAs (more passes, each on more SMs)
  const int Mdef = c64 ? BT_TILE_M_C64 : BT_TILE_M_C128;
  const int M = std::min(p->tune_m ? std::min(p->tune_m, Mdef) : Mdef, p->nbits);
  const int c = c64 ? BT_TILE_LOW_C64 : BT_TILE_LOW_C128;
  const bool fuse = (mode == 0 || mode == 2 || mode == 3) && M >= NB + 5;
  // specialised kernels compile in time superlinear in their length: bound the
  // ops of a pass when they will be specialised
  const int max_ops = bt_jit_available() ? (p->tune_max_ops ? p->tune_max_ops : bt_jit_max_ops()) : BT_FUSED_MAX_OPS;
  std::vector<int> rem(p->gates.size());
  for (size_t i = 0; i < rem.size(); ++i) rem[i] = (int)i;
  const uint64_t lowmask = (1ULL << c) - 1;
  while (!rem.empty()) {
    const PGate& g0 = p->gates[rem[0]];
    if (!fuse || !eligible(g0)) {
      PPass ps;
      ps.kind = 1;
      ps.gate = rem[0];
      ps.ngates = 1;
      p->passes.push_back(std::move(ps));
      rem.erase(rem.begin());
      continue;
    }
    uint64_t Q = 0;
    std::vector<int> take;
    select_bits(p, rem, lowmask, M, c, max_ops, Q, take);
    for (int b = 0; b < p->nbits && popc(Q) < M; ++b) Q |= 1ULL << b;  // pad with the lowest free bits
    std::vector<int> kept;
    PPass ps;
    ps.kind = 0;
    int64_t nph = 0;
    if (c64) {
      ps.args.resize(sizeof(FusedArgs<float>));
      // pair-lane code where every pass gets a specialised kernel of 5 register bits
      const bool lanes = mode == 0 && bt_jit_available() && NB == 5 && lanes_on();
      build_fused<float>(p, take, Q, M, NB, c, kept, *reinterpret_cast<FusedArgs<float>*>(ps.args.data()), &nph,
                         ps.op_b0, ps.op_b1, lanes);
      // two-lane code where the pass has no dense two-qubit op: a dense 4x4 costs as
      // much either way and its packed form compiles several times slower
      FusedArgs<float>& fa = *reinterpret_cast<FusedArgs<float>*>(ps.args.data());
      bool dense2 = false;
      for (int oi = 0; oi < (int)kept.size(); ++oi) dense2 |= fa.op[oi].type == FOP_G2;
      fa.packed = packed && !dense2;
    } else {
      ps.args.resize(sizeof(FusedArgs<double>));
      build_fused<double>(p, take, Q, M, NB, c, kept, *reinterpret_cast<FusedArgs<double>*>(ps.args.data()), &nph,
                          ps.op_b0, ps.op_b1);
    }
    ps.op_gate = kept;
    ps.ngates = (int)kept.size();
    p->nphases += nph;
    p->passes.push_back(std::move(ps));
    // remove the kept gates; the rest keep their order
    std::vector<char> done(p->gates.size(), 0);
    for (int gi : kept) done[gi] = 1;
    std::vector<int> nr;
    for (int gi : rem)
      if (!done[gi]) nr.push_back(gi);
    rem.swap(nr);
  }
  // specialise the fused passes (one NVRTC program per batch of new pass
  // structures); until a pass has its kernel, or without NVRTC, it runs on the
  // generic k_fused kernel.  Mode 2 compiles on a background thread (tiered).
  p->jit.reset(new std::atomic<void*>[p->passes.size() + 1]);
  for (size_t i = 0; i <= p->passes.size(); ++i) p->jit[i].store(nullptr);
  p->njit.store(0);
  p->compiled = true;
  if (fuse && bt_jit_available()) {
    if (mode == 2) p->jit_thread = std::thread([p] { specialise(p); });
    else specialise(p);
  }
  if (mode == 3) {
    const int rc = build_tc_blocks(p);
    if (rc) {
      p->compiled = false;
      return rc;
    }
  }
  return BT_OK;
}

int bt_plan_set_tuning(bt_plan* p, int max_ops, int tile_rb, int packed, int tile_bits) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  const int mmin = p->prec == BT_PREC_C64 ? 10 : 9, mmax = p->prec == BT_PREC_C64 ? BT_TILE_M_C64 : BT_TILE_M_C128;
  if (max_ops < 0 || max_ops > BT_FUSED_MAX_OPS || (tile_rb != 0 && (tile_rb < 4 || tile_rb > 6)) || packed < -1 ||
      packed > 1 || (tile_bits != 0 && (tile_bits < mmin || tile_bits > mmax)))
    return bt_fail(p->ctx, BT_ERR_BAD_ARG,
                   "tuning: 0 <= max_ops <= 192, tile_rb in {0, 4, 5, 6}, packed in {-1, 0, 1}, tile_bits 0 or "
                   "10..13 (complex64) / 9..12 (complex128)");
  join_jit(p);
  p->tune_max_ops = max_ops;
  p->tune_rb = tile_rb;
  p->tune_packed = packed;
  p->tune_m = tile_bits;
  p->compiled = false;
  return BT_OK;
}

}  // extern "C"

// entries an encoded op reads (from its moff)
static int op_reals(const FOp& o) {
  switch (o.type) {
    case FOP_G1: case FOP_D2: case FOP_P2: return 8;
    case FOP_G2: return 32;
    case FOP_D1: case FOP_R1: case FOP_X1: return 4;
    case FOP_RX1: case FOP_DH: case FOP_RN: return 2;
    case FOP_RXN: return 1;
    default: return 0;  // CX, SW, HB
  }
}

// Per-member entries of fused pass `pass`: row m holds what the pass reads when the
// gates of these adds take member m's matrices (mats: `members` blocks of `per`
// reals, each the matrices of add_index back to back as bt_plan_set_matrices reads
// them).  The gates must already be variable, so no member changes the pass's
// structure.  The gates' own matrices are left as they were.
template <typename R>
static int member_table(bt_plan* p, size_t pass, int64_t members, int count, const int64_t* add_index,
                        const double* mats, size_t per, std::vector<R>& table, int* used) {
  PPass& ps = p->passes[pass];
  std::vector<unsigned char> scratch(ps.args);
  FusedArgs<R>& sa = *reinterpret_cast<FusedArgs<R>*>(scratch.data());
  int u = 0;
  for (int i = 0; i < ps.ngates; ++i) u = std::max(u, (int)sa.op[i].moff + op_reals(sa.op[i]));
  std::vector<std::pair<int, std::vector<double>>> saved;
  for (int i = 0; i < count; ++i)
    if (add_index[i] >= 0 && add_index[i] < (int64_t)p->adds.size())
      for (int j = 0; j < p->adds[add_index[i]].second; ++j) {
        const int gi = p->adds[add_index[i]].first + j;
        saved.push_back({gi, p->gates[gi].m});
      }
  table.assign((size_t)members * (size_t)u, (R)0);
  std::vector<char> touched;
  int rc = BT_OK;
  for (int64_t m = 0; m < members && !rc; ++m) {
    rc = assign_matrices(p, count, add_index, mats + (size_t)m * per, touched);
    if (rc) break;
    if (!encode_pass<R>(p, ps.op_gate, ps.op_b0, ps.op_b1, sa, true)) {
      rc = bt_fail(p->ctx, BT_ERR_BAD_ARG,
                   "a member's matrix changes a pass's structure: mark the gates variable and compile first");
      break;
    }
    memcpy(&table[(size_t)m * u], sa.mat, sizeof(R) * u);
  }
  for (auto& sv : saved) p->gates[sv.first].m = sv.second;
  *used = u;
  return rc;
}

// the touched gates (of these adds) made variable, the plan compiled with their
// entry-independent forms, and the per-member kernel of every fused pass that
// holds one of them built (or written to BTGPU_JIT_DUMP)
static int prepare_members(bt_plan* p, int count, const int64_t* add_index, std::vector<char>& touched) {
  size_t per = 0;
  int rc = bt_plan_gate_dims(p, add_index, count, &per);
  if (rc) return rc;
  touched.assign(p->gates.size(), 0);
  bool changed = false;
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < p->adds[add_index[i]].second; ++j) {
      PGate& g = p->gates[p->adds[add_index[i]].first + j];
      touched[p->adds[add_index[i]].first + j] = 1;
      changed |= !g.var;
      g.var = true;
    }
  // per-member entries live in fused passes: an unfused plan (mode 1) has none;
  // a fused or tiered plan keeps its mode (the tiered kernels are joined below)
  if (p->compile_mode == 1)
    return bt_fail(p->ctx, BT_ERR_UNSUPPORTED,
                   "per-member matrices need a fused plan (compile mode 0 or 2), not the unfused mode 1");
  if (changed || !p->compiled) {
    rc = bt_plan_compile(p, p->compile_mode);
    if (rc) return rc;
  }
  join_jit(p);
  if (!bt_jit_available())
    return bt_fail(p->ctx, BT_ERR_UNSUPPORTED, "per-member matrices need the specialised kernels (NVRTC)");
  const bool c64 = p->prec == BT_PREC_C64;
  std::vector<size_t> idx;
  for (size_t i = 0; i < p->passes.size(); ++i) {
    PPass& ps = p->passes[i];
    bool hit = false;
    if (ps.kind == 1) {
      if (touched[ps.gate])
        return bt_fail(p->ctx, BT_ERR_UNSUPPORTED,
                       "per-member matrices for a gate outside fused passes (more than two qubits or wide controls)");
      continue;
    }
    for (int gi : ps.op_gate) hit |= touched[gi] != 0;
    if (!hit || ps.pm_jit) continue;
    ps.pm_args = ps.args;
    if (c64) reinterpret_cast<FusedArgs<float>*>(ps.pm_args.data())->permem = 1;
    else reinterpret_cast<FusedArgs<double>*>(ps.pm_args.data())->permem = 1;
    idx.push_back(i);
  }
  if (idx.empty()) return BT_OK;
  std::vector<void*> ent;
  if (c64) {
    std::vector<const FusedArgs<float>*> v;
    for (size_t i : idx) v.push_back(reinterpret_cast<const FusedArgs<float>*>(p->passes[i].pm_args.data()));
    rc = bt_jit_prepare_f(p->ctx, v, ent);
  } else {
    std::vector<const FusedArgs<double>*> v;
    for (size_t i : idx) v.push_back(reinterpret_cast<const FusedArgs<double>*>(p->passes[i].pm_args.data()));
    rc = bt_jit_prepare_d(p->ctx, v, ent);
  }
  if (rc) return rc;
  for (size_t j = 0; j < idx.size(); ++j) p->passes[idx[j]].pm_jit = ent[j];
  return BT_OK;
}

extern "C" {

int bt_plan_prepare_members(bt_plan* p, int count, const int64_t* add_index) {
  if (!p || count < 1 || !add_index) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "bad arguments");
  std::vector<char> touched;
  return prepare_members(p, count, add_index, touched);
}

int bt_plan_member_table(bt_plan* p, int64_t pass, int64_t members, int count, const int64_t* add_index,
                         const double* mats, double* out, int64_t cap, int* used) {
  if (!p || !add_index || !mats || !used || members < 1 || count < 1)
    return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "bad arguments");
  if (!p->compiled) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "plan is not compiled");
  if (pass < 0 || pass >= (int64_t)p->passes.size() || p->passes[pass].kind != 0)
    return bt_fail(p->ctx, BT_ERR_BAD_ARG, "not a fused pass");
  size_t per = 0;
  int rc = bt_plan_gate_dims(p, add_index, count, &per);
  if (rc) return rc;
  if (p->prec == BT_PREC_C64) {
    std::vector<float> t;
    rc = member_table<float>(p, (size_t)pass, members, count, add_index, mats, per, t, used);
    if (!rc && out && cap >= (int64_t)t.size())
      for (size_t e = 0; e < t.size(); ++e) out[e] = t[e];
  } else {
    std::vector<double> t;
    rc = member_table<double>(p, (size_t)pass, members, count, add_index, mats, per, t, used);
    if (!rc && out && cap >= (int64_t)t.size())
      for (size_t e = 0; e < t.size(); ++e) out[e] = t[e];
  }
  return rc;
}

// arithmetic of one op per amplitude of the state, in real flops (an FMA counts
// two), as the specialised code does it
static double op_flops(const FOp& o) {
  switch (o.type) {
    case FOP_G1: return 14;
    case FOP_G2: return 32;
    case FOP_D1: case FOP_R1: case FOP_RX1: case FOP_D2: return 6;
    case FOP_P2: case FOP_X1: return o.unit ? 0 : 6;
    case FOP_DH: return o.unit ? 0 : 3;
    case FOP_RN: case FOP_RXN: return 4;
    case FOP_HB: return 2;
    default: return 0;  // CX, SW: register renaming
  }
}

int bt_plan_cost(const bt_plan* p, double* flops_per_amp, double* bytes_per_amp) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  if (!p->compiled) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "plan is not compiled");
  const bool c64 = p->prec == BT_PREC_C64;
  double fl = 0, by = 0;
  for (const auto& ps : p->passes) {
    by += 2.0 * (c64 ? 8 : 16);
    if (ps.kind == 0) {
      const FOp* ops = c64 ? reinterpret_cast<const FusedArgs<float>*>(ps.args.data())->op
                           : reinterpret_cast<const FusedArgs<double>*>(ps.args.data())->op;
      for (int i = 0; i < ps.ngates; ++i) fl += op_flops(ops[i]);
    } else {
      fl += 8.0 * (1 << p->gates[ps.gate].k);  // dense sweep: 2^k complex multiply-adds
    }
  }
  if (flops_per_amp) *flops_per_amp = fl;
  if (bytes_per_amp) *bytes_per_amp = by;
  return BT_OK;
}

int bt_plan_pass_ops(const bt_plan* p, int64_t pass, int* kind, int* nops, int32_t* ops, double* mats, int cap_ops,
                     int cap_reals) {
  if (!p || !kind || !nops) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL argument");
  if (!p->compiled) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "plan is not compiled");
  if (pass < 0 || pass >= (int64_t)p->passes.size()) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "pass out of range");
  const PPass& ps = p->passes[pass];
  *kind = ps.kind;
  if (ps.kind != 0) {  // sweep: k, bits[0..4], control mask (low, high 32 bits); the row-major matrix
    const PGate& g = p->gates[ps.gate];
    const int d = 1 << g.k;
    *nops = 1;
    if (cap_ops < 2 || cap_reals < 2 * d * d || !ops || !mats)
      return bt_fail(p->ctx, BT_ERR_BAD_ARG, "output arrays too small");
    ops[0] = g.k;
    for (int i = 0; i < 5; ++i) ops[1 + i] = i < g.k ? g.bits[i] : -1;
    ops[6] = (int32_t)(uint32_t)g.cmask;
    ops[7] = (int32_t)(uint32_t)(g.cmask >> 32);
    for (int e = 0; e < 2 * d * d; ++e) mats[e] = g.m[e];
    return BT_OK;
  }
  const bool c64 = p->prec == BT_PREC_C64;
  const void* args = ps.args.data();
  const FPhase* ph = c64 ? reinterpret_cast<const FusedArgs<float>*>(args)->ph
                         : reinterpret_cast<const FusedArgs<double>*>(args)->ph;
  const FOp* op = c64 ? reinterpret_cast<const FusedArgs<float>*>(args)->op
                      : reinterpret_cast<const FusedArgs<double>*>(args)->op;
  const int* tbits = c64 ? reinterpret_cast<const FusedArgs<float>*>(args)->tbits
                         : reinterpret_cast<const FusedArgs<double>*>(args)->tbits;
  const int nph = c64 ? reinterpret_cast<const FusedArgs<float>*>(args)->nphase
                      : reinterpret_cast<const FusedArgs<double>*>(args)->nphase;
  const int nreals = c64 ? BT_FUSED_MAX_REALS_F : BT_FUSED_MAX_REALS_D;
  *nops = ps.ngates;
  if (cap_ops < ps.ngates || !ops || !mats || cap_reals < nreals)
    return bt_fail(p->ctx, BT_ERR_BAD_ARG, "output arrays too small");
  for (int q = 0; q < nph; ++q)
    for (int i = ph[q].op0; i < ph[q].op0 + ph[q].nop; ++i) {
      const FOp& o = op[i];
      int32_t* r = ops + 6 * i;
      r[0] = o.type;
      r[1] = tbits[ph[q].reg[o.b0]];
      r[2] = tbits[ph[q].reg[o.b1]];
      r[3] = o.flags;
      r[4] = o.unit;
      r[5] = o.moff;
    }
  for (int e = 0; e < nreals; ++e)
    mats[e] = c64 ? reinterpret_cast<const FusedArgs<float>*>(args)->mat[e]
                  : reinterpret_cast<const FusedArgs<double>*>(args)->mat[e];
  return BT_OK;
}

int bt_plan_stats(const bt_plan* p, int64_t* ngates, int64_t* npasses, int64_t* nfused, int64_t* nphases,
                  int64_t* njit) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  int64_t nf = 0;
  for (auto& ps : p->passes) nf += ps.kind == 0;
  if (ngates) *ngates = (int64_t)p->gates.size();
  if (npasses) *npasses = (int64_t)p->passes.size();
  if (nfused) *nfused = nf;
  if (nphases) *nphases = p->nphases;
  if (njit) *njit = p->njit.load();
  return BT_OK;
}

int bt_plan_run(bt_plan* p, bt_state* s, int64_t member) {
  if (!p || !s) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "NULL argument");
  bt_ctx* ctx = s->ctx;
  if (s->n != p->n || s->repr != p->repr || s->prec != p->prec)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "plan and state differ in n, repr or prec");
  if (!p->compiled) {
    int rc = bt_plan_compile(p, p->compile_mode);
    if (rc) return rc;
  }
  int64_t lo = 0, nm = s->batch;
  if (member != -1) {
    if (member < 0 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
    lo = member;
    nm = 1;
  }
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  for (size_t i = 0; i < p->passes.size() && !rc; ++i) {
    PPass& ps = p->passes[i];
    if (ps.kind == 1) {
      const PGate& g = p->gates[ps.gate];
      rc = bt_launch_gate(s, g.k, g.bits, g.m.data(), g.cmask, lo, nm, nullptr, 0);
    } else if (p->prec == BT_PREC_C64 && ps.tc_block >= 0 && p->d_tc) {
      const FusedArgs<float>& a = *reinterpret_cast<const FusedArgs<float>*>(ps.args.data());
      TcPass t;
      t.nbits = a.nbits;
      t.c = a.c;
      t.nphase = a.nphase;
      t.lg_tiles = a.lg_tiles;
      t.member_lo = lo;
      t.nmem = nm;
      for (int b = 0; b < 16; ++b) t.tbits[b] = a.tbits[b];
      for (int ph = 0; ph < a.nphase; ++ph)
        for (int b = 0; b < 5; ++b) t.reg[ph][b] = a.ph[ph].reg[b];
      t.bmat = p->d_tc + (size_t)ps.tc_block * 8192;
      if (p->d_tc_device != ctx->device) rc = bt_fail(ctx, BT_ERR_BAD_ARG, "tensor-core plan compiled for another device");
      else rc = bt_launch_tc_pass(ctx, s->d, t);
    } else if (p->prec == BT_PREC_C64) {
      FusedArgs<float>& a = *reinterpret_cast<FusedArgs<float>*>(ps.args.data());
      a.member_lo = lo;
      a.nmem = nm;
      void* e = p->jit[i].load(std::memory_order_acquire);
      rc = e ? bt_jit_launch_f(ctx, e, s->d, a) : bt_launch_fused_f(ctx, s->d, a);
    } else {
      FusedArgs<double>& a = *reinterpret_cast<FusedArgs<double>*>(ps.args.data());
      a.member_lo = lo;
      a.nmem = nm;
      void* e = p->jit[i].load(std::memory_order_acquire);
      rc = e ? bt_jit_launch_d(ctx, e, s->d, a) : bt_launch_fused_d(ctx, s->d, a);
    }
  }
  return rc;
}

int bt_plan_run_members(bt_plan* p, bt_state* s, int count, const int64_t* add_index, const double* mats) {
  if (!p || !s) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "bad arguments");
  return bt_plan_run_members_n(p, s, s->batch, count, add_index, mats);
}

}  // extern "C"

// members [0, nmem) of s (the serving engine runs as many as it has requests)
int bt_plan_run_members_n(bt_plan* p, bt_state* s, int64_t nmem, int count, const int64_t* add_index,
                          const double* mats) {
  if (!p || !s || count < 1 || !add_index || !mats) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "bad arguments");
  bt_ctx* ctx = s->ctx;
  if (s->n != p->n || s->repr != p->repr || s->prec != p->prec)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "plan and state differ in n, repr or prec");
  if (nmem < 1 || nmem > s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member count outside the batch");
  std::vector<char> touched;
  int rc = prepare_members(p, count, add_index, touched);
  if (rc) return rc;
  size_t per = 0;
  rc = bt_plan_gate_dims(p, add_index, count, &per);
  if (rc) return rc;
  const int64_t B = nmem;
  const bool c64 = p->prec == BT_PREC_C64;
  rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  for (size_t i = 0; i < p->passes.size() && !rc; ++i) {
    PPass& ps = p->passes[i];
    if (ps.kind == 1) {
      const PGate& g = p->gates[ps.gate];
      rc = bt_launch_gate(s, g.k, g.bits, g.m.data(), g.cmask, 0, B, nullptr, 0);
      continue;
    }
    void* e = p->jit[i].load(std::memory_order_acquire);
    bool hit = false;
    for (int gi : ps.op_gate) hit |= touched[gi] != 0;
    if (hit && !ps.pm_jit) {
      rc = bt_fail(ctx, BT_ERR_DEVICE, "the per-member kernel of a pass was not built");
      break;
    }
    if (!hit) {  // no member-dependent gate in this pass
      if (c64) {
        FusedArgs<float>& a = *reinterpret_cast<FusedArgs<float>*>(ps.args.data());
        a.member_lo = 0;
        a.nmem = B;
        rc = e ? bt_jit_launch_f(ctx, e, s->d, a) : bt_launch_fused_f(ctx, s->d, a);
      } else {
        FusedArgs<double>& a = *reinterpret_cast<FusedArgs<double>*>(ps.args.data());
        a.member_lo = 0;
        a.nmem = B;
        rc = e ? bt_jit_launch_d(ctx, e, s->d, a) : bt_launch_fused_d(ctx, s->d, a);
      }
      continue;
    }
    // the pass's entries for every member, uploaded to the plan's table (stream
    // order keeps the previous pass's reads before this upload)
    std::vector<float> tf;
    std::vector<double> td;
    int used = 0;
    rc = c64 ? member_table<float>(p, i, B, count, add_index, mats, per, tf, &used)
             : member_table<double>(p, i, B, count, add_index, mats, per, td, &used);
    if (rc) break;
    const size_t bytes = c64 ? tf.size() * sizeof(float) : td.size() * sizeof(double);
    if (bytes > p->d_pm_bytes || p->d_pm_device != ctx->device) {
      if (p->d_pm) {
        cudaSetDevice(p->d_pm_device);
        cudaFree(p->d_pm);
        cudaSetDevice(ctx->device);
        p->d_pm = nullptr;
      }
      rc = bt_cuda_check(ctx, cudaMalloc(&p->d_pm, bytes), "per-member table");
      if (rc) break;
      p->d_pm_bytes = bytes;
      p->d_pm_device = ctx->device;
    }
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(p->d_pm, c64 ? (const void*)tf.data() : (const void*)td.data(), bytes,
                                            cudaMemcpyHostToDevice, ctx->stream),
                       "per-member table upload");
    if (rc) break;
    if (c64) {
      FusedArgs<float>& a = *reinterpret_cast<FusedArgs<float>*>(ps.pm_args.data());
      a.member_lo = 0;
      a.nmem = B;
      rc = bt_jit_launch_members_f(ctx, ps.pm_jit, s->d, a, (const float*)p->d_pm, used);
    } else {
      FusedArgs<double>& a = *reinterpret_cast<FusedArgs<double>*>(ps.pm_args.data());
      a.member_lo = 0;
      a.nmem = B;
      rc = bt_jit_launch_members_d(ctx, ps.pm_jit, s->d, a, (const double*)p->d_pm, used);
    }
  }
  return rc;
}

// ------------------------------------------------------------------ serving hooks (bt_serve.cu)
// add indices whose gates are all variable (the gates a client's requests rewrite)
int bt_plan_variable_adds(const bt_plan* p, std::vector<int64_t>& idx) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  idx.clear();
  for (size_t a = 0; a < p->adds.size(); ++a) {
    bool var = p->adds[a].second > 0;
    for (int j = 0; j < p->adds[a].second; ++j) var &= p->gates[p->adds[a].first + j].var;
    if (var) idx.push_back((int64_t)a);
  }
  return BT_OK;
}

int bt_plan_shape(const bt_plan* p, int* n, int* repr, int* prec) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "plan is NULL");
  *n = p->n;
  *repr = p->repr;
  *prec = p->prec;
  return BT_OK;
}

// reals of the matrices that bt_plan_set_matrices reads for these add indices
int bt_plan_gate_dims(const bt_plan* p, const int64_t* idx, int count, size_t* reals) {
  size_t r = 0;
  for (int i = 0; i < count; ++i) {
    const int64_t ai = idx[i];
    if (ai < 0 || ai >= (int64_t)p->adds.size()) return bt_fail(nullptr, BT_ERR_BAD_ARG, "add index out of range");
    if (p->adds[ai].second == 0) return bt_fail(nullptr, BT_ERR_BAD_ARG, "a Kraus sum cannot be updated");
    const int d = 1 << p->gates[p->adds[ai].first].ku;
    r += (size_t)2 * d * d;
  }
  *reals = r;
  return BT_OK;
}
