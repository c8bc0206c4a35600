// Noisy-circuit programs executed whole inside one CTA per member.
//
// For members small enough to live in shared memory (2^n complex numbers,
// n <= 14 for complex64 and 13 for complex128), a trajectory batch runs its whole
// op sequence -- gates, Monte-Carlo Kraus branches and mid-circuit measurements --
// in a single launch: CTA m loads member m into shared memory, and for every
// channel or measurement reduces the reduced density matrix of its qubits in FP64
// across the block, lets thread 0 draw the branch / outcome with the rules of the
// reference (first i with u <= cumsum(p), src/hilbert.jl:810-819; u < p0,
// src/hilbert.jl:693), and applies the renormalised Kraus operator or projector.
// There is no host round trip and no global synchronisation between ops: this is
// the per-shot loop of the reference's noisy measure(circuit, shots)
// (src/ops.jl:617-630: to_state once per shot) with every shot a CTA.  Members whose program is shorter
// (ZNE repetitions, no measurement at that point) skip ops through per-member
// flags; per-member gate matrices carry twirl frames.
#include <string.h>

#include <atomic>
#include <type_traits>
#include <vector>

#include "bt_internal.cuh"

enum { PG_GATE1 = 1, PG_GATE2 = 2, PG_CHANNEL = 3, PG_MEASURE = 4 };

struct PGOp {
  int type;
  int b0, b1;      // bit positions; b0 = most significant bit of the matrix index
  int k, nk;       // channel: qubits and Kraus operators
  int flags;       // channel: 1 reference branch order for the pair, 2 unitary mixture
  int moff;        // gate: offset into gm (reals); channel: offset into km (reals)
  int mstride;     // gate: per-member stride in gm (0: one matrix for all)
  int skip_off;    // offset into the skip table (one byte per member), -1: none
  int rand_idx;    // index of this op's draw, -1: none
  int rec_idx;     // measurement: record slot
  int mlo, mhi;    // members [mlo, mhi) take part; per-member matrices are indexed from mlo
};

// A group of consecutive ops acting inside one set Q of at most two qubits (the
// grouped executor for members too large for shared memory): one reduction of the
// member's reduced density matrix on Q, one decision per member (every branch and
// outcome of the group decided from rho_Q, which each op on Q transforms exactly:
// rho_Q -> K rho_Q K^dagger / p), one pass applying the product of the chosen
// matrices.
struct PGGroup {
  int nb;        // qubits in Q (1 or 2)
  int q0, q1;    // bit positions, q0 = most significant bit of the group index
  int op0, nop;  // ops [op0, op0 + nop)
  int need_rho;  // some op's decision depends on the state
  int mlo, mhi;  // members [mlo, mhi) hold every member active in the group (launch range)
};

struct bt_program {
  bt_ctx* ctx = nullptr;
  int device = 0;  // ctx's device, kept so that freeing needs no live context
  int n = 0, prec = 0, batch = 0;
  int executor = 0;  // 0 automatic, 1 shared memory, 2 grouped
  std::vector<PGGroup> groups;
  void* d_gact = nullptr;  // [group][member] 1 = the member does something in the group
  void* d_rho = nullptr;   // [member][32] reduced matrices (FP64)
  void* d_mat = nullptr;   // [member][32] chosen group matrices (state precision)
  std::vector<PGOp> ops;
  std::vector<double> gm;   // gate matrices, row-major interleaved (converted to the state precision)
  std::vector<double> km;   // Kraus sets, row-major interleaved FP64
  std::vector<int8_t> skip;
  int ndraws = 0, nrec = 0;
  int range_lo = 0, range_hi = -1;  // member range of the ops added next (-1: to the batch's end)
  // device copies
  bool uploaded = false;
  bool gm_dirty = false;     // gate matrices rewritten since the upload
  std::vector<float> gstage; // complex64 copy of gm for uploads
  void* d_ops = nullptr;
  void* d_gm = nullptr;
  void* d_km = nullptr;
  void* d_skip = nullptr;
  void* d_rec = nullptr;
  void* d_u = nullptr;
  size_t u_bytes = 0;
};

#define PG_THREADS 256
#define PG_MAX_KRAUS 64
#define FULLM 0xffffffffu

template <int W>
__device__ __forceinline__ void block_reduce(double (&v)[W], double* sh /* 8*W */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    double x = v[w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULLM, x, o);
    if (lane == 0) sh[warp * W + w] = x;
  }
  __syncthreads();
  if (threadIdx.x < W) {
    double s = 0;
    for (int i = 0; i < PG_THREADS / 32; ++i) s += sh[i * W + threadIdx.x];
    sh[8 * W + threadIdx.x] = s;  // results after the per-warp partials
  }
  __syncthreads();
}

template <typename R>
__device__ __forceinline__ void apply1(typename CT<R>::T* st, int nbits, int b, const R* m) {
  const int np = 1 << (nbits - 1);
  const R m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3], m10r = m[4], m10i = m[5], m11r = m[6], m11i = m[7];
  for (int p = threadIdx.x; p < np; p += PG_THREADS) {
    const int i0 = ((p >> b) << (b + 1)) | (p & ((1 << b) - 1)), i1 = i0 | (1 << b);
    typename CT<R>::T a = st[i0], c = st[i1];
    typename CT<R>::T x, y;
    x.x = m00r * a.x - m00i * a.y + m01r * c.x - m01i * c.y;
    x.y = m00r * a.y + m00i * a.x + m01r * c.y + m01i * c.x;
    y.x = m10r * a.x - m10i * a.y + m11r * c.x - m11i * c.y;
    y.y = m10r * a.y + m10i * a.x + m11r * c.y + m11i * c.x;
    st[i0] = x;
    st[i1] = y;
  }
}

template <typename R>
__device__ __forceinline__ void apply2(typename CT<R>::T* st, int nbits, int b0, int b1, const R* m) {
  const int lo = b0 < b1 ? b0 : b1, hi = b0 < b1 ? b1 : b0;
  const int nq = 1 << (nbits - 2);
  for (int p = threadIdx.x; p < nq; p += PG_THREADS) {
    int base = ((p >> lo) << (lo + 1)) | (p & ((1 << lo) - 1));
    base = ((base >> hi) << (hi + 1)) | (base & ((1 << hi) - 1));
    const int q[4] = {base, base | (1 << b1), base | (1 << b0), base | (1 << b0) | (1 << b1)};
    R ar[4], ai[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      typename CT<R>::T v = st[q[c]];
      ar[c] = v.x;
      ai[c] = v.y;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      R yr = 0, yi = 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const R mr = m[2 * (4 * r + c)], mi = m[2 * (4 * r + c) + 1];
        yr += mr * ar[c] - mi * ai[c];
        yi += mr * ai[c] + mi * ar[c];
      }
      typename CT<R>::T v;
      v.x = yr;
      v.y = yi;
      st[q[r]] = v;
    }
  }
}

// reduced density matrix of k = 1 / 2 bits (row-major interleaved, FP64) into rho
template <typename R, int K>
__device__ void reduce_rho(const typename CT<R>::T* st, int nbits, int b0, int b1, double* sh, double* rho) {
  constexpr int D = 1 << K, W = 2 * D * D;
  // complex64: FP32 products summed over 8 consecutive iterations of a thread,
  // each group added to FP64 accumulators (GB300's FP64 issue rate would
  // otherwise bound the reduction); complex128: FP64 throughout
  typedef typename std::conditional<sizeof(R) == 4, float, double>::type A;
  constexpr int J = sizeof(R) == 4 ? 8 : 1;
  double acc[W];
#pragma unroll
  for (int w = 0; w < W; ++w) acc[w] = 0;
  const int lo = K == 2 ? (b0 < b1 ? b0 : b1) : b0, hi = K == 2 ? (b0 < b1 ? b1 : b0) : b0;
  const int ng = 1 << (nbits - K);
  for (int p0 = threadIdx.x; p0 < ng; p0 += PG_THREADS * J) {
    A f[W];
#pragma unroll
    for (int w = 0; w < W; ++w) f[w] = 0;
#pragma unroll
    for (int jj = 0; jj < J; ++jj) {
      const int p = p0 + jj * PG_THREADS;
      if (p >= ng) break;
      int base = ((p >> lo) << (lo + 1)) | (p & ((1 << lo) - 1));
      if (K == 2) base = ((base >> hi) << (hi + 1)) | (base & ((1 << hi) - 1));
      A xr[D], xi[D];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        int idx = base;
        if (K == 1) idx |= (j & 1) << b0;
        else idx |= ((j >> 1) & 1) << b0 | (j & 1) << b1;
        typename CT<R>::T v = st[idx];
        xr[j] = (A)v.x;
        xi[j] = (A)v.y;
      }
#pragma unroll
      for (int a = 0; a < D; ++a)
#pragma unroll
        for (int b = a; b < D; ++b) {
          f[2 * (a * D + b)] += xr[a] * xr[b] + xi[a] * xi[b];
          if (b != a) f[2 * (a * D + b) + 1] += xi[a] * xr[b] - xr[a] * xi[b];
        }
    }
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = a; b < D; ++b) {
        acc[2 * (a * D + b)] += (double)f[2 * (a * D + b)];
        acc[2 * (a * D + b) + 1] += (double)f[2 * (a * D + b) + 1];
      }
  }
  // lower triangle from the upper one: rho[b, a] = conj(rho[a, b])
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = 0; b < a; ++b) {
      acc[2 * (a * D + b)] = acc[2 * (b * D + a)];
      acc[2 * (a * D + b) + 1] = -acc[2 * (b * D + a) + 1];
    }
  block_reduce<W>(acc, sh);
  if (threadIdx.x < W) rho[threadIdx.x] = sh[8 * W + threadIdx.x];
  __syncthreads();
}

__device__ double tr_krk(const double* K, const double* r, int D, bool diag_rho, bool ref_perm) {
  const int perm[4] = {0, 2, 1, 3};
  double p = 0;
  for (int c = 0; c < D; ++c)
    for (int a = 0; a < D; ++a) {
      const double kar = K[2 * (c * D + a)], kai = K[2 * (c * D + a) + 1];
      for (int b = 0; b < D; ++b) {
        const int ra = ref_perm ? perm[a] : a, rb = ref_perm ? perm[b] : b;
        const double rr = diag_rho ? (ra == rb ? 1.0 / D : 0.0) : r[2 * (ra * D + rb)];
        const double ri = diag_rho ? 0.0 : r[2 * (ra * D + rb) + 1];
        const double kbr = K[2 * (c * D + b)], kbi = -K[2 * (c * D + b) + 1];
        const double tr_ = kar * rr - kai * ri, ti = kar * ri + kai * rr;
        p += tr_ * kbr - ti * kbi;
      }
    }
  return p;
}

template <typename R>
__global__ void __launch_bounds__(PG_THREADS) k_program(typename CT<R>::T* __restrict__ states, int nbits,
                                                        const PGOp* __restrict__ ops, int nops,
                                                        const R* __restrict__ gm, const double* __restrict__ km,
                                                        const int8_t* __restrict__ skip, const double* __restrict__ u,
                                                        uint64_t key, uint64_t stream, int batch,
                                                        int32_t* __restrict__ rec, int nrec, int* __restrict__ status) {
  typedef typename CT<R>::T C2;
  extern __shared__ __align__(16) unsigned char smem[];
  C2* st = reinterpret_cast<C2*>(smem);
  double* sh = reinterpret_cast<double*>(smem + (sizeof(C2) << nbits));  // 9 * 32 doubles
  double* pk = sh + 9 * 32;                                               // PG_MAX_KRAUS branch probabilities
  double* nk = pk + PG_MAX_KRAUS;                                         // PG_MAX_KRAUS branch norms
  R* mat = reinterpret_cast<R*>(nk + PG_MAX_KRAUS);                       // 32 reals
  __shared__ int s_ok;
  const int m = blockIdx.x;
  C2* g = states + ((int64_t)m << nbits);
  const int len = 1 << nbits;
  for (int i = threadIdx.x; i < len; i += PG_THREADS) st[i] = g[i];
  __syncthreads();
  for (int oi = 0; oi < nops; ++oi) {
    const PGOp op = ops[oi];
    if (m < op.mlo || m >= op.mhi || (op.skip_off >= 0 && skip[op.skip_off + m])) {  // uniform across the block
      if (op.type == PG_MEASURE && threadIdx.x == 0) rec[(int64_t)m * nrec + op.rec_idx] = -1;
      continue;
    }
    if (op.type == PG_GATE1) {
      apply1<R>(st, nbits, op.b0, gm + op.moff + (int64_t)op.mstride * (m - op.mlo));
      __syncthreads();
    } else if (op.type == PG_GATE2) {
      apply2<R>(st, nbits, op.b0, op.b1, gm + op.moff + (int64_t)op.mstride * (m - op.mlo));
      __syncthreads();
    } else if (op.type == PG_CHANNEL) {
      const int D = 1 << op.k;
      double* rho = sh + 8 * 32;  // the reduction's result row
      const bool umix = op.flags & 2;
      if (!umix) {
        if (op.k == 1) reduce_rho<R, 1>(st, nbits, op.b0, op.b1, sh, rho);
        else reduce_rho<R, 2>(st, nbits, op.b0, op.b1, sh, rho);
      }
      // branch probabilities (reference order) and norms (application order), one
      // Kraus operator per lane of warp 0
      if (threadIdx.x < 32) {
        const bool perm = (op.flags & 1) && op.k == 2;
        for (int i = threadIdx.x; i < op.nk; i += 32) {
          const double* Ki = km + op.moff + (int64_t)i * 2 * D * D;
          const double pi = tr_krk(Ki, rho, D, umix, perm);
          pk[i] = pi;
          nk[i] = perm ? tr_krk(Ki, rho, D, umix, false) : pi;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const double uu = u ? u[(int64_t)op.rand_idx * batch + m] : bt_uniform(key, stream ^ (uint64_t)op.rand_idx, m);
        double cum = 0;
        int ind = -1;
        for (int i = 0; i < op.nk; ++i) {
          cum += pk[i];
          if (ind < 0 && uu <= cum) ind = i;
        }
        s_ok = 1;
        const double nrm = ind >= 0 ? nk[ind] : 0.0;
        if (ind < 0 || !(nrm > 0)) {
          atomicExch(status, ind < 0 ? 2 : 3);
          s_ok = 0;
        } else {
          const double sc = 1.0 / sqrt(nrm);
          const double* K = km + op.moff + (int64_t)ind * 2 * D * D;
          for (int e = 0; e < 2 * D * D; ++e) mat[e] = (R)(K[e] * sc);
        }
      }
      __syncthreads();
      if (s_ok) {
        if (op.k == 1) apply1<R>(st, nbits, op.b0, mat);
        else apply2<R>(st, nbits, op.b0, op.b1, mat);
      }
      __syncthreads();
    } else if (op.type == PG_MEASURE) {
      double* rho = sh + 8 * 32;
      reduce_rho<R, 1>(st, nbits, op.b0, 0, sh, rho);
      if (threadIdx.x == 0) {
        const double s0 = rho[0], s1 = rho[6];
        const double uu = u ? u[(int64_t)op.rand_idx * batch + m] : bt_uniform(key, stream ^ (uint64_t)op.rand_idx, m);
        const int ind = uu < s0 ? 0 : 1;
        const double keep = ind ? s1 : s0;
        s_ok = keep > 0;
        if (!s_ok) atomicExch(status, 1);
        rec[(int64_t)m * nrec + op.rec_idx] = s_ok ? ind : -1;
        mat[0] = s_ok ? (R)(1.0 / sqrt(keep)) : (R)1;
        mat[1] = (R)ind;
      }
      __syncthreads();
      if (s_ok) {
        const int ind = (int)mat[1];
        const R sc = mat[0];
        for (int i = threadIdx.x; i < len; i += PG_THREADS) {
          C2 v = st[i];
          if (((i >> op.b0) & 1) == ind) {
            v.x *= sc;
            v.y *= sc;
          } else {
            v.x = 0;
            v.y = 0;
          }
          st[i] = v;
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < len; i += PG_THREADS) g[i] = st[i];
}

// ------------------------------------------------------------------ grouped executor: decisions
// the group's reduced matrix restricted to the op's qubits, in the op's order
__device__ void restrict_rho(const double* rho, int opk, int x, const PGGroup& g, double* out) {
  const int D = 1 << g.nb;
  if (g.nb == 1 || (opk == 2 && x == g.q0)) {
    for (int e = 0; e < 2 * D * D; ++e) out[e] = rho[e];
    return;
  }
  if (opk == 2) {
    const int sw[4] = {0, 2, 1, 3};
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) {
        out[2 * (r * 4 + c)] = rho[2 * (sw[r] * 4 + sw[c])];
        out[2 * (r * 4 + c) + 1] = rho[2 * (sw[r] * 4 + sw[c]) + 1];
      }
    return;
  }
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      double sr = 0, si = 0;
      for (int c = 0; c < 2; ++c) {
        const int r = x == g.q0 ? 2 * a + c : 2 * c + a, col = x == g.q0 ? 2 * b + c : 2 * c + b;
        sr += rho[2 * (r * 4 + col)];
        si += rho[2 * (r * 4 + col) + 1];
      }
      out[2 * (a * 2 + b)] = sr;
      out[2 * (a * 2 + b) + 1] = si;
    }
}

// A team of 16 threads per member (two members per warp): every op of group g,
// decided from rho_Q; writes the product of the chosen (renormalised) matrices in
// the state precision.  The 4x4 complex algebra of an op (the product E M, the
// update E rho E^dagger) is split one matrix entry per thread, and a channel's
// branch probabilities one Kraus operator per thread, in shared memory; the
// decisions themselves (the cumulative sums against the member's draw) are made
// by the team's first thread in the reference's order, so they equal the
// one-thread form's.  GB300's FP64 rate is a small share of its FP32 rate: split
// this way a member's chain of FP64 operations is 16 times shorter.  Failure rules
// as in k_program: an op whose branch or outcome has zero probability is skipped
// for that member (record -1) and reported through the status word.
#define PGD_TEAM 16
#define PGD_TEAMS 8  // members per block (128 threads)
struct PGDShared {
  double M[32], rho[32], tmp[32], E[32], K[32], rop[32], p[PG_MAX_KRAUS];
  int ind, skipped;
  double sc;
};

template <typename R>
__global__ void __launch_bounds__(PGD_TEAM * PGD_TEAMS) k_group_decide(
    const PGGroup g, const PGOp* __restrict__ ops, const R* __restrict__ gm, const double* __restrict__ km,
    const int8_t* __restrict__ skip, const int8_t* __restrict__ act, const double* __restrict__ u, uint64_t key,
    uint64_t stream, int batch, const double* __restrict__ rho_in, R* __restrict__ mat_out,
    int32_t* __restrict__ rec, int nrec, int* __restrict__ status) {
  __shared__ PGDShared shm[PGD_TEAMS];
  const int team = threadIdx.x / PGD_TEAM, t = threadIdx.x % PGD_TEAM;
  const unsigned mask = 0xFFFFu << (16 * (team & 1));  // the team's lanes of its warp
  const int m = g.mlo + blockIdx.x * PGD_TEAMS + team;
  if (m >= g.mhi) return;  // the whole team leaves together
  PGDShared& S = shm[team];
  const int D = 1 << g.nb;
  const bool on = act[m];
  const int r = t / D, c = t % D;  // the matrix entry of this thread (t < D*D)
  const bool ent = t < D * D;
  if (ent) {
    S.M[2 * t] = r == c ? 1.0 : 0.0;
    S.M[2 * t + 1] = 0.0;
    S.rho[2 * t] = g.need_rho && on ? rho_in[(int64_t)(m - g.mlo) * 2 * D * D + 2 * t] : 0.0;
    S.rho[2 * t + 1] = g.need_rho && on ? rho_in[(int64_t)(m - g.mlo) * 2 * D * D + 2 * t + 1] : 0.0;
  }
  __syncwarp(mask);
  for (int oi = g.op0; oi < g.op0 + g.nop; ++oi) {
    const PGOp op = ops[oi];
    const bool skipped = !on || m < op.mlo || m >= op.mhi || (op.skip_off >= 0 && skip[op.skip_off + m]);
    if (skipped) {
      if (op.type == PG_MEASURE && t == 0) rec[(int64_t)m * nrec + op.rec_idx] = -1;
      continue;
    }
    const int opk = op.type == PG_GATE2 ? 2 : (op.type == PG_CHANNEL ? op.k : 1);
    const int d = 1 << opk;
    if (op.type == PG_GATE1 || op.type == PG_GATE2) {
      const R* src = gm + op.moff + (int64_t)op.mstride * (m - op.mlo);
      for (int e = t; e < 2 * d * d; e += PGD_TEAM) S.K[e] = (double)src[e];
    } else if (op.type == PG_CHANNEL) {
      const bool umix = op.flags & 2;
      if (t == 0 && !umix) restrict_rho(S.rho, opk, op.b0, g, S.rop);
      __syncwarp(mask);
      for (int i = t; i < op.nk; i += PGD_TEAM)
        S.p[i] = tr_krk(km + op.moff + (int64_t)i * 2 * d * d, S.rop, d, umix, (op.flags & 1) && opk == 2);
      __syncwarp(mask);
      if (t == 0) {
        const double uu = u ? u[(int64_t)op.rand_idx * batch + m] : bt_uniform(key, stream ^ (uint64_t)op.rand_idx, m);
        double cum = 0;
        int ind = -1;
        for (int i = 0; i < op.nk; ++i) {
          cum += S.p[i];
          if (ind < 0 && uu <= cum) ind = i;
        }
        const double nrm = ind >= 0 ? tr_krk(km + op.moff + (int64_t)ind * 2 * d * d, S.rop, d, umix, false) : 0.0;
        S.skipped = ind < 0 || !(nrm > 0);
        if (S.skipped) atomicExch(status, ind < 0 ? 2 : 3);
        S.ind = ind < 0 ? 0 : ind;
        S.sc = S.skipped ? 0.0 : 1.0 / sqrt(nrm);
      }
      __syncwarp(mask);
      if (S.skipped) continue;
      const double* Ki = km + op.moff + (int64_t)S.ind * 2 * d * d;
      for (int e = t; e < 2 * d * d; e += PGD_TEAM) S.K[e] = Ki[e] * S.sc;
    } else {  // measurement: outcome u < p0 ? 0 : 1 from the qubit's reduced matrix
      if (t == 0) {
        restrict_rho(S.rho, 1, op.b0, g, S.rop);
        const double s0 = S.rop[0], s1 = S.rop[6];
        const double uu = u ? u[(int64_t)op.rand_idx * batch + m] : bt_uniform(key, stream ^ (uint64_t)op.rand_idx, m);
        const int ind = uu < s0 ? 0 : 1;
        const double keep = ind ? s1 : s0;
        S.skipped = !(keep > 0);
        if (S.skipped) {
          atomicExch(status, 1);
          rec[(int64_t)m * nrec + op.rec_idx] = -1;
        } else {
          rec[(int64_t)m * nrec + op.rec_idx] = ind;
          for (int e = 0; e < 8; ++e) S.K[e] = 0;
          S.K[ind ? 6 : 0] = 1.0 / sqrt(keep);
        }
      }
      __syncwarp(mask);
      if (S.skipped) continue;
    }
    __syncwarp(mask);
    // E: the op's matrix in the group's space (q0 the most significant bit)
    if (ent) {
      double er = 0, ei = 0;
      if (g.nb == 1 || (opk == 2 && op.b0 == g.q0)) {
        er = S.K[2 * t];
        ei = S.K[2 * t + 1];
      } else if (opk == 2) {  // (x, y) = (q1, q0): the two index bits swapped
        const int sw[4] = {0, 2, 1, 3};
        er = S.K[2 * (sw[r] * 4 + sw[c])];
        ei = S.K[2 * (sw[r] * 4 + sw[c]) + 1];
      } else if (op.b0 == g.q0) {  // K (x) I
        if ((r & 1) == (c & 1)) {
          er = S.K[2 * ((r >> 1) * 2 + (c >> 1))];
          ei = S.K[2 * ((r >> 1) * 2 + (c >> 1)) + 1];
        }
      } else {  // I (x) K
        if ((r >> 1) == (c >> 1)) {
          er = S.K[2 * ((r & 1) * 2 + (c & 1))];
          ei = S.K[2 * ((r & 1) * 2 + (c & 1)) + 1];
        }
      }
      S.E[2 * t] = er;
      S.E[2 * t + 1] = ei;
    }
    __syncwarp(mask);
    // M <- E M; rho <- E rho E^dagger (every read of M and rho before the barrier,
    // every write after it)
    double sr = 0, si = 0;
    if (ent) {
      double tr_ = 0, ti = 0;
      for (int k = 0; k < D; ++k) {
        const double ar = S.E[2 * (r * D + k)], ai = S.E[2 * (r * D + k) + 1];
        const double br = S.M[2 * (k * D + c)], bi = S.M[2 * (k * D + c) + 1];
        sr += ar * br - ai * bi;
        si += ar * bi + ai * br;
        if (g.need_rho) {
          const double cr = S.rho[2 * (k * D + c)], ci = S.rho[2 * (k * D + c) + 1];
          tr_ += ar * cr - ai * ci;
          ti += ar * ci + ai * cr;
        }
      }
      S.tmp[2 * t] = tr_;
      S.tmp[2 * t + 1] = ti;
    }
    __syncwarp(mask);
    if (ent) {
      S.M[2 * t] = sr;
      S.M[2 * t + 1] = si;
      if (g.need_rho) {
        double qr = 0, qi = 0;
        for (int k = 0; k < D; ++k) {
          const double xr = S.tmp[2 * (r * D + k)], xi = S.tmp[2 * (r * D + k) + 1];
          const double er = S.E[2 * (c * D + k)], ei = -S.E[2 * (c * D + k) + 1];  // conj(E[c][k])
          qr += xr * er - xi * ei;
          qi += xr * ei + xi * er;
        }
        S.rho[2 * t] = qr;
        S.rho[2 * t + 1] = qi;
      }
    }
    __syncwarp(mask);
  }
  if (ent) {
    R* out = mat_out + (int64_t)m * 32;
    out[2 * t] = (R)S.M[2 * t];
    out[2 * t + 1] = (R)S.M[2 * t + 1];
  }
}

// ------------------------------------------------------------------ host API
static int prog_qubits(bt_program* p, int k, const int32_t* q) {
  if (k < 1 || k > 2 || !q) return bt_fail(p->ctx, BT_ERR_UNSUPPORTED, "program ops act on 1 or 2 qubits");
  for (int i = 0; i < k; ++i)
    if (q[i] < 1 || q[i] > p->n) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "N must be larger than qubits");
  if (k == 2 && q[0] == q[1]) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "qubits must differ");
  return BT_OK;
}

static int prog_skip(bt_program* p, const int32_t* skip) {
  if (!skip) return -1;
  const int off = (int)p->skip.size();
  for (int m = 0; m < p->batch; ++m) p->skip.push_back(skip[m] ? 1 : 0);
  return off;
}

extern "C" {

int bt_program_create(bt_ctx* ctx, int n, int prec, int batch, bt_program** out) {
  if (!ctx || !out) return bt_fail(ctx, BT_ERR_BAD_ARG, "NULL argument");
  if (prec != BT_PREC_C128 && prec != BT_PREC_C64) return bt_fail(ctx, BT_ERR_BAD_ARG, "prec must be C128 or C64");
  if (n < 2 || n > 34) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "programs take 2 <= n <= 34 qubits");
  if (batch < 1 || batch > (1 << 30)) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad batch");
  bt_program* p = new bt_program();
  p->ctx = ctx;
  p->device = ctx->device;
  p->n = n;
  p->prec = prec;
  p->batch = batch;
  *out = p;
  return BT_OK;
}

int bt_program_free(bt_program* p) {
  if (!p) return BT_OK;
  // cudaFree waits for the device; the program's context may already be gone
  cudaSetDevice(p->device);
  for (void* d : {p->d_ops, p->d_gm, p->d_km, p->d_skip, p->d_rec, p->d_u, p->d_gact, p->d_rho, p->d_mat})
    if (d) cudaFree(d);
  delete p;
  return BT_OK;
}

int bt_program_set_range(bt_program* p, int64_t lo, int64_t hi) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  if (hi < 0) hi = p->batch;
  if (lo < 0 || lo >= hi || hi > p->batch) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "member range outside the batch");
  p->range_lo = (int)lo;
  p->range_hi = (int)hi;
  return BT_OK;
}

int bt_program_add_gate(bt_program* p, int k, const int32_t* qubits, const double* mats, int per_member) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  int rc = prog_qubits(p, k, qubits);
  if (rc) return rc;
  if (!mats) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "matrix is NULL");
  const int d = 1 << k;
  const int lo = p->range_lo, hi = p->range_hi < 0 ? p->batch : p->range_hi;
  const int cnt = per_member ? hi - lo : 1;
  PGOp op = {};
  op.mlo = lo;
  op.mhi = hi;
  op.type = k == 1 ? PG_GATE1 : PG_GATE2;
  op.b0 = p->n - qubits[0];
  op.b1 = k == 2 ? p->n - qubits[1] : 0;
  op.moff = (int)p->gm.size();
  op.mstride = per_member ? 2 * d * d : 0;
  op.skip_off = -1;
  op.rand_idx = -1;
  for (int m = 0; m < cnt; ++m) {
    const double* cm = mats + (size_t)m * 2 * d * d;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        p->gm.push_back(cm[2 * (r + c * d)]);
        p->gm.push_back(cm[2 * (r + c * d) + 1]);
      }
  }
  p->ops.push_back(op);
  p->uploaded = false;
  return BT_OK;
}

int bt_program_add_channel(bt_program* p, int k, const int32_t* qubits, int nk, const double* kraus, int flags,
                           const int32_t* skip) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  int rc = prog_qubits(p, k, qubits);
  if (rc) return rc;
  if (nk < 1 || !kraus) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "need at least one Kraus operator");
  if (nk > PG_MAX_KRAUS) return bt_fail(p->ctx, BT_ERR_UNSUPPORTED, "programs take at most 64 Kraus operators per channel");
  const int d = 1 << k;
  PGOp op = {};
  op.mlo = p->range_lo;
  op.mhi = p->range_hi < 0 ? p->batch : p->range_hi;
  op.type = PG_CHANNEL;
  op.k = k;
  op.nk = nk;
  op.b0 = p->n - qubits[0];
  op.b1 = k == 2 ? p->n - qubits[1] : 0;
  op.flags = ((flags & BT_KRAUS_REF_ORDER) && k == 2 && qubits[0] > qubits[1] ? 1 : 0) |
             ((flags & BT_KRAUS_UNITARY_MIX) ? 2 : 0);
  op.moff = (int)p->km.size();
  op.skip_off = prog_skip(p, skip);
  op.rand_idx = p->ndraws++;
  for (int i = 0; i < nk; ++i) {
    const double* K = kraus + (size_t)i * 2 * d * d;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        p->km.push_back(K[2 * (r + c * d)]);
        p->km.push_back(K[2 * (r + c * d) + 1]);
      }
  }
  p->ops.push_back(op);
  p->uploaded = false;
  return BT_OK;
}

int bt_program_add_measure(bt_program* p, int qubit, const int32_t* skip) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  int rc = prog_qubits(p, 1, &qubit);
  if (rc) return rc;
  PGOp op = {};
  op.mlo = p->range_lo;
  op.mhi = p->range_hi < 0 ? p->batch : p->range_hi;
  op.type = PG_MEASURE;
  op.b0 = p->n - qubit;
  op.skip_off = prog_skip(p, skip);
  op.rand_idx = p->ndraws++;
  op.rec_idx = p->nrec++;
  p->ops.push_back(op);
  p->uploaded = false;
  return BT_OK;
}

static bool use_grouped(const bt_program* p);

int bt_program_set_gate(bt_program* p, int64_t op_index, const double* mats) {
  if (!p || !mats) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "NULL argument");
  if (op_index < 0 || op_index >= (int64_t)p->ops.size())
    return bt_fail(p->ctx, BT_ERR_BAD_ARG, "op index out of range");
  const PGOp& op = p->ops[op_index];
  if (op.type != PG_GATE1 && op.type != PG_GATE2) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "op is not a gate");
  // the grouped executor's member activity depends on which matrices are identities
  if (op.mstride && use_grouped(p)) p->uploaded = false;
  const int d = op.type == PG_GATE1 ? 2 : 4;
  const int cnt = op.mstride ? op.mhi - op.mlo : 1;
  double* dst = p->gm.data() + op.moff;
  for (int m = 0; m < cnt; ++m) {
    const double* cm = mats + (size_t)m * 2 * d * d;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        *dst++ = cm[2 * (r + c * d)];
        *dst++ = cm[2 * (r + c * d) + 1];
      }
  }
  if (p->uploaded) p->gm_dirty = true;
  return BT_OK;
}

int bt_program_info(const bt_program* p, int64_t* nops, int64_t* ndraws, int64_t* nrecords) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  if (nops) *nops = (int64_t)p->ops.size();
  if (ndraws) *ndraws = p->ndraws;
  if (nrecords) *nrecords = p->nrec;
  return BT_OK;
}

int bt_program_set_executor(bt_program* p, int executor) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  if (executor < 0 || executor > 2) return bt_fail(p->ctx, BT_ERR_BAD_ARG, "executor must be 0, 1 or 2");
  if (executor == 1 && p->n > (p->prec == BT_PREC_C64 ? 14 : 13))
    return bt_fail(p->ctx, BT_ERR_UNSUPPORTED, "a member of more than 14 (c64) / 13 (c128) qubits exceeds shared memory");
  if (p->executor != executor) p->uploaded = false;
  p->executor = executor;
  return BT_OK;
}

static bool use_grouped(const bt_program* p) {
  return p->executor == 2 || (p->executor == 0 && p->n > (p->prec == BT_PREC_C64 ? 14 : 13));
}

// groups of consecutive ops within at most two qubits, and per group and member
// whether the member does anything in it
static void form_groups(bt_program* p, std::vector<int8_t>& gact) {
  p->groups.clear();
  auto bits_of = [](const PGOp& o, int* b) {
    b[0] = o.b0;
    const int k = o.type == PG_GATE2 ? 2 : (o.type == PG_CHANNEL ? o.k : 1);
    if (k == 2) b[1] = o.b1;
    return k;
  };
  for (size_t i = 0; i < p->ops.size();) {
    PGGroup g = {};
    int b[2];
    const int k = bits_of(p->ops[i], b);
    g.nb = k;
    g.q0 = b[0];
    g.q1 = k == 2 ? b[1] : -1;
    g.op0 = (int)i;
    size_t j = i;
    for (; j < p->ops.size(); ++j) {
      int c[2];
      const int kc = bits_of(p->ops[j], c);
      bool fits = true;
      for (int e = 0; e < kc && fits; ++e) {
        if (c[e] == g.q0 || c[e] == g.q1) continue;
        if (g.nb == 1) {  // a one-qubit group takes a second qubit
          g.nb = 2;
          g.q1 = c[e];
        } else {
          fits = false;
        }
      }
      if (!fits) break;
      const PGOp& o = p->ops[j];
      if (o.type == PG_MEASURE || (o.type == PG_CHANNEL && !(o.flags & 2))) g.need_rho = 1;
    }
    g.nop = (int)(j - i);
    p->groups.push_back(g);
    i = j;
  }
  // a member is active in a group when one of the group's ops does something to
  // it: not skipped, and for a gate with per-member matrices not exactly the
  // identity (members whose op sequence is shorter at a position -- trajectories
  // beside ZNE or twirled copies in one batch -- carry identities there)
  auto identity = [](const double* m, int d) {
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c)
        if (m[2 * (r * d + c)] != (r == c ? 1.0 : 0.0) || m[2 * (r * d + c) + 1] != 0.0) return false;
    return true;
  };
  gact.assign(p->groups.size() * (size_t)p->batch, 0);
  for (size_t gi = 0; gi < p->groups.size(); ++gi) {
    PGGroup& g = p->groups[gi];
    int8_t* row = gact.data() + gi * p->batch;
    for (int oi = g.op0; oi < g.op0 + g.nop; ++oi) {
      const PGOp& o = p->ops[oi];
      const bool gate = o.type == PG_GATE1 || o.type == PG_GATE2;
      const int d = o.type == PG_GATE1 ? 2 : 4;
      for (int m = o.mlo; m < o.mhi; ++m) {
        if (o.skip_off >= 0 && p->skip[o.skip_off + m]) continue;
        if (gate && o.mstride && identity(p->gm.data() + o.moff + (size_t)(m - o.mlo) * o.mstride, d)) continue;
        row[m] = 1;
      }
    }
    // the launches of the group cover its first to last active member only
    g.mlo = 0;
    g.mhi = 0;
    for (int m = 0; m < p->batch; ++m)
      if (row[m]) {
        if (g.mhi == 0) g.mlo = m;
        g.mhi = m + 1;
      }
  }
}

static int upload(bt_program* p) {
  bt_ctx* ctx = p->ctx;
  for (void** d : {&p->d_gact, &p->d_rho, &p->d_mat})
    if (*d) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(*d);
      *d = nullptr;
    }
  if (use_grouped(p)) {
    std::vector<int8_t> gact;
    form_groups(p, gact);
    int rc = bt_cuda_check(ctx, cudaMalloc(&p->d_gact, gact.size() ? gact.size() : 16), "program allocation");
    if (!rc && gact.size())
      rc = bt_cuda_check(ctx, cudaMemcpy(p->d_gact, gact.data(), gact.size(), cudaMemcpyHostToDevice), "program upload");
    if (!rc) rc = bt_cuda_check(ctx, cudaMalloc(&p->d_rho, (size_t)p->batch * 32 * 8), "program allocation");
    if (!rc) rc = bt_cuda_check(ctx, cudaMalloc(&p->d_mat, (size_t)p->batch * 32 * elem_bytes(p->prec) / 2),
                                "program allocation");
    if (rc) return rc;
  }
  for (void** d : {&p->d_ops, &p->d_gm, &p->d_km, &p->d_skip, &p->d_rec})
    if (*d) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(*d);
      *d = nullptr;
    }
  const bool f = p->prec == BT_PREC_C64;
  std::vector<float>& gf = p->gstage;
  if (f) gf.assign(p->gm.begin(), p->gm.end());
  const size_t gbytes = f ? gf.size() * 4 : p->gm.size() * 8;
  struct Buf { void** d; const void* h; size_t bytes; };
  const Buf bufs[] = {{&p->d_ops, p->ops.data(), p->ops.size() * sizeof(PGOp)},
                      {&p->d_gm, f ? (const void*)gf.data() : (const void*)p->gm.data(), gbytes},
                      {&p->d_km, p->km.data(), p->km.size() * 8},
                      {&p->d_skip, p->skip.data(), p->skip.size()},
                      {&p->d_rec, nullptr, (size_t)p->batch * (p->nrec ? p->nrec : 1) * 4}};
  for (const Buf& b : bufs) {
    int rc = bt_cuda_check(ctx, cudaMalloc(b.d, b.bytes ? b.bytes : 16), "program allocation");
    if (rc) return rc;
    if (b.h && b.bytes) {
      rc = bt_cuda_check(ctx, cudaMemcpy(*b.d, b.h, b.bytes, cudaMemcpyHostToDevice), "program upload");
      if (rc) return rc;
    }
  }
  p->uploaded = true;
  p->gm_dirty = false;
  return BT_OK;
}

// re-sends the gate matrices after bt_program_set_gate (same size, stream-ordered)
static int upload_gm(bt_program* p, bt_ctx* ctx) {
  const bool f = p->prec == BT_PREC_C64;
  if (f) p->gstage.assign(p->gm.begin(), p->gm.end());
  const void* h = f ? (const void*)p->gstage.data() : (const void*)p->gm.data();
  const size_t bytes = f ? p->gstage.size() * 4 : p->gm.size() * 8;
  p->gm_dirty = false;
  if (!bytes) return BT_OK;
  return bt_cuda_check(ctx, cudaMemcpyAsync(p->d_gm, h, bytes, cudaMemcpyHostToDevice, ctx->stream), "gate upload");
}

static void launch_program(bt_program* p, bt_state* s, const double* du, uint64_t stream, int nrec);

int bt_program_prepare(bt_program* p, bt_ctx* ctx) {
  if (!p || !ctx) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "NULL argument");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!rc && !p->uploaded) rc = upload(p);
  if (!rc && p->gm_dirty) rc = upload_gm(p, ctx);
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "program prepare");
  return rc;
}

int bt_program_run(bt_program* p, bt_state* s, const double* uniforms, uint64_t seed, int32_t* records) {
  if (!p || !s) return bt_fail(p ? p->ctx : nullptr, BT_ERR_BAD_ARG, "NULL argument");
  bt_ctx* ctx = s->ctx;
  if (s->repr != BT_REPR_SV || s->n != p->n || s->prec != p->prec || s->batch != p->batch)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "program and state differ in n, prec or batch (or the state is a density matrix)");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  if (!p->uploaded && (rc = upload(p))) return rc;
  if (p->gm_dirty && (rc = upload_gm(p, ctx))) return rc;
  const double* du = nullptr;
  if (uniforms && p->ndraws) {
    const size_t ub = (size_t)p->ndraws * p->batch * 8;
    if (p->u_bytes < ub) {
      if (p->d_u) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(p->d_u);
      }
      if ((rc = bt_cuda_check(ctx, cudaMalloc(&p->d_u, ub), "draw buffer"))) return rc;
      p->u_bytes = ub;
    }
    if ((rc = bt_cuda_check(ctx, cudaMemcpyAsync(p->d_u, uniforms, ub, cudaMemcpyHostToDevice, ctx->stream), "draws")))
      return rc;
    du = (const double*)p->d_u;
  }
  const bool f = p->prec == BT_PREC_C64;
  // draws depend on (ctx seed, seed) only, as bt_sample's: a run is reproducible
  const uint64_t stream = (seed * 0x9E3779B97F4A7C15ULL) ^ 0x5052000000000000ULL;
  const int nrec = p->nrec ? p->nrec : 1;
  if (use_grouped(p)) {
    // per group: reduce rho_Q (when a decision needs it), decide per member,
    // apply the chosen matrices; members idle in a group are neither read nor written
    // records of members a group does not reach stay -1
    if (p->nrec && (rc = bt_cuda_check(ctx, cudaMemsetAsync(p->d_rec, 0xFF, (size_t)p->batch * p->nrec * 4,
                                                            ctx->stream), "records")))
      return rc;
    const int8_t* gact = (const int8_t*)p->d_gact;
    for (size_t gi = 0; gi < p->groups.size() && !rc; ++gi) {
      const PGGroup& g = p->groups[gi];
      if (g.mhi <= g.mlo) continue;  // no member acts in this group
      const int8_t* act = gact + gi * p->batch;
      const int bits[2] = {g.q0, g.q1};
      const int D = 1 << g.nb;
      const int64_t nm = g.mhi - g.mlo;
      if (g.need_rho) rc = bt_launch_rdm(s, g.nb, bits, g.mlo, nm, (double*)p->d_rho, act);
      if (rc) break;
      const unsigned grid = (unsigned)((nm + PGD_TEAMS - 1) / PGD_TEAMS);
      if (f)
        k_group_decide<float><<<grid, PGD_TEAM * PGD_TEAMS, 0, ctx->stream>>>(
            g, (const PGOp*)p->d_ops, (const float*)p->d_gm, (const double*)p->d_km, (const int8_t*)p->d_skip, act,
            du, ctx->seed, stream, p->batch, (const double*)p->d_rho, (float*)p->d_mat, (int32_t*)p->d_rec, nrec,
            ctx->d_status);
      else
        k_group_decide<double><<<grid, PGD_TEAM * PGD_TEAMS, 0, ctx->stream>>>(
            g, (const PGOp*)p->d_ops, (const double*)p->d_gm, (const double*)p->d_km, (const int8_t*)p->d_skip, act,
            du, ctx->seed, stream, p->batch, (const double*)p->d_rho, (double*)p->d_mat, (int32_t*)p->d_rec, nrec,
            ctx->d_status);
      ctx->launches++;
      if ((rc = bt_cuda_check(ctx, cudaGetLastError(), "group decide launch"))) break;
      rc = bt_launch_gate(s, g.nb, bits, nullptr, 0, g.mlo, nm, p->d_mat, 32, act);
      (void)D;
    }
    if (rc) return rc;
  } else {
    static std::atomic<bool> attr[2][64] = {};
    std::atomic<bool>& done = attr[f][ctx->device & 63];
    if (!done.load()) {
      cudaError_t e = f ? cudaFuncSetAttribute(k_program<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)
                        : cudaFuncSetAttribute(k_program<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if ((rc = bt_cuda_check(ctx, e, "program smem attribute"))) return rc;
      done.store(true);
    }
    launch_program(p, s, du, stream, nrec);
  }
  if ((rc = bt_cuda_check(ctx, cudaGetLastError(), "program launch"))) return rc;
  if (records && p->nrec)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(records, p->d_rec, (size_t)p->batch * p->nrec * 4, cudaMemcpyDeviceToHost,
                                            ctx->stream), "records");
  if (rc) return rc;
  rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "program sync");
  if (rc) return rc;
  int st = 0;
  rc = bt_cuda_check(ctx, cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
  if (rc) return rc;
  if (st) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return bt_fail(ctx, st == 1 ? BT_ERR_BAD_ARG : (st == 2 ? BT_ERR_NO_BRANCH : BT_ERR_BAD_ARG),
                   "a program branch or outcome had zero probability; that member kept its state");
  }
  return BT_OK;
}

}  // extern "C"

static void launch_program(bt_program* p, bt_state* s, const double* du, uint64_t stream, int nrec) {
  bt_ctx* ctx = s->ctx;
  const size_t smem = (elem_bytes(p->prec) << p->n) + (9 * 32 + 2 * PG_MAX_KRAUS) * 8 + 32 * 8;
  if (p->prec == BT_PREC_C64)
    k_program<float><<<p->batch, PG_THREADS, smem, ctx->stream>>>(
        (float2*)s->d, s->nbits, (const PGOp*)p->d_ops, (int)p->ops.size(), (const float*)p->d_gm,
        (const double*)p->d_km, (const int8_t*)p->d_skip, du, ctx->seed, stream, p->batch, (int32_t*)p->d_rec,
        nrec, ctx->d_status);
  else
    k_program<double><<<p->batch, PG_THREADS, smem, ctx->stream>>>(
        (double2*)s->d, s->nbits, (const PGOp*)p->d_ops, (int)p->ops.size(), (const double*)p->d_gm,
        (const double*)p->d_km, (const int8_t*)p->d_skip, du, ctx->seed, stream, p->batch, (int32_t*)p->d_rec,
        nrec, ctx->d_status);
  ctx->launches++;
}

// ------------------------------------------------------------------ serving hook (bt_serve.cu)
// matrix dimension of every op (0 where the op is not a gate) and the shape
int bt_program_gate_dims(const bt_program* p, std::vector<int>& dims, int* n, int* prec, int* batch,
                         std::vector<char>* per_member) {
  if (!p) return bt_fail(nullptr, BT_ERR_BAD_ARG, "program is NULL");
  dims.assign(p->ops.size(), 0);
  for (size_t i = 0; i < p->ops.size(); ++i)
    dims[i] = p->ops[i].type == PG_GATE1 ? 2 : (p->ops[i].type == PG_GATE2 ? 4 : 0);
  if (per_member) {
    per_member->assign(p->ops.size(), 0);
    for (size_t i = 0; i < p->ops.size(); ++i) (*per_member)[i] = dims[i] && p->ops[i].mstride != 0;
  }
  *n = p->n;
  *prec = p->prec;
  *batch = p->batch;
  return BT_OK;
}
