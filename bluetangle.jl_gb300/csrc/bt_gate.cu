// Gate sweeps: op.expand(N)*state for dense k-qubit matrices (k <= 5), the
// replacement of the reference's full-space sparse operator construction and
// SpMV (BlueTangle.jl src/hilbert.jl:143-159, :18-70, :106-128, :505).
//
// One thread owns V adjacent groups of 2^k amplitudes (a group = the 2^k
// amplitudes that differ only in the target bits).  Each pass reads and writes
// every touched amplitude once: 2 * 2^nbits * sizeof(complex) bytes per member
// (half that when a control bit must read 1), which makes a sweep HBM-bound
// for c64 and, for dense matrices, FP64-issue-bound for c128 on GB300.
//
// The matrix arrives by value in the kernel parameters (constant bank, read
// uniformly by the warp) or, for per-member matrices (trajectory branches), from
// global memory.  For c64 with no target or control on bit 0, V = 2 and every
// access is a 16-byte float4; c128 amplitudes are 16-byte double2 already.
#include "bt_internal.cuh"

template <typename R, int K>
struct GateArgs {
  R m[2 * (1 << K) * (1 << K)];  // row-major interleaved: m[2*(r*D+c)], m[2*(r*D+c)+1]
  int bits[K];                   // bits[0] = most significant bit of the matrix index
  int sorted[K];                 // ascending
  uint64_t cmask;
  int nbits;
  int lg_per;                    // log2(thread-units per member)
  int64_t member_lo, nmem;
  const R* per_member;           // optional [member][2*D*D]
  int64_t pm_stride;
  const int8_t* active;          // optional [member]: 0 = leave the member untouched
};

template <typename R, int V> struct VecIO;
template <> struct VecIO<float, 2> {
  static __device__ __forceinline__ void load(const float2* p, float (&re)[2], float (&im)[2]) {
    float4 v = *reinterpret_cast<const float4*>(p);
    re[0] = v.x; im[0] = v.y; re[1] = v.z; im[1] = v.w;
  }
  static __device__ __forceinline__ void store(float2* p, const float (&re)[2], const float (&im)[2]) {
    *reinterpret_cast<float4*>(p) = make_float4(re[0], im[0], re[1], im[1]);
  }
};
template <typename R> struct VecIO<R, 1> {
  typedef typename CT<R>::T C2;
  static __device__ __forceinline__ void load(const C2* p, R (&re)[1], R (&im)[1]) {
    C2 v = *p;
    re[0] = v.x; im[0] = v.y;
  }
  static __device__ __forceinline__ void store(C2* p, const R (&re)[1], const R (&im)[1]) {
    C2 v; v.x = re[0]; v.y = im[0];
    *p = v;
  }
};

template <typename R, int K, int V>
__global__ void __launch_bounds__(BT_THREADS) k_gate(typename CT<R>::T* __restrict__ psi,
                                                     const GateArgs<R, K> a) {
  constexpr int D = 1 << K;
  typedef typename CT<R>::T C2;
  int64_t off[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    int64_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> (K - 1 - b)) & 1) o |= 1LL << a.bits[b];
    off[j] = o;
  }
  const int64_t per = 1LL << a.lg_per;
  const int64_t total = per * a.nmem;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
    const int64_t mem = a.member_lo + (t >> a.lg_per);
    uint64_t base = (uint64_t)(t & (per - 1)) * V;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int p = a.sorted[i];
      base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
    }
    if ((base & a.cmask) != a.cmask) continue;
    if (a.active && !a.active[mem]) continue;
    C2* s = psi + (mem << a.nbits) + base;
    const R* m = a.per_member ? a.per_member + mem * a.pm_stride : a.m;
    R xr[D][V], xi[D][V];
#pragma unroll
    for (int j = 0; j < D; ++j) VecIO<R, V>::load(s + off[j], xr[j], xi[j]);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      R yr[V], yi[V];
#pragma unroll
      for (int v = 0; v < V; ++v) { yr[v] = 0; yi[v] = 0; }
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const R mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
#pragma unroll
        for (int v = 0; v < V; ++v) {
          yr[v] = fma(mr, xr[c][v], fma(-mi, xi[c][v], yr[v]));
          yi[v] = fma(mr, xi[c][v], fma(mi, xr[c][v], yi[v]));
        }
      }
      VecIO<R, V>::store(s + off[r], yr, yi);
    }
  }
}

template <typename R, int K, int V>
static int launch_t(bt_state* s, const int* bits, const double* m, uint64_t cmask, int64_t mem_lo,
                    int64_t nmem, const void* per_member, int64_t pm_stride, const int8_t* active) {
  constexpr int D = 1 << K;
  GateArgs<R, K> a;
  for (int i = 0; i < 2 * D * D; ++i) a.m[i] = m ? (R)m[i] : (R)0;
  for (int i = 0; i < K; ++i) a.bits[i] = a.sorted[i] = bits[i];
  for (int i = 0; i < K; ++i)
    for (int j = i + 1; j < K; ++j)
      if (a.sorted[j] < a.sorted[i]) { int t = a.sorted[i]; a.sorted[i] = a.sorted[j]; a.sorted[j] = t; }
  a.cmask = cmask;
  a.nbits = s->nbits;
  int lgv = V == 2 ? 1 : 0;
  a.lg_per = s->nbits - K - lgv;
  a.member_lo = mem_lo;
  a.nmem = nmem;
  a.per_member = (const R*)per_member;
  a.pm_stride = pm_stride;
  a.active = active;
  int64_t work = (1LL << a.lg_per) * nmem;
  int grid = bt_grid(s->ctx, work, BT_THREADS, 32);
  k_gate<R, K, V><<<grid, BT_THREADS, 0, s->ctx->stream>>>((typename CT<R>::T*)s->d, a);
  s->ctx->launches++;
  return bt_cuda_check(s->ctx, cudaGetLastError(), "gate kernel launch");
}

template <typename R>
static int launch_r(bt_state* s, int k, const int* bits, const double* m, uint64_t cmask, int64_t mem_lo,
                    int64_t nmem, const void* pm, int64_t pms, const int8_t* active) {
  int minbit = 64;
  for (int i = 0; i < k; ++i) minbit = bits[i] < minbit ? bits[i] : minbit;
  bool vec2 = sizeof(R) == 4 && minbit >= 1 && !(cmask & 1ULL) && s->nbits - k >= 1;
  if constexpr (sizeof(R) == 4) {
    if (vec2) {
      switch (k) {
        case 1: return launch_t<R, 1, 2>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
        case 2: return launch_t<R, 2, 2>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
        case 3: return launch_t<R, 3, 2>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
        case 4: return launch_t<R, 4, 2>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
        case 5: return launch_t<R, 5, 2>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
      }
    }
  }
  {
    switch (k) {
      case 1: return launch_t<R, 1, 1>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
      case 2: return launch_t<R, 2, 1>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
      case 3: return launch_t<R, 3, 1>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
      case 4: return launch_t<R, 4, 1>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
      case 5: return launch_t<R, 5, 1>(s, bits, m, cmask, mem_lo, nmem, pm, pms, active);
    }
  }
  return bt_fail(s->ctx, BT_ERR_UNSUPPORTED, "gate sweep supports 1 <= k <= 5");
}

int bt_launch_gate(bt_state* s, int k, const int* bits, const double* m_rowmajor, uint64_t cmask,
                   int64_t mem_lo, int64_t nmem, const void* per_member, int64_t pm_stride, const int8_t* active) {
  if (k < 1 || k > BT_MAX_K || k > s->nbits)
    return bt_fail(s->ctx, BT_ERR_UNSUPPORTED, "gate sweep supports 1 <= k <= 5 target qubits");
  if (nmem <= 0) return BT_OK;
  if (s->prec == BT_PREC_C64)
    return launch_r<float>(s, k, bits, m_rowmajor, cmask, mem_lo, nmem, per_member, pm_stride, active);
  return launch_r<double>(s, k, bits, m_rowmajor, cmask, mem_lo, nmem, per_member, pm_stride, active);
}
