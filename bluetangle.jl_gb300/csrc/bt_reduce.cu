// Reductions (FP64 accumulation; complex64 states form 8-term FP32 micro-sums
// first, see Micro below), measurement collapse, density-matrix dephasing and
// the device-side branch/outcome decisions.
//
// Every reduction writes one partial per (member, block) and a second kernel
// sums the partials of a member in a fixed order, so results are bit-for-bit
// reproducible run to run.  Replaces the reference's partial traces
// (BlueTangle.jl src/linalg.jl:83-230), Born probabilities
// (src/hilbert.jl:682-696), Kraus branch probabilities (src/struct.jl:9-29)
// and observables (src/func.jl:91-147).
#include <string.h>

#include <algorithm>
#include <atomic>

#include "bt_internal.cuh"

#define FULL 0xffffffffu

// ------------------------------------------------------------ block reduce
// sums acc[0..W-1] over the block and writes the W results to out (thread 0..W-1)
template <int W>
__device__ __forceinline__ void block_sum_store(double (&acc)[W], double* out, int wcount) {
  __shared__ double sh[BT_THREADS / 32][W];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    double v = acc[w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    if (lane == 0) sh[warp][w] = v;
  }
  __syncthreads();
  for (int w = threadIdx.x; w < wcount; w += blockDim.x) {
    double s = 0;
#pragma unroll
    for (int i = 0; i < BT_THREADS / 32; ++i) s += sh[i][w];
    out[w] = s;
  }
}

// out[mem][w] = sum over blocks of part[mem][blk][w] (fixed order)
__global__ void k_finalize(const double* __restrict__ part, int nblk, int W, double* __restrict__ out) {
  const int64_t mem = blockIdx.x;
  for (int w = threadIdx.x; w < W; w += blockDim.x) {
    double s = 0;
    const double* p = part + (mem * nblk) * W + w;
    for (int b = 0; b < nblk; ++b) s += p[(int64_t)b * W];
    out[mem * W + w] = s;
  }
}

// Micro-sums.  GB300 issues FP64 at a small fraction of its FP32 rate, so a
// complex64 reduction that forms every product and every partial sum in FP64 is
// bound by FP64 issue, far below HBM speed.  For complex64 states each thread
// forms products and sums MICRO consecutive terms of its grid-stride sequence in
// FP32 (relative error <= MICRO * 2^-24 per group, below the rounding the
// complex64 amplitudes already carry) and adds each group to FP64 accumulators;
// every longer sum -- over groups, threads, blocks -- is FP64, in a fixed order.
// complex128 states keep FP64 throughout.
template <typename R> struct Micro { typedef double T; enum { J = 1 }; };
template <> struct Micro<float> { typedef float T; enum { J = 8 }; };

// Hermitian packing of a D x D reduced matrix: D real diagonal entries, then
// (re, im) of each a < b; herm_index gives the packed slots of entry (a, b).
template <int D>
__device__ __forceinline__ int herm_re(int a, int b) {
  if (a == b) return a;
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  // pairs (lo, hi) in row order: before row lo come sum_{r<lo} (D-1-r) pairs
  const int pair = lo * (2 * D - lo - 1) / 2 + (hi - lo - 1);
  return D + 2 * pair;
}

// blocks per member for a reduction over `units` thread-units per member
static int blocks_per_member(const bt_ctx* ctx, int64_t units, int64_t nmem) {
  int64_t want = (int64_t)ctx->sm_count * 8;
  int64_t per = (want + nmem - 1) / nmem;
  int64_t maxb = (units + BT_THREADS - 1) / BT_THREADS;
  if (per > maxb) per = maxb;
  if (per > 1024) per = 1024;
  if (per < 1) per = 1;
  return (int)per;
}

static int finalize(bt_ctx* ctx, double* part, int nblk, int W, int64_t nmem, double* out) {
  k_finalize<<<(unsigned)nmem, 64, 0, ctx->stream>>>(part, nblk, W, out);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "finalize launch");
}

// partials live in ctx->work, a device buffer separate from ctx->scratch so that
// they never alias API-level results and tables carved from the scratch buffer
int bt_work(bt_ctx* ctx, size_t bytes, double** out) {
  if (ctx->work_bytes < bytes) {
    if (ctx->work) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->work);
      ctx->work = nullptr;
      ctx->work_bytes = 0;
    }
    size_t nb = bytes < (1u << 20) ? (1u << 20) : bytes;
    cudaError_t e = cudaMalloc(&ctx->work, nb);
    if (e != cudaSuccess) return bt_fail(ctx, BT_ERR_OOM, "reduction workspace allocation failed");
    ctx->work_bytes = nb;
  }
  *out = (double*)ctx->work;
  return BT_OK;
}

// ------------------------------------------------------------ reduced density matrix
template <typename R, int K>
__global__ void __launch_bounds__(BT_THREADS) k_rdm(const typename CT<R>::T* __restrict__ psi, int nbits,
                                                    int4 bits4, int4 sorted4, int64_t mem_lo, int nblk,
                                                    double* __restrict__ part, const int8_t* __restrict__ active) {
  constexpr int D = 1 << K, W = 2 * D * D;
  const int bits[4] = {bits4.x, bits4.y, bits4.z, bits4.w};
  const int sorted[4] = {sorted4.x, sorted4.y, sorted4.z, sorted4.w};
  int64_t off[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    int64_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> (K - 1 - b)) & 1) o |= 1LL << bits[b];
    off[j] = o;
  }
  const int64_t mem = mem_lo + blockIdx.y;
  const typename CT<R>::T* s = psi + (mem << nbits);
  // an inactive member reads nothing and gets a zero matrix
  const int64_t ng = (!active || active[mem]) ? (1LL << (nbits - K)) : 0;
  const int64_t stride = (int64_t)nblk * blockDim.x;
  if constexpr (K <= 2) {
    // Hermitian: accumulate the D*D packed reals, expand to the full matrix at the end
    typedef typename Micro<R>::T A;
    constexpr int WH = D * D, J = Micro<R>::J;
    double acc[WH];
#pragma unroll
    for (int w = 0; w < WH; ++w) acc[w] = 0;
    for (int64_t g0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g0 < ng; g0 += stride * J) {
      A f[WH];
#pragma unroll
      for (int w = 0; w < WH; ++w) f[w] = 0;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t g = g0 + jj * stride;
        if (g >= ng) break;
        uint64_t base = (uint64_t)g;
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const int p = sorted[i];
          base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
        }
        A xr[D], xi[D];
#pragma unroll
        for (int j = 0; j < D; ++j) {
          typename CT<R>::T v = s[base + off[j]];
          xr[j] = (A)v.x;
          xi[j] = (A)v.y;
        }
#pragma unroll
        for (int a = 0; a < D; ++a) {
          f[a] += xr[a] * xr[a] + xi[a] * xi[a];
#pragma unroll
          for (int b = a + 1; b < D; ++b) {
            const int r = herm_re<D>(a, b);
            f[r] += xr[a] * xr[b] + xi[a] * xi[b];      // Re x_a conj(x_b)
            f[r + 1] += xi[a] * xr[b] - xr[a] * xi[b];  // Im x_a conj(x_b)
          }
        }
      }
#pragma unroll
      for (int w = 0; w < WH; ++w) acc[w] += (double)f[w];
    }
    // block reduction of the packed sums, then the full row-major matrix
    __shared__ double sh[BT_THREADS / 32][WH];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int w = 0; w < WH; ++w) {
      double v = acc[w];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
      if (lane == 0) sh[warp][w] = v;
    }
    __syncthreads();
    double* out = part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * W;
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
      const int e = w >> 1, a = e / D, b = e % D, im = w & 1;
      double v = 0;
      if (a == b) {
        if (!im)
          for (int i = 0; i < BT_THREADS / 32; ++i) v += sh[i][a];
      } else {
        const int r = herm_re<D>(a, b) + im;
        for (int i = 0; i < BT_THREADS / 32; ++i) v += sh[i][r];
        if (im && a > b) v = -v;  // rho[a, b] = conj(rho[b, a])
      }
      out[w] = v;
    }
  } else {
    double acc[W];
#pragma unroll
    for (int w = 0; w < W; ++w) acc[w] = 0;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += stride) {
      uint64_t base = (uint64_t)g;
#pragma unroll
      for (int i = 0; i < K; ++i) {
        const int p = sorted[i];
        base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
      }
      double xr[D], xi[D];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        typename CT<R>::T v = s[base + off[j]];
        xr[j] = (double)v.x;
        xi[j] = (double)v.y;
      }
      // rho[a, b] += x_a conj(x_b), row-major interleaved
#pragma unroll
      for (int a = 0; a < D; ++a)
#pragma unroll
        for (int b = 0; b < D; ++b) {
          acc[2 * (a * D + b)] += xr[a] * xr[b] + xi[a] * xi[b];
          acc[2 * (a * D + b) + 1] += xi[a] * xr[b] - xr[a] * xi[b];
        }
    }
    block_sum_store<W>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * W, W);
  }
}

template <typename R, int K>
static int rdm_t(bt_state* s, const int* bits, int64_t mem_lo, int64_t nmem, double* out, const int8_t* active) {
  bt_ctx* ctx = s->ctx;
  constexpr int W = 2 * (1 << K) * (1 << K);
  int b4[4] = {0, 0, 0, 0}, s4[4] = {0, 0, 0, 0};
  for (int i = 0; i < K; ++i) b4[i] = s4[i] = bits[i];
  for (int i = 0; i < K; ++i)
    for (int j = i + 1; j < K; ++j)
      if (s4[j] < s4[i]) { int t = s4[i]; s4[i] = s4[j]; s4[j] = t; }
  int64_t ng = 1LL << (s->nbits - K);
  int nblk = blocks_per_member(ctx, ng, nmem);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * (size_t)nmem * nblk * W, &part);
  if (rc) return rc;
  dim3 grid(nblk, (unsigned)nmem);
  k_rdm<R, K><<<grid, BT_THREADS, 0, ctx->stream>>>((const typename CT<R>::T*)s->d, s->nbits,
                                                    make_int4(b4[0], b4[1], b4[2], b4[3]),
                                                    make_int4(s4[0], s4[1], s4[2], s4[3]), mem_lo, nblk, part,
                                                    active);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "rdm launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, W, nmem, out);
}

int bt_launch_rdm(bt_state* s, int k, const int* bits, int64_t mem_lo, int64_t nmem, double* out,
                  const int8_t* active) {
  if (nmem > 65535) return bt_fail(s->ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per reduction");
  bool c64 = s->prec == BT_PREC_C64;
  const int8_t* a = active;
  switch (k) {
    case 1: return c64 ? rdm_t<float, 1>(s, bits, mem_lo, nmem, out, a) : rdm_t<double, 1>(s, bits, mem_lo, nmem, out, a);
    case 2: return c64 ? rdm_t<float, 2>(s, bits, mem_lo, nmem, out, a) : rdm_t<double, 2>(s, bits, mem_lo, nmem, out, a);
    case 3: return c64 ? rdm_t<float, 3>(s, bits, mem_lo, nmem, out, a) : rdm_t<double, 3>(s, bits, mem_lo, nmem, out, a);
  }
  return bt_fail(s->ctx, BT_ERR_UNSUPPORTED, "reduced density matrix supports 1 <= k <= 3");
}

// ------------------------------------------------------------ Pauli strings
struct PauliArgs {
  uint64_t x;
  uint64_t z[8];
  int T;
  int hbit;  // highest set bit of x, or -1
  int nbits, nsys;
  int dm;    // 1: density matrix, element rho[a, a^x] at a + ((a^x) << nsys)
};

template <typename T>
__device__ __forceinline__ void phase_of(uint64_t i, uint64_t x, uint64_t z, T& pr, T& pi) {
  // P|i> = i^{popcount(x&z)} (-1)^{popcount(i&z)} |i^x>
  int ny = __popcll(x & z) & 3;
  int sg = __popcll(i & z) & 1;
  pr = (ny == 0) ? (T)1 : (ny == 2 ? (T)-1 : (T)0);
  pi = (ny == 1) ? (T)1 : (ny == 3 ? (T)-1 : (T)0);
  if (sg) { pr = -pr; pi = -pi; }
}

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_pauli(const typename CT<R>::T* __restrict__ psi, PauliArgs a,
                                                      int64_t mem_lo, int nblk, double* __restrict__ part) {
  typedef typename Micro<R>::T A;
  constexpr int J = Micro<R>::J;
  double acc[8];
  A f[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) acc[t] = 0;
  const int64_t mem = mem_lo + blockIdx.y;
  const typename CT<R>::T* s = psi + (mem << a.nbits);
  const int64_t stride = (int64_t)nblk * blockDim.x;
  const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // phases are exactly +-1, +-i: computed in double and converted without rounding
  if (a.dm) {
    const int64_t n = 1LL << a.nsys;
    for (int64_t i0 = start; i0 < n; i0 += stride * J) {
#pragma unroll
      for (int t = 0; t < 8; ++t) f[t] = 0;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t i = i0 + jj * stride;
        if (i >= n) break;
        uint64_t j = (uint64_t)i ^ a.x;
        typename CT<R>::T v = s[(uint64_t)i + (j << a.nsys)];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          if (t < a.T) {
            A pr, pi;
            phase_of<A>((uint64_t)i, a.x, a.z[t], pr, pi);
            f[t] += pr * (A)v.x - pi * (A)v.y;
          }
        }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] += (double)f[t];
    }
  } else if (a.hbit < 0) {
    const int64_t n = 1LL << a.nbits;
    for (int64_t i0 = start; i0 < n; i0 += stride * J) {
#pragma unroll
      for (int t = 0; t < 8; ++t) f[t] = 0;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t i = i0 + jj * stride;
        if (i >= n) break;
        typename CT<R>::T v = s[i];
        const A p = (A)v.x * (A)v.x + (A)v.y * (A)v.y;
#pragma unroll
        for (int t = 0; t < 8; ++t)
          if (t < a.T) f[t] += (__popcll((uint64_t)i & a.z[t]) & 1) ? -p : p;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] += (double)f[t];
    }
  } else {
    const int64_t n = 1LL << (a.nbits - 1);
    const int h = a.hbit;
    for (int64_t g0 = start; g0 < n; g0 += stride * J) {
#pragma unroll
      for (int t = 0; t < 8; ++t) f[t] = 0;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t g = g0 + jj * stride;
        if (g >= n) break;
        uint64_t i = (((uint64_t)g >> h) << (h + 1)) | ((uint64_t)g & ((1ULL << h) - 1));
        uint64_t j = i ^ a.x;
        typename CT<R>::T vi = s[i], vj = s[j];
        // c = conj(psi_j) * psi_i
        const A cr = (A)vj.x * (A)vi.x + (A)vj.y * (A)vi.y;
        const A ci = (A)vj.x * (A)vi.y - (A)vj.y * (A)vi.x;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          if (t < a.T) {
            A p1r, p1i, p2r, p2i;
            phase_of<A>(i, a.x, a.z[t], p1r, p1i);
            phase_of<A>(j, a.x, a.z[t], p2r, p2i);
            // Re(ph_i c) + Re(conj(ph_j) c)
            f[t] += (p1r + p2r) * cr - (p1i - p2i) * ci;
          }
        }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t] += (double)f[t];
    }
  }
  block_sum_store<8>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * 8, 8);
}

int bt_launch_pauli(bt_state* s, uint64_t x, int T, const uint64_t* z, int64_t mem_lo, int64_t nmem, double* out) {
  bt_ctx* ctx = s->ctx;
  if (T < 1 || T > 8) return bt_fail(ctx, BT_ERR_BAD_ARG, "pauli batch must hold 1..8 terms");
  if (nmem > 65535) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per reduction");
  PauliArgs a;
  a.x = x;
  for (int t = 0; t < 8; ++t) a.z[t] = t < T ? z[t] : 0;
  a.T = T;
  a.hbit = x ? 63 - __builtin_clzll(x) : -1;
  a.nbits = s->nbits;
  a.nsys = s->n;
  a.dm = s->repr == BT_REPR_DM;
  int64_t units = a.dm ? (1LL << s->n) : (a.hbit < 0 ? (1LL << s->nbits) : (1LL << (s->nbits - 1)));
  int nblk = blocks_per_member(ctx, units, nmem);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * (size_t)nmem * nblk * 8, &part);
  if (rc) return rc;
  dim3 grid(nblk, (unsigned)nmem);
  if (s->prec == BT_PREC_C64)
    k_pauli<float><<<grid, BT_THREADS, 0, ctx->stream>>>((const float2*)s->d, a, mem_lo, nblk, part);
  else
    k_pauli<double><<<grid, BT_THREADS, 0, ctx->stream>>>((const double2*)s->d, a, mem_lo, nblk, part);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "pauli launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, 8, nmem, out);
}

// ------------------------------------------------------------ Pauli strings, tiled
// Many Pauli strings from one read of the state: a CTA stages a tile of 2^M
// amplitudes (the M tile bits contain the x-mask bits of every string of the
// group and the lowest c bits, so the tile is 2^(M-c) contiguous runs) in shared
// memory, and for each amplitude i of the tile adds
//   Re( phase_t(i) * psi_i * conj(psi_{i ^ x_t}) ),  P_t|i> = phase_t(i)|i ^ x_t>,
// phase_t(i) = i^{|x_t & z_t|} (-1)^{|i & z_t|}, for every string t of the group;
// i ^ x_t lies in the same tile.  Strings sharing an x-mask share the product.
// Sums as in k_pauli: 8-element FP32 micro-sums for complex64, FP64 beyond.
struct PauliTileArgs {
  int nbits, M, c, T, lg_tiles;
  int tbits[16];   // tile bit -> global bit, ascending; tbits[i] = i for i < c
  uint64_t z[BT_PAULI_TILE_TERMS];
  uint32_t xl[BT_PAULI_TILE_TERMS];  // x-mask in tile-local bits
  int ny[BT_PAULI_TILE_TERMS];       // |x & z| mod 4
};

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_pauli_tile(const typename CT<R>::T* __restrict__ psi,
                                                           const PauliTileArgs a, int64_t mem_lo, int nblk,
                                                           double* __restrict__ part) {
  typedef typename CT<R>::T C2;
  typedef typename Micro<R>::T A;
  constexpr int NT = BT_PAULI_TILE_TERMS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* tile = reinterpret_cast<C2*>(smem_raw);
  int64_t* runoff = reinterpret_cast<int64_t*>(smem_raw + (sizeof(C2) << a.M));
  const int M = a.M, c = a.c, cmask = (1 << c) - 1;
  const int nruns = 1 << (M - c);
  for (int r = threadIdx.x; r < nruns; r += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < M - c; ++b)
      if ((r >> b) & 1) o |= 1LL << a.tbits[c + b];
    runoff[r] = o;
  }
  double acc[NT];
  A f[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) acc[t] = 0, f[t] = 0;
  const int64_t mem = mem_lo + blockIdx.y;
  const C2* s = psi + (mem << a.nbits);
  const int64_t ntiles = 1LL << a.lg_tiles;
  const int E = (1 << M) / blockDim.x;  // elements per thread per tile (M >= 8)
  int cnt = 0;
  for (int64_t tid = blockIdx.x; tid < ntiles; tid += nblk) {
    uint64_t base = (uint64_t)tid;
    for (int i = 0; i < M; ++i) {
      const int p = a.tbits[i];
      base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
    }
    __syncthreads();  // the previous tile is no longer read
    for (int k = 0; k < E; ++k) {
      const int l = threadIdx.x + k * blockDim.x;
      tile[l] = s[base + runoff[l >> c] + (l & cmask)];
    }
    __syncthreads();
    for (int k = 0; k < E; ++k) {
      const int l = threadIdx.x + k * blockDim.x;
      const uint64_t gi = base + runoff[l >> c] + (l & cmask);
      const C2 v = tile[l];
      const A vr = (A)v.x, vi = (A)v.y;
      uint32_t lastx = 0xffffffffu;
      A cr = 0, ci = 0;
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        if (t < a.T) {
          if (a.xl[t] != lastx) {  // psi_i * conj(psi_{i^x})
            lastx = a.xl[t];
            const C2 w = tile[l ^ lastx];
            cr = vr * (A)w.x + vi * (A)w.y;
            ci = vi * (A)w.x - vr * (A)w.y;
          }
          const int ny = a.ny[t];
          A val = (ny & 1) ? ci : cr;  // Re(i^ny c): cr, -ci, -cr, ci
          if (ny == 1 || ny == 2) val = -val;
          f[t] += (__popcll(gi & a.z[t]) & 1) ? -val : val;
        }
      }
      if (++cnt == Micro<R>::J) {
#pragma unroll
        for (int t = 0; t < NT; ++t) acc[t] += (double)f[t], f[t] = 0;
        cnt = 0;
      }
    }
  }
#pragma unroll
  for (int t = 0; t < NT; ++t) acc[t] += (double)f[t];
  __syncthreads();
  block_sum_store<NT>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * NT, NT);
}

int bt_launch_pauli_tile(bt_state* s, int M, uint64_t tilemask, int T, const uint64_t* x, const uint64_t* z,
                         int64_t mem_lo, int64_t nmem, double* out) {
  bt_ctx* ctx = s->ctx;
  if (T < 1 || T > BT_PAULI_TILE_TERMS) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad tiled Pauli group");
  if (nmem > 65535) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per reduction");
  PauliTileArgs a;
  memset(&a, 0, sizeof(a));
  a.nbits = s->nbits;
  a.M = M;
  a.c = s->prec == BT_PREC_C64 ? 5 : 4;
  a.T = T;
  a.lg_tiles = s->nbits - M;
  int local[64], nb = 0;
  for (int b = 0; b < s->nbits; ++b) {
    local[b] = -1;
    if ((tilemask >> b) & 1) {
      a.tbits[nb] = b;
      local[b] = nb++;
    }
  }
  if (nb != M || M < 8 || M > 13 || (tilemask & ((1ULL << a.c) - 1)) != ((1ULL << a.c) - 1))
    return bt_fail(ctx, BT_ERR_BAD_ARG, "bad tile for Pauli strings");
  for (int t = 0; t < T; ++t) {
    uint32_t xl = 0;
    for (int b = 0; b < s->nbits; ++b)
      if ((x[t] >> b) & 1) {
        if (local[b] < 0) return bt_fail(ctx, BT_ERR_BAD_ARG, "Pauli x-mask outside the tile");
        xl |= 1u << local[b];
      }
    a.xl[t] = xl;
    a.z[t] = z[t];
    a.ny[t] = __builtin_popcountll(x[t] & z[t]) & 3;
  }
  const int64_t ntiles = 1LL << a.lg_tiles;
  const int nblk = (int)std::min<int64_t>(ntiles, std::max<int64_t>(1, (ctx->sm_count * 2 + nmem - 1) / nmem));
  double* part;
  int rc = bt_work(ctx, sizeof(double) * (size_t)nmem * nblk * BT_PAULI_TILE_TERMS, &part);
  if (rc) return rc;
  const size_t esz = elem_bytes(s->prec);
  const size_t smem = (esz << M) + sizeof(int64_t) * (1 << (M - a.c));
  dim3 grid(nblk, (unsigned)nmem);
  // the largest tile of either precision (2^13 x 8 B or 2^12 x 16 B, plus 256 run
  // offsets), set once per device: a per-launch setting would race between
  // contexts launching concurrently from different threads
  const int kMaxSmem = (1 << 16) + 8 * 256;
  static std::atomic<bool> attr[2][64] = {};
  const bool f = s->prec == BT_PREC_C64;
  std::atomic<bool>& done = attr[f][ctx->device & 63];
  if (!done.load()) {
    cudaError_t e = f ? cudaFuncSetAttribute(k_pauli_tile<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem)
                      : cudaFuncSetAttribute(k_pauli_tile<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    if ((rc = bt_cuda_check(ctx, e, "pauli tile attribute"))) return rc;
    done.store(true);
  }
  if (f)
    k_pauli_tile<float><<<grid, BT_THREADS, smem, ctx->stream>>>((const float2*)s->d, a, mem_lo, nblk, part);
  else
    k_pauli_tile<double><<<grid, BT_THREADS, smem, ctx->stream>>>((const double2*)s->d, a, mem_lo, nblk, part);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "pauli tile launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, BT_PAULI_TILE_TERMS, nmem, out);
}

// float-float accumulation: x added to (hi, lo) by TwoSum, the rounding error of
// each add kept in lo
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x, bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

// ------------------------------------------------------------ per-bit sums
// out[mem][0] = total weight, out[mem][1+b] = weight with bit b set (b < nsys).
// A warp walks chunks of 1024 consecutive amplitudes, lane l taking entries
// l + 32 j: bits 0-4 are the lane's, bits 5-9 the unrolled j's, and bits >= 10
// are constant over the chunk, so each weight costs a handful of FP64 adds.
#define BS_W 36
// complex64 state vectors of at least 2^BS_SC amplitudes: a warp takes
// super-chunks of 32 consecutive chunks.  The FP32 sums of 8 weights are
// accumulated per lane in float-float (TwoSum) and reach FP64 once per
// super-chunk: about 0.04 FP64 adds per amplitude instead of 1.7 (the chunk form
// is FP64-issue bound on this part, 3.3x its HBM time at 33 qubits).  Bits 5-9
// are the unrolled j's, bits 10-14 the chunk index k (the same in every lane of
// the warp), bits >= 15 constant over the super-chunk.
#define BS_SC 15
__device__ __forceinline__ void bitsums_superchunks(const float2* __restrict__ s, int nsys, int lane, int64_t wid,
                                                    int64_t warps_total, double (&acc)[BS_W]) {
  const int64_t nsc = (1LL << nsys) >> BS_SC;
  double lanetot = 0;
  for (int64_t sc = wid; sc < nsc; sc += warps_total) {
    float th = 0, tl = 0;                                     // the lane's total
    float jh[5] = {0, 0, 0, 0, 0}, jl[5] = {0, 0, 0, 0, 0};  // bits 5-9
    float kh[5] = {0, 0, 0, 0, 0}, kl[5] = {0, 0, 0, 0, 0};  // bits 10-14
    const float2* base = s + ((uint64_t)sc << BS_SC) + lane;
    for (int k = 0; k < 32; ++k) {
      const float2* cp = base + ((uint64_t)k << 10);
      float ch = 0, cl = 0;  // the chunk's total
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        float gs = 0, gb[3] = {0, 0, 0};
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const float2 v = cp[(g * 8 + jj) << 5];
          const float p = fmaf(v.x, v.x, v.y * v.y);
          gs += p;
#pragma unroll
          for (int b = 0; b < 3; ++b)
            if ((jj >> b) & 1) gb[b] += p;
        }
        two_sum_acc(ch, cl, gs);
#pragma unroll
        for (int b = 0; b < 3; ++b) two_sum_acc(jh[b], jl[b], gb[b]);
        if (g & 1) two_sum_acc(jh[3], jl[3], gs);
        if (g & 2) two_sum_acc(jh[4], jl[4], gs);
      }
      two_sum_acc(th, tl, ch);
      tl += cl;
#pragma unroll
      for (int b = 0; b < 5; ++b)
        if ((k >> b) & 1) {
          two_sum_acc(kh[b], kl[b], ch);
          kl[b] += cl;
        }
    }
    const double tot = (double)th + (double)tl;
    lanetot += tot;
#pragma unroll
    for (int b = 0; b < 5; ++b) {
      acc[1 + 5 + b] += (double)jh[b] + (double)jl[b];
      acc[1 + 10 + b] += (double)kh[b] + (double)kl[b];
    }
    const uint64_t hi = (uint64_t)sc << BS_SC;
#pragma unroll
    for (int b = BS_SC; b < BS_W - 1; ++b) acc[1 + b] += ((hi >> b) & 1) ? tot : 0.0;
  }
  acc[0] += lanetot;
#pragma unroll
  for (int b = 0; b < 5; ++b)
    if ((lane >> b) & 1) acc[1 + b] += lanetot;
}

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_bitsums(const typename CT<R>::T* __restrict__ psi, int nbits,
                                                        int nsys, int dm, int64_t mem_lo, int nblk,
                                                        double* __restrict__ part) {
  double acc[BS_W];
#pragma unroll
  for (int w = 0; w < BS_W; ++w) acc[w] = 0;
  const int64_t mem = mem_lo + blockIdx.y;
  const typename CT<R>::T* s = psi + (mem << nbits);
  const int lane = threadIdx.x & 31;
  const int64_t nent = 1LL << nsys;
  const int64_t warps_total = (int64_t)nblk * (blockDim.x >> 5);
  const int64_t wid = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if constexpr (sizeof(R) == 4) {
    if (!dm && nsys >= BS_SC) {  // the same branch in every thread of the launch
      bitsums_superchunks(s, nsys, lane, wid, warps_total, acc);
      block_sum_store<BS_W>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * BS_W, BS_W);
      return;
    }
  }
  if (nsys >= 10) {
    const int64_t nchunk = nent >> 10;
    double lanetot = 0;
    typedef typename Micro<R>::T A;
    for (int64_t c = wid; c < nchunk; c += warps_total) {
      double csum = 0;
      double jb[5] = {0, 0, 0, 0, 0};
      // four groups of 8 j's: per group an FP32 (complex64) or FP64 micro-sum and
      // the sums for j-bits 0-2; j-bits 3-4 are constant within a group
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        A gs = 0, gb[3] = {0, 0, 0};
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const int j = g * 8 + jj;
          uint64_t i = ((uint64_t)c << 10) + ((uint64_t)j << 5) + lane;
          typename CT<R>::T v = dm ? s[i + (i << nsys)] : s[i];
          const A p = dm ? (A)v.x : (A)v.x * (A)v.x + (A)v.y * (A)v.y;
          gs += p;
#pragma unroll
          for (int b = 0; b < 3; ++b)
            if ((jj >> b) & 1) gb[b] += p;
        }
        csum += (double)gs;
#pragma unroll
        for (int b = 0; b < 3; ++b) jb[b] += (double)gb[b];
        if (g & 1) jb[3] += (double)gs;
        if (g & 2) jb[4] += (double)gs;
      }
      lanetot += csum;
#pragma unroll
      for (int b = 0; b < 5; ++b) acc[1 + 5 + b] += jb[b];
      // compile-time accumulator indices (a run-time index would spill acc[] to
      // local memory); bits at or above nsys are never set in the chunk index
      const uint64_t hi = (uint64_t)c << 10;
#pragma unroll
      for (int b = 10; b < BS_W - 1; ++b) acc[1 + b] += ((hi >> b) & 1) ? csum : 0.0;
    }
    acc[0] += lanetot;
#pragma unroll
    for (int b = 0; b < 5; ++b)
      if ((lane >> b) & 1) acc[1 + b] += lanetot;
  } else {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nent; i += (int64_t)nblk * blockDim.x) {
      typename CT<R>::T v = dm ? s[(uint64_t)i + ((uint64_t)i << nsys)] : s[i];
      double p = dm ? (double)v.x : (double)v.x * v.x + (double)v.y * v.y;
      acc[0] += p;
#pragma unroll
      for (int b = 0; b < 10; ++b) acc[1 + b] += ((i >> b) & 1) ? p : 0.0;
    }
  }
  block_sum_store<BS_W>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x) * BS_W, BS_W);
}

// ------------------------------------------------------------ norms
// sum |psi|^2 (state) or Re tr(rho) (density matrix) per member.  complex64:
// every square is split exactly (TwoProduct: p = a*a, e = fma(a, a, -p)) and the
// terms of a thread's 8-term groups are added with TwoSum into a float-float
// (hi, lo) pair, so a group carries ~44 significant bits at FP32 issue rate;
// groups, threads and blocks then sum in FP64.  complex128: FP64 throughout.
template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_norm2(const typename CT<R>::T* __restrict__ psi, int nbits, int nsys,
                                                      int dm, int64_t mem_lo, int nblk, double* __restrict__ part) {
  double acc[1] = {0};
  const int64_t mem = mem_lo + blockIdx.y;
  const typename CT<R>::T* s = psi + (mem << nbits);
  const int64_t n = dm ? (1LL << nsys) : (1LL << nbits);
  const int64_t stride = (int64_t)nblk * blockDim.x;
  constexpr int J = 8;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += stride * J) {
    if constexpr (sizeof(R) == 4) {
      float hi = 0, lo = 0;
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t i = i0 + jj * stride;
        if (i >= n) break;
        const typename CT<R>::T v = dm ? s[(uint64_t)i + ((uint64_t)i << nsys)] : s[i];
        if (dm) {
          two_sum_acc(hi, lo, v.x);
        } else {
          const float p1 = v.x * v.x, e1 = fmaf(v.x, v.x, -p1);
          const float p2 = v.y * v.y, e2 = fmaf(v.y, v.y, -p2);
          two_sum_acc(hi, lo, p1);
          two_sum_acc(hi, lo, p2);
          lo += e1 + e2;
        }
      }
      acc[0] += (double)hi + (double)lo;
    } else {
#pragma unroll
      for (int jj = 0; jj < J; ++jj) {
        const int64_t i = i0 + jj * stride;
        if (i >= n) break;
        const typename CT<R>::T v = dm ? s[(uint64_t)i + ((uint64_t)i << nsys)] : s[i];
        acc[0] += dm ? (double)v.x : (double)v.x * v.x + (double)v.y * v.y;
      }
    }
  }
  block_sum_store<1>(acc, part + ((int64_t)blockIdx.y * nblk + blockIdx.x), 1);
}

int bt_launch_norm2(bt_state* s, int64_t mem_lo, int64_t nmem, double* out) {
  bt_ctx* ctx = s->ctx;
  if (nmem > 65535) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per reduction");
  const int dm = s->repr == BT_REPR_DM;
  const int64_t units = dm ? (1LL << s->n) : (1LL << s->nbits);
  const int nblk = blocks_per_member(ctx, units, nmem);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * (size_t)nmem * nblk, &part);
  if (rc) return rc;
  dim3 grid(nblk, (unsigned)nmem);
  if (s->prec == BT_PREC_C64)
    k_norm2<float><<<grid, BT_THREADS, 0, ctx->stream>>>((const float2*)s->d, s->nbits, s->n, dm, mem_lo, nblk, part);
  else
    k_norm2<double><<<grid, BT_THREADS, 0, ctx->stream>>>((const double2*)s->d, s->nbits, s->n, dm, mem_lo, nblk, part);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "norm2 launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, 1, nmem, out);
}

// blocks per member of the super-chunk form: every SM filled to the kernel's
// occupancy (the grid loops, so no partial last wave) and at least one
// super-chunk per warp
static int superchunk_blocks(const bt_ctx* ctx, int64_t nsc, int64_t nmem) {
  static std::atomic<int> occ{0};
  int o = occ.load();
  if (!o) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_bitsums<float>, BT_THREADS, 0) != cudaSuccess || o < 1) {
      (void)cudaGetLastError();  // leave no error behind for the launch check
      o = 1;
    }
    occ.store(o);
  }
  int64_t per = ((int64_t)ctx->sm_count * o + nmem - 1) / nmem;
  const int64_t maxb = (nsc + BT_THREADS / 32 - 1) / (BT_THREADS / 32);
  if (per > maxb) per = maxb;
  if (per < 1) per = 1;
  return (int)per;
}

int bt_launch_bitsums(bt_state* s, int64_t mem_lo, int64_t nmem, double* out) {
  bt_ctx* ctx = s->ctx;
  if (s->n > BS_W - 1) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "too many qubits for per-bit sums");
  if (nmem > 65535) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per reduction");
  const bool superchunks = s->prec == BT_PREC_C64 && s->repr != BT_REPR_DM && s->n >= BS_SC;
  int64_t units = s->n >= 10 ? (1LL << s->n) / 32 : (1LL << s->n);
  int nblk = superchunks ? superchunk_blocks(ctx, (1LL << s->n) >> BS_SC, nmem) : blocks_per_member(ctx, units, nmem);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * (size_t)nmem * nblk * BS_W, &part);
  if (rc) return rc;
  dim3 grid(nblk, (unsigned)nmem);
  int dm = s->repr == BT_REPR_DM;
  if (s->prec == BT_PREC_C64)
    k_bitsums<float><<<grid, BT_THREADS, 0, ctx->stream>>>((const float2*)s->d, s->nbits, s->n, dm, mem_lo, nblk, part);
  else
    k_bitsums<double><<<grid, BT_THREADS, 0, ctx->stream>>>((const double2*)s->d, s->nbits, s->n, dm, mem_lo, nblk, part);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "bitsums launch");
  if (rc) return rc;
  // out receives BS_W values per member
  return finalize(ctx, part, nblk, BS_W, nmem, out);
}

// ------------------------------------------------------------ inner product
template <typename Ra, typename Rb>
__global__ void __launch_bounds__(BT_THREADS) k_inner(const typename CT<Ra>::T* __restrict__ a,
                                                      const typename CT<Rb>::T* __restrict__ b, int64_t n,
                                                      int nblk, double* __restrict__ part) {
  // FP32 micro-sums only when both states are complex64
  typedef typename Micro<decltype(Ra() + Rb())>::T A;
  constexpr int J = Micro<decltype(Ra() + Rb())>::J;
  double acc[2] = {0, 0};
  const int64_t stride = (int64_t)nblk * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += stride * J) {
    A f0 = 0, f1 = 0;
#pragma unroll
    for (int jj = 0; jj < J; ++jj) {
      const int64_t i = i0 + jj * stride;
      if (i >= n) break;
      typename CT<Ra>::T x = a[i];
      typename CT<Rb>::T y = b[i];
      f0 += (A)x.x * (A)y.x + (A)x.y * (A)y.y;
      f1 += (A)x.x * (A)y.y - (A)x.y * (A)y.x;
    }
    acc[0] += (double)f0;
    acc[1] += (double)f1;
  }
  block_sum_store<2>(acc, part + (int64_t)blockIdx.x * 2, 2);
}

int bt_launch_inner(bt_state* a, int64_t am, bt_state* b, int64_t bm, double* out) {
  bt_ctx* ctx = a->ctx;
  int64_t n = a->member_elems;
  int nblk = blocks_per_member(ctx, n, 1);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * nblk * 2, &part);
  if (rc) return rc;
  const char* pa = (const char*)a->d + am * n * elem_bytes(a->prec);
  const char* pb = (const char*)b->d + bm * n * elem_bytes(b->prec);
  bool fa = a->prec == BT_PREC_C64, fb = b->prec == BT_PREC_C64;
  if (fa && fb) k_inner<float, float><<<nblk, BT_THREADS, 0, ctx->stream>>>((const float2*)pa, (const float2*)pb, n, nblk, part);
  else if (fa) k_inner<float, double><<<nblk, BT_THREADS, 0, ctx->stream>>>((const float2*)pa, (const double2*)pb, n, nblk, part);
  else if (fb) k_inner<double, float><<<nblk, BT_THREADS, 0, ctx->stream>>>((const double2*)pa, (const float2*)pb, n, nblk, part);
  else k_inner<double, double><<<nblk, BT_THREADS, 0, ctx->stream>>>((const double2*)pa, (const double2*)pb, n, nblk, part);
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "inner launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, 2, 1, out);
}

// ------------------------------------------------------------ <psi|M|psi>
template <typename R, int K>
__global__ void __launch_bounds__(BT_THREADS) k_expect_matrix(const typename CT<R>::T* __restrict__ s, int nbits,
                                                              int4 bits4, int4 sorted4, uint64_t cmask,
                                                              const double* __restrict__ m, int nblk,
                                                              double* __restrict__ part) {
  constexpr int D = 1 << K;
  const int bits[4] = {bits4.x, bits4.y, bits4.z, bits4.w};
  const int sorted[4] = {sorted4.x, sorted4.y, sorted4.z, sorted4.w};
  int64_t off[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    int64_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> (K - 1 - b)) & 1) o |= 1LL << bits[b];
    off[j] = o;
  }
  double acc[1] = {0};
  const int64_t ng = 1LL << (nbits - K);
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (int64_t)nblk * blockDim.x) {
    uint64_t base = (uint64_t)g;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int p = sorted[i];
      base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
    }
    double xr[D], xi[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      typename CT<R>::T v = s[base + off[j]];
      xr[j] = v.x;
      xi[j] = v.y;
    }
    if ((base & cmask) != cmask) {
      // identity on this group: sum |x|^2
#pragma unroll
      for (int j = 0; j < D; ++j) acc[0] += xr[j] * xr[j] + xi[j] * xi[j];
      continue;
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      double yr = 0, yi = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) {
        double mr = m[2 * (r * D + c)], mi = m[2 * (r * D + c) + 1];
        yr += mr * xr[c] - mi * xi[c];
        yi += mr * xi[c] + mi * xr[c];
      }
      acc[0] += xr[r] * yr + xi[r] * yi;
    }
  }
  block_sum_store<1>(acc, part + (int64_t)blockIdx.x, 1);
}

int bt_launch_expect_matrix(bt_state* s, int k, const int* bits, const double* m_rowmajor_dev, uint64_t cmask,
                            int64_t mem, double* out) {
  bt_ctx* ctx = s->ctx;
  int b4[4] = {0, 0, 0, 0}, s4[4] = {0, 0, 0, 0};
  for (int i = 0; i < k; ++i) b4[i] = s4[i] = bits[i];
  for (int i = 0; i < k; ++i)
    for (int j = i + 1; j < k; ++j)
      if (s4[j] < s4[i]) { int t = s4[i]; s4[i] = s4[j]; s4[j] = t; }
  int64_t ng = 1LL << (s->nbits - k);
  int nblk = blocks_per_member(ctx, ng, 1);
  double* part;
  int rc = bt_work(ctx, sizeof(double) * nblk, &part);
  if (rc) return rc;
  const char* p = (const char*)s->d + mem * s->member_elems * elem_bytes(s->prec);
  int4 bb = make_int4(b4[0], b4[1], b4[2], b4[3]), ss = make_int4(s4[0], s4[1], s4[2], s4[3]);
  bool f = s->prec == BT_PREC_C64;
  if (k == 1) {
    if (f) k_expect_matrix<float, 1><<<nblk, BT_THREADS, 0, ctx->stream>>>((const float2*)p, s->nbits, bb, ss, cmask, m_rowmajor_dev, nblk, part);
    else k_expect_matrix<double, 1><<<nblk, BT_THREADS, 0, ctx->stream>>>((const double2*)p, s->nbits, bb, ss, cmask, m_rowmajor_dev, nblk, part);
  } else if (k == 2) {
    if (f) k_expect_matrix<float, 2><<<nblk, BT_THREADS, 0, ctx->stream>>>((const float2*)p, s->nbits, bb, ss, cmask, m_rowmajor_dev, nblk, part);
    else k_expect_matrix<double, 2><<<nblk, BT_THREADS, 0, ctx->stream>>>((const double2*)p, s->nbits, bb, ss, cmask, m_rowmajor_dev, nblk, part);
  } else {
    return bt_fail(ctx, BT_ERR_UNSUPPORTED, "expect_matrix supports k <= 2");
  }
  ctx->launches++;
  rc = bt_cuda_check(ctx, cudaGetLastError(), "expect_matrix launch");
  if (rc) return rc;
  return finalize(ctx, part, nblk, 1, 1, out);
}

// ------------------------------------------------------------ collapse / dephase
template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_collapse(typename CT<R>::T* __restrict__ psi, int nbits, int bit,
                                                         const int* __restrict__ outcome,
                                                         const double* __restrict__ scale, int64_t mem_lo,
                                                         int64_t nmem) {
  const int64_t per = 1LL << nbits;
  const int64_t total = per * nmem;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t mi = t >> nbits;
    const int64_t mem = mem_lo + mi;
    const int64_t i = t & (per - 1);
    typename CT<R>::T* p = psi + (mem << nbits) + i;
    const int oc = outcome[mi];
    if (oc < 0) continue;  // member whose decision failed: left untouched
    if ((int)((i >> bit) & 1) == oc) {
      const R sc = (R)scale[mi];
      typename CT<R>::T v = *p;
      v.x *= sc;
      v.y *= sc;
      *p = v;
    } else {
      typename CT<R>::T z;
      z.x = 0;
      z.y = 0;
      *p = z;
    }
  }
}

int bt_launch_collapse(bt_state* s, int bit, const int* d_outcome, const double* d_scale, int64_t mem_lo, int64_t nmem) {
  bt_ctx* ctx = s->ctx;
  int64_t work = (1LL << s->nbits) * nmem;
  int grid = bt_grid(ctx, work, BT_THREADS, 32);
  if (s->prec == BT_PREC_C64)
    k_collapse<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d, s->nbits, bit, d_outcome, d_scale, mem_lo, nmem);
  else
    k_collapse<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d, s->nbits, bit, d_outcome, d_scale, mem_lo, nmem);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "collapse launch");
}

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_dephase(typename CT<R>::T* __restrict__ rho, int nbits, int nsys, int b,
                                                        int64_t mem_lo, int64_t nmem) {
  const int64_t per = 1LL << nbits;
  const int64_t total = per * nmem;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t mem = mem_lo + (t >> nbits);
    const int64_t e = t & (per - 1);
    if (((e >> b) & 1) != ((e >> (b + nsys)) & 1)) {
      typename CT<R>::T z;
      z.x = 0;
      z.y = 0;
      rho[(mem << nbits) + e] = z;
    }
  }
}

int bt_launch_dephase(bt_state* s, int b, int64_t mem_lo, int64_t nmem) {
  bt_ctx* ctx = s->ctx;
  int64_t work = (1LL << s->nbits) * nmem;
  int grid = bt_grid(ctx, work, BT_THREADS, 32);
  if (s->prec == BT_PREC_C64)
    k_dephase<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d, s->nbits, s->n, b, mem_lo, nmem);
  else
    k_dephase<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d, s->nbits, s->n, b, mem_lo, nmem);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "dephase launch");
}

// ------------------------------------------------------------ decisions
// measurement: rdm[mem] is the 2x2 reduced matrix (row-major interleaved, 8 doubles)
__global__ void k_decide_measure(int64_t nmem, const double* __restrict__ rdm, const double* __restrict__ u,
                                 const int* __restrict__ forced, uint64_t key, uint64_t stream,
                                 int* __restrict__ outcome, double* __restrict__ scale, double* __restrict__ p0,
                                 int* __restrict__ status) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  const double s0 = rdm[m * 8 + 0], s1 = rdm[m * 8 + 6];
  int f = forced ? forced[m] : -1;
  if (f == -2) {  // this member is not measured
    outcome[m] = -1;
    scale[m] = 1.0;
    p0[m] = s0;
    return;
  }
  double uu = u ? u[m] : bt_uniform(key, stream, (uint64_t)m);
  int ind = f >= 0 ? f : (uu < s0 ? 0 : 1);
  double keep = ind ? s1 : s0;
  p0[m] = s0;
  if (!(keep > 0) || ind > 1) {
    // an outcome of zero probability: report it and leave this member untouched
    atomicExch(status, 1);
    outcome[m] = -1;
    scale[m] = 1.0;
    return;
  }
  outcome[m] = ind;
  scale[m] = 1.0 / sqrt(keep);
}

int bt_launch_decide_measure(bt_ctx* ctx, int64_t nmem, const double* rdm, const double* u, const int* forced,
                             uint64_t rng_stream, int* outcome, double* scale, double* p0) {
  unsigned grid = (unsigned)((nmem + 127) / 128);
  k_decide_measure<<<grid, 128, 0, ctx->stream>>>(nmem, rdm, u, forced, ctx->seed, rng_stream, outcome, scale, p0,
                                                  ctx->d_status);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "decide_measure launch");
}

// two-qubit measurement (born_measure_Z(N, psi, q1, q2), src/hilbert.jl:705-721):
// rdm[mem] is the 4x4 reduced matrix on (q1, q2), q1 the most significant bit
// (32 doubles, row-major interleaved).  The reference lists the outcomes as
// [P0 P0, P1 P0, P0 P1, P1 P1] on (q1, q2), i.e. outcome k (1-based) keeps
// q1 = (k - 1) & 1 and q2 = (k - 1) >> 1, with weights |psi' P_k psi| drawn by
// _weighted_sample (first k with u <= cumsum(p)[k], no renormalisation).
__device__ __forceinline__ int meas2_index(int k) {  // reference outcome (0-based) -> reduced index
  return ((k & 1) << 1) | (k >> 1);
}

__global__ void k_decide_measure2(int64_t nmem, const double* __restrict__ rdm, const double* __restrict__ u,
                                  const int* __restrict__ forced, uint64_t key, uint64_t stream,
                                  int* __restrict__ outcome, double* __restrict__ scale, double* __restrict__ probs,
                                  int* __restrict__ status) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  double p[4];
  for (int k = 0; k < 4; ++k) {
    const int a = meas2_index(k);
    p[k] = fabs(rdm[m * 32 + 2 * (a * 4 + a)]);
    probs[m * 4 + k] = p[k];
  }
  const int f = forced ? forced[m] : -1;
  if (f == -2) {  // this member is not measured
    outcome[m] = -1;
    scale[m] = 1.0;
    return;
  }
  int ind = -1;
  if (f >= 1 && f <= 4) {
    ind = f - 1;
  } else {
    const double uu = u ? u[m] : bt_uniform(key, stream, (uint64_t)m);
    double cum = 0;
    for (int k = 0; k < 4 && ind < 0; ++k) {
      cum += p[k];
      if (uu <= cum) ind = k;
    }
    if (ind < 0) {  // u beyond the cumulative weight: no outcome, as in the reference
      atomicExch(status, 2);
      outcome[m] = -1;
      scale[m] = 1.0;
      return;
    }
  }
  if (!(p[ind] > 0)) {
    atomicExch(status, 1);
    outcome[m] = -1;
    scale[m] = 1.0;
    return;
  }
  outcome[m] = ind + 1;
  scale[m] = 1.0 / sqrt(p[ind]);
}

int bt_launch_decide_measure2(bt_ctx* ctx, int64_t nmem, const double* rdm, const double* u, const int* forced,
                              uint64_t rng_stream, int* outcome, double* scale, double* probs) {
  unsigned grid = (unsigned)((nmem + 127) / 128);
  k_decide_measure2<<<grid, 128, 0, ctx->stream>>>(nmem, rdm, u, forced, ctx->seed, rng_stream, outcome, scale, probs,
                                                   ctx->d_status);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "decide_measure2 launch");
}

// member m keeps the amplitudes whose bits (b1, b2) match its outcome (1..4 in the
// reference's order) scaled by scale[m]; the rest become zero
template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_collapse2(typename CT<R>::T* __restrict__ psi, int nbits, int b1, int b2,
                                                          const int* __restrict__ outcome,
                                                          const double* __restrict__ scale, int64_t mem_lo,
                                                          int64_t nmem) {
  const int64_t per = 1LL << nbits;
  const int64_t total = per * nmem;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t mi = t >> nbits;
    const int oc = outcome[mi];
    if (oc < 1) continue;  // member not measured, or whose decision failed: left untouched
    const int64_t i = t & (per - 1);
    typename CT<R>::T* p = psi + ((mem_lo + mi) << nbits) + i;
    const int keep1 = (oc - 1) & 1, keep2 = (oc - 1) >> 1;
    if ((int)((i >> b1) & 1) == keep1 && (int)((i >> b2) & 1) == keep2) {
      const R sc = (R)scale[mi];
      typename CT<R>::T v = *p;
      v.x *= sc;
      v.y *= sc;
      *p = v;
    } else {
      typename CT<R>::T z;
      z.x = 0;
      z.y = 0;
      *p = z;
    }
  }
}

int bt_launch_collapse2(bt_state* s, int b1, int b2, const int* d_outcome, const double* d_scale, int64_t mem_lo,
                        int64_t nmem) {
  bt_ctx* ctx = s->ctx;
  int64_t work = (1LL << s->nbits) * nmem;
  int grid = bt_grid(ctx, work, BT_THREADS, 32);
  if (s->prec == BT_PREC_C64)
    k_collapse2<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d, s->nbits, b1, b2, d_outcome, d_scale,
                                                             mem_lo, nmem);
  else
    k_collapse2<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d, s->nbits, b1, b2, d_outcome, d_scale,
                                                              mem_lo, nmem);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "collapse2 launch");
}

// Kraus branch: rdm[mem] is the D x D reduced matrix in application order (q, t);
// kraus holds nk row-major interleaved D x D matrices (FP64).
template <typename R>
__global__ void k_decide_kraus(int64_t nmem, int k, int nk, int ref_perm, const double* __restrict__ rdm,
                               const double* __restrict__ kraus, const double* __restrict__ u,
                               const int* __restrict__ forced, uint64_t key, uint64_t stream,
                               int* __restrict__ branch, double* __restrict__ probs, R* __restrict__ pm,
                               int* __restrict__ status) {
  int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nmem) return;
  const int D = 1 << k;
  R* out = pm + m * 2 * D * D;
  int f = forced ? forced[m] : -1;
  if (f == -2) {  // this member skips the channel: identity, no draw consumed
    branch[m] = -1;
    for (int e = 0; e < 2 * D * D; ++e) out[e] = (R)((e % (2 * D + 2)) == 0 ? 1.0 : 0.0);
    return;
  }
  // rdm == nullptr: the Kraus operators are multiples of unitaries, so the branch
  // probabilities |c_i|^2 do not depend on the (normalised) state: rho_A = I/D
  const double* r = rdm ? rdm + m * 2 * D * D : nullptr;
  const double diag = 1.0 / D;
  // reference-order reduced matrix: for a pair with q > t the reference reads
  // rho_A in (t, q) order, i.e. indices permuted by [0, 2, 1, 3]
  const int perm[4] = {0, 2, 1, 3};
  double cum = 0;
  double uu = u ? u[m] : bt_uniform(key, stream, (uint64_t)m);
  int ind = -1;
  for (int i = 0; i < nk; ++i) {
    const double* K = kraus + (int64_t)i * 2 * D * D;
    // p = Re tr(K rho K^dagger) = Re sum_{a,b,c} K[c,a] rho[a,b] conj(K[c,b])
    double p = 0;
    for (int c = 0; c < D; ++c)
      for (int a = 0; a < D; ++a) {
        double kar = K[2 * (c * D + a)], kai = K[2 * (c * D + a) + 1];
        for (int b = 0; b < D; ++b) {
          int ra = ref_perm ? perm[a] : a, rb = ref_perm ? perm[b] : b;
          double rr = r ? r[2 * (ra * D + rb)] : (ra == rb ? diag : 0.0);
          double ri = r ? r[2 * (ra * D + rb) + 1] : 0.0;
          double kbr = K[2 * (c * D + b)], kbi = -K[2 * (c * D + b) + 1];
          // (ka * rho) * conj(kb)
          double tr_ = kar * rr - kai * ri, ti = kar * ri + kai * rr;
          p += tr_ * kbr - ti * kbi;
        }
      }
    if (probs) probs[m * nk + i] = p;
    cum += p;
    if (ind < 0 && uu <= cum) ind = i;
  }
  if (f >= 0) ind = f;
  if (ind < 0 || ind >= nk) {
    // no branch (the reference's _weighted_sample returns nothing): report it and
    // leave this member untouched with an identity matrix
    atomicExch(status, 2);
    branch[m] = -1;
    for (int e = 0; e < 2 * D * D; ++e) out[e] = (R)((e % (2 * D + 2)) == 0 ? 1.0 : 0.0);
    return;
  }
  branch[m] = ind;
  // norm of K_ind psi in application order
  const double* K = kraus + (int64_t)ind * 2 * D * D;
  double nrm = 0;
  for (int c = 0; c < D; ++c)
    for (int a = 0; a < D; ++a) {
      double kar = K[2 * (c * D + a)], kai = K[2 * (c * D + a) + 1];
      for (int b = 0; b < D; ++b) {
        double rr = r ? r[2 * (a * D + b)] : (a == b ? diag : 0.0);
        double ri = r ? r[2 * (a * D + b) + 1] : 0.0;
        double kbr = K[2 * (c * D + b)], kbi = -K[2 * (c * D + b) + 1];
        double tr_ = kar * rr - kai * ri, ti = kar * ri + kai * rr;
        nrm += tr_ * kbr - ti * kbi;
      }
    }
  if (!(nrm > 0)) {
    atomicExch(status, 3);
    for (int e = 0; e < 2 * D * D; ++e) out[e] = (R)((e % (2 * D + 2)) == 0 ? 1.0 : 0.0);
    return;
  }
  const double sc = 1.0 / sqrt(nrm);
  for (int e = 0; e < 2 * D * D; ++e) out[e] = (R)(K[e] * sc);
}

int bt_launch_decide_kraus(bt_state* s, bt_kraus_desc kd, int64_t nmem, const double* rdm, const double* kraus,
                           const double* u, const int* forced, uint64_t rng_stream, int* branch, double* probs,
                           void* pm) {
  bt_ctx* ctx = s->ctx;
  unsigned grid = (unsigned)((nmem + 127) / 128);
  if (s->prec == BT_PREC_C64)
    k_decide_kraus<float><<<grid, 128, 0, ctx->stream>>>(nmem, kd.k, kd.nk, kd.ref_perm, rdm, kraus, u, forced,
                                                         ctx->seed, rng_stream, branch, probs, (float*)pm,
                                                         ctx->d_status);
  else
    k_decide_kraus<double><<<grid, 128, 0, ctx->stream>>>(nmem, kd.k, kd.nk, kd.ref_perm, rdm, kraus, u, forced,
                                                          ctx->seed, rng_stream, branch, probs, (double*)pm,
                                                          ctx->d_status);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "decide_kraus launch");
}
