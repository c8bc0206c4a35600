// Shot sampling from |psi|^2 (or diag(rho)) with a device prefix sum in FP64,
// and state maintenance kernels (basis states, precision conversion).
//
// sample(psi, shots) in the reference draws with StatsBase's weighted sampler
// (BlueTangle.jl src/ops.jl:46-62): per shot t = u * sum(w) and the outcome is
// the first index whose cumulative weight reaches t.  Here the cumulative
// weights are a two-level prefix: chunk sums of 2^12 weights (one block per
// chunk), an inclusive scan over the chunk sums (one block), then one warp per
// shot binary-searches the chunk prefix and scans the 2^12 weights of the
// chosen chunk with warp shuffles.  Scratch: one double per chunk.
#include "bt_internal.cuh"

#define FULL 0xffffffffu
#define CHUNK_LG 12

template <typename R>
__device__ __forceinline__ double weight(const typename CT<R>::T* s, int dm, int nsys, uint64_t i) {
  if (dm) return (double)s[i + (i << nsys)].x;
  typename CT<R>::T v = s[i];
  return (double)v.x * v.x + (double)v.y * v.y;
}

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_chunk_sums(const typename CT<R>::T* __restrict__ s, int dm, int nsys,
                                                           int clg, double* __restrict__ sums) {
  __shared__ double sh[BT_THREADS / 32];
  const uint64_t c0 = (uint64_t)blockIdx.x << clg;
  double acc = 0;
  for (uint64_t i = threadIdx.x; i < (1ULL << clg); i += blockDim.x) acc += weight<R>(s, dm, nsys, c0 + i);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < BT_THREADS / 32; ++w) t += sh[w];
    sums[blockIdx.x] = t;
  }
}

// in-place inclusive scan of n doubles with one block of 1024 threads
__global__ void __launch_bounds__(1024) k_scan(double* __restrict__ a, int64_t n) {
  __shared__ double sh[1024];
  const int64_t per = (n + 1023) / 1024;
  const int64_t lo = threadIdx.x * per, hi = lo + per < n ? lo + per : n;
  double t = 0;
  for (int64_t i = lo; i < hi; ++i) t += a[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {  // sequential scan of the 1024 segment totals (fixed order)
    double run = 0;
    for (int i = 0; i < 1024; ++i) {
      double v = sh[i];
      sh[i] = run;
      run += v;
    }
  }
  __syncthreads();
  double run = sh[threadIdx.x];
  for (int64_t i = lo; i < hi; ++i) {
    run += a[i];
    a[i] = run;
  }
}

template <typename R>
__global__ void k_shots(const typename CT<R>::T* __restrict__ s, int dm, int nsys, int clg,
                        const double* __restrict__ cum, int64_t nchunk, int64_t shots,
                        const double* __restrict__ u, uint64_t key, uint64_t stream, int64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t shot = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (shot >= shots) return;
  const double total = cum[nchunk - 1];
  const double uu = u ? u[shot] : bt_uniform(key, stream, (uint64_t)shot);
  const double t = uu * total;
  // first chunk with cum >= t
  int64_t lo = 0, hi = nchunk - 1;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (cum[mid] < t) lo = mid + 1; else hi = mid;
  }
  const uint64_t c0 = (uint64_t)lo << clg;
  double run = lo > 0 ? cum[lo - 1] : 0.0;
  int64_t found = -1, lastnz = -1;
  for (uint64_t b = 0; b < (1ULL << clg) && found < 0; b += 32) {
    double w = (b + lane < (1ULL << clg)) ? weight<R>(s, dm, nsys, c0 + b + lane) : 0.0;
    double incl = w;
    for (int o = 1; o < 32; o <<= 1) {
      double v = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += v;
    }
    double cw = run + incl;
    unsigned hit = __ballot_sync(FULL, cw >= t);
    unsigned nz = __ballot_sync(FULL, w > 0);
    if (nz) lastnz = (int64_t)(c0 + b + 31 - __clz(nz));
    if (hit) found = (int64_t)(c0 + b + __ffs(hit) - 1);
    run = __shfl_sync(FULL, cw, 31);
  }
  if (found < 0) found = lastnz >= 0 ? lastnz : (int64_t)c0;  // t beyond the chunk by rounding
  if (lane == 0) out[shot] = found;
}

int bt_launch_sample(bt_state* s, int64_t mem, int64_t shots, const double* d_u, uint64_t seed_stream, int64_t* d_out) {
  bt_ctx* ctx = s->ctx;
  const int nsys = s->n;
  const int dm = s->repr == BT_REPR_DM;
  const int clg = nsys < CHUNK_LG ? nsys : CHUNK_LG;
  const int64_t nchunk = 1LL << (nsys - clg);
  double* cum = nullptr;
  int rc = bt_work(ctx, sizeof(double) * nchunk, &cum);
  if (rc) return rc;
  const char* base = (const char*)s->d + mem * s->member_elems * elem_bytes(s->prec);
  bool f = s->prec == BT_PREC_C64;
  if (f) k_chunk_sums<float><<<(unsigned)nchunk, BT_THREADS, 0, ctx->stream>>>((const float2*)base, dm, nsys, clg, cum);
  else k_chunk_sums<double><<<(unsigned)nchunk, BT_THREADS, 0, ctx->stream>>>((const double2*)base, dm, nsys, clg, cum);
  ctx->launches++;
  k_scan<<<1, 1024, 0, ctx->stream>>>(cum, nchunk);
  ctx->launches++;
  const int64_t threads = shots * 32;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  if (f) k_shots<float><<<grid, 256, 0, ctx->stream>>>((const float2*)base, dm, nsys, clg, cum, nchunk, shots, d_u, ctx->seed, seed_stream, d_out);
  else k_shots<double><<<grid, 256, 0, ctx->stream>>>((const double2*)base, dm, nsys, clg, cum, nchunk, shots, d_u, ctx->seed, seed_stream, d_out);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "sample launch");
}

// One shot from every member of a batch (measure(circuit, shots) draws a single
// shot from each re-simulated state, src/ops.jl:619-630): the same two-level
// prefix per member (chunk sums with blockIdx.y = member, one scan block per
// member), then one warp per member searches its own prefix.
template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_chunk_sums_each(const typename CT<R>::T* __restrict__ s, int dm,
                                                                int nsys, int nbits, int clg, int64_t nchunk,
                                                                double* __restrict__ sums) {
  __shared__ double sh[BT_THREADS / 32];
  const typename CT<R>::T* sm = s + ((int64_t)blockIdx.y << nbits);
  const uint64_t c0 = (uint64_t)blockIdx.x << clg;
  double acc = 0;
  for (uint64_t i = threadIdx.x; i < (1ULL << clg); i += blockDim.x) acc += weight<R>(sm, dm, nsys, c0 + i);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < BT_THREADS / 32; ++w) t += sh[w];
    sums[(int64_t)blockIdx.y * nchunk + blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_each(double* __restrict__ a, int64_t n) {
  double* am = a + (int64_t)blockIdx.x * n;
  __shared__ double sh[1024];
  const int64_t per = (n + 1023) / 1024;
  const int64_t lo = threadIdx.x * per, hi = lo + per < n ? lo + per : n;
  double t = 0;
  for (int64_t i = lo; i < hi; ++i) t += am[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0;
    for (int i = 0; i < 1024; ++i) {
      double v = sh[i];
      sh[i] = run;
      run += v;
    }
  }
  __syncthreads();
  double run = sh[threadIdx.x];
  for (int64_t i = lo; i < hi; ++i) {
    run += am[i];
    am[i] = run;
  }
}

template <typename R>
__global__ void k_shot_each(const typename CT<R>::T* __restrict__ s, int dm, int nsys, int nbits, int clg,
                            const double* __restrict__ cum_all, int64_t nchunk, int64_t nmem,
                            const double* __restrict__ u, uint64_t key, uint64_t stream, int64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t m = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (m >= nmem) return;
  const typename CT<R>::T* sm = s + (m << nbits);
  const double* cum = cum_all + m * nchunk;
  const double total = cum[nchunk - 1];
  const double uu = u ? u[m] : bt_uniform(key, stream, (uint64_t)m);
  const double t = uu * total;
  int64_t lo = 0, hi = nchunk - 1;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (cum[mid] < t) lo = mid + 1; else hi = mid;
  }
  const uint64_t c0 = (uint64_t)lo << clg;
  double run = lo > 0 ? cum[lo - 1] : 0.0;
  int64_t found = -1, lastnz = -1;
  for (uint64_t b = 0; b < (1ULL << clg) && found < 0; b += 32) {
    double w = (b + lane < (1ULL << clg)) ? weight<R>(sm, dm, nsys, c0 + b + lane) : 0.0;
    double incl = w;
    for (int o = 1; o < 32; o <<= 1) {
      double v = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += v;
    }
    double cw = run + incl;
    unsigned hit = __ballot_sync(FULL, cw >= t);
    unsigned nz = __ballot_sync(FULL, w > 0);
    if (nz) lastnz = (int64_t)(c0 + b + 31 - __clz(nz));
    if (hit) found = (int64_t)(c0 + b + __ffs(hit) - 1);
    run = __shfl_sync(FULL, cw, 31);
  }
  if (found < 0) found = lastnz >= 0 ? lastnz : (int64_t)c0;
  if (lane == 0) out[m] = found;
}

int bt_launch_sample_each(bt_state* s, const double* d_u, uint64_t seed_stream, int64_t* d_out) {
  bt_ctx* ctx = s->ctx;
  const int nsys = s->n;
  const int dm = s->repr == BT_REPR_DM;
  const int clg = nsys < CHUNK_LG ? nsys : CHUNK_LG;
  const int64_t nchunk = 1LL << (nsys - clg);
  const int64_t B = s->batch;
  if (B > 65535) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 65535 members per call");
  double* cum = nullptr;
  int rc = bt_work(ctx, sizeof(double) * nchunk * B, &cum);
  if (rc) return rc;
  const bool f = s->prec == BT_PREC_C64;
  dim3 g1((unsigned)nchunk, (unsigned)B);
  if (f) k_chunk_sums_each<float><<<g1, BT_THREADS, 0, ctx->stream>>>((const float2*)s->d, dm, nsys, s->nbits, clg, nchunk, cum);
  else k_chunk_sums_each<double><<<g1, BT_THREADS, 0, ctx->stream>>>((const double2*)s->d, dm, nsys, s->nbits, clg, nchunk, cum);
  ctx->launches++;
  k_scan_each<<<(unsigned)B, 1024, 0, ctx->stream>>>(cum, nchunk);
  ctx->launches++;
  const unsigned grid = (unsigned)((B * 32 + 255) / 256);
  if (f) k_shot_each<float><<<grid, 256, 0, ctx->stream>>>((const float2*)s->d, dm, nsys, s->nbits, clg, cum, nchunk, B, d_u, ctx->seed, seed_stream, d_out);
  else k_shot_each<double><<<grid, 256, 0, ctx->stream>>>((const double2*)s->d, dm, nsys, s->nbits, clg, cum, nchunk, B, d_u, ctx->seed, seed_stream, d_out);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "sample_each launch");
}

template <typename R>
__global__ void k_probs(const typename CT<R>::T* __restrict__ s, int dm, int nsys, int64_t offset, int64_t len,
                        double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = weight<R>(s, dm, nsys, (uint64_t)(offset + i));
}

int bt_launch_probs(bt_state* s, int64_t mem, int64_t offset, int64_t len, double* d_out) {
  bt_ctx* ctx = s->ctx;
  const char* base = (const char*)s->d + mem * s->member_elems * elem_bytes(s->prec);
  int grid = bt_grid(ctx, len);
  int dm = s->repr == BT_REPR_DM;
  if (s->prec == BT_PREC_C64) k_probs<float><<<grid, BT_THREADS, 0, ctx->stream>>>((const float2*)base, dm, s->n, offset, len, d_out);
  else k_probs<double><<<grid, BT_THREADS, 0, ctx->stream>>>((const double2*)base, dm, s->n, offset, len, d_out);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "probs launch");
}

// ------------------------------------------------------------ state maintenance
template <typename R>
__global__ void k_set_basis(typename CT<R>::T* __restrict__ p, int nbits, int64_t mem_lo, int64_t nmem, uint64_t index) {
  const int64_t per = 1LL << nbits;
  const int64_t total = per * nmem;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t & (per - 1);
    typename CT<R>::T v;
    v.x = (uint64_t)i == index ? (R)1 : (R)0;
    v.y = 0;
    p[((mem_lo + (t >> nbits)) << nbits) + i] = v;
  }
}

int bt_launch_set_basis(bt_state* s, int64_t mem_lo, int64_t nmem, uint64_t index) {
  bt_ctx* ctx = s->ctx;
  int64_t work = s->member_elems * nmem;
  int grid = bt_grid(ctx, work, BT_THREADS, 32);
  if (s->prec == BT_PREC_C64) k_set_basis<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d, s->nbits, mem_lo, nmem, index);
  else k_set_basis<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d, s->nbits, mem_lo, nmem, index);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "set_basis launch");
}

__global__ void k_d2f(const double2* __restrict__ src, float2* __restrict__ dst, int64_t len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    double2 v = src[i];
    dst[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_f2d(const float2* __restrict__ src, double2* __restrict__ dst, int64_t len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    float2 v = src[i];
    dst[i] = make_double2((double)v.x, (double)v.y);
  }
}

int bt_launch_convert_in(bt_state* s, int64_t mem, int64_t offset, int64_t len, const double* d_src) {
  bt_ctx* ctx = s->ctx;
  float2* dst = (float2*)s->d + mem * s->member_elems + offset;
  k_d2f<<<bt_grid(ctx, len), BT_THREADS, 0, ctx->stream>>>((const double2*)d_src, dst, len);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "convert launch");
}

int bt_launch_convert_out(bt_state* s, int64_t mem, int64_t offset, int64_t len, double* d_dst) {
  bt_ctx* ctx = s->ctx;
  const float2* src = (const float2*)s->d + mem * s->member_elems + offset;
  k_f2d<<<bt_grid(ctx, len), BT_THREADS, 0, ctx->stream>>>(src, (double2*)d_dst, len);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "convert launch");
}

// ------------------------------------------------------------ allocation-free sampling
// bt_sample_noalloc: the sampler above for callers that must not allocate device
// memory.  Its only scratch, the chunk-sum prefix, lives in this file-scope
// device array, so the entry point calls no cudaMalloc/cudaFree and allocates
// nothing on the host side of the CUDA runtime either.
//   size: BT_NOALLOC_CHUNKS doubles (512 KiB), i.e. states of at most
//         2^(12 + 16) = 2^28 amplitudes (n <= 28); every GPU that loads the
//         library holds the array until the process exits.
//   sharing: every device holds its own copy of the array; all calls on one
//         device share that copy, and it keeps the last call's contents.  Each
//         call overwrites every entry it reads before reading it (chunk sums,
//         then the in-place scan), so nothing needs clearing, but calls on the
//         same device whose work overlaps on the GPU (different streams, or
//         host threads) race on it.  Calls on different devices never race.
//   address: the array's device address is looked up once per device and kept
//         for the life of the process; after cudaDeviceReset (or anything else
//         that destroys the device's primary context) it is stale, so a process
//         that resets a device must not call this entry point on it again.
#define BT_NOALLOC_CHUNKS (1 << 16)
#define BT_NOALLOC_MAX_QUBITS (CHUNK_LG + 16)
static __device__ __align__(256) double g_noalloc_cum[BT_NOALLOC_CHUNKS];

#include <mutex>
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64];  // device address of g_noalloc_cum, per device

// Host code must not take the address of g_noalloc_cum directly (that is a
// host-side shadow, not a device address): it asks the runtime once per device,
// with that device current.
static int noalloc_scratch(int dev, double** out) {
  if (dev < 0 || dev >= 64) return bt_fail(nullptr, BT_ERR_DEVICE, "device index beyond 63");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_cum);
    if (e != cudaSuccess || !p)
      return bt_fail(nullptr, BT_ERR_DEVICE, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_ptr[dev];
  return BT_OK;
}

extern "C" int bt_sample_noalloc(const void* d_state, int n, int prec, int64_t shots, const double* d_uniforms,
                                 uint64_t key, uint64_t seed, int64_t* d_out, void* stream) {
  if (!d_state || (shots > 0 && !d_out)) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state or output pointer is NULL");
  if (prec != BT_PREC_C128 && prec != BT_PREC_C64) return bt_fail(nullptr, BT_ERR_BAD_ARG, "prec must be C128 or C64");
  if (n < 1 || n > BT_NOALLOC_MAX_QUBITS)
    return bt_fail(nullptr, BT_ERR_BAD_ARG,
                   "bt_sample_noalloc supports 1 <= n <= 28 qubits (its static prefix holds 65536 chunk sums)");
  if (shots < 0 || shots > (1LL << 33)) return bt_fail(nullptr, BT_ERR_BAD_ARG, "shots must be in [0, 2^33]");
  if (shots == 0) return BT_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return bt_fail(nullptr, BT_ERR_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  double* cum = nullptr;
  int rc = noalloc_scratch(dev, &cum);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int clg = n < CHUNK_LG ? n : CHUNK_LG;
  const int64_t nchunk = 1LL << (n - clg);
  const bool f = prec == BT_PREC_C64;
  if (f) k_chunk_sums<float><<<(unsigned)nchunk, BT_THREADS, 0, st>>>((const float2*)d_state, 0, n, clg, cum);
  else k_chunk_sums<double><<<(unsigned)nchunk, BT_THREADS, 0, st>>>((const double2*)d_state, 0, n, clg, cum);
  k_scan<<<1, 1024, 0, st>>>(cum, nchunk);
  const unsigned grid = (unsigned)((shots * 32 + 255) / 256);
  const uint64_t sstream = seed ^ 0x53414d5000000000ULL;
  if (f) k_shots<float><<<grid, 256, 0, st>>>((const float2*)d_state, 0, n, clg, cum, nchunk, shots, d_uniforms, key, sstream, d_out);
  else k_shots<double><<<grid, 256, 0, st>>>((const double2*)d_state, 0, n, clg, cum, nchunk, shots, d_uniforms, key, sstream, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return bt_fail(nullptr, BT_ERR_DEVICE, std::string("sample launch: ") + cudaGetErrorString(e));
  return BT_OK;
}
