// Tensor-core fused passes (complex64): every register phase of a fused tile pass
// applied as one dense 32 x 32 complex block on the 5th-generation tensor cores
// (tcgen05.mma kind::tf32), in three TF32 products with FP32 accumulation.
//
// A fused pass (planner: bt_plan.cu) holds a tile of 2^13 amplitudes whose gates
// are grouped into phases of 5 register bits.  For the tensor-core form the host
// multiplies the gates of each phase into one 32 x 32 unitary U (complex128) and
// writes its real form
//     [Re out_j']   [ Re U  -Im U ] [Re in_j]
//     [Im out_j'] = [ Im U   Re U ] [Im in_j]     (rows 2j'+c', columns 2j+c)
// as the MMA's B operand, split into TF32 hi and lo parts (bt_tc_block_image).  On
// the device a tile's 256 columns (the 8 non-block tile bits) are the MMA's A
// operand rows, each row the column's 32 amplitudes as 64 reals (split into hi and
// lo the same way), and D = A B^T, 256 x 64 in FP32, lands in tensor memory:
//     D = A_hi B_hi + A_hi B_lo + A_lo B_hi
// (hi and lo both rounded to TF32, so each operand carries about 22 bits; the
// product of the two lo parts is at that level too).  Thread t owns column
// t: it writes the column's row of A, reads the row of D back with tcgen05.ld,
// and the amplitudes move between phases through an amplitude-indexed shared
// tile, as the scalar passes do.  One CTA per SM (194 KiB of shared memory):
//     [0, 64K)    A hi (256 rows x 64 TF32) -- also the amplitude tile between phases
//     [64K,128K)  A lo
//     [128K,192K) two buffers of a phase's B (hi and lo, 64 x 64 each): the next
//                 phase's block is copied in (one bulk copy, mbarrier completion)
//                 while the current one runs
//     [192K,194K) run offsets of the tile; then the mbarriers, the TMEM address, a flag
// Each CTA asks L2 for its next tile when it starts a tile.
// Operands use the K-major layout without swizzle: 8-row x 16-byte core matrices,
// element (r, k) at (r / 8) * 2048 + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4
// bytes; adjacent core matrices along K are 128 bytes apart (the descriptor's
// leading byte offset), along rows 2048 (its stride byte offset).
#include "bt_internal.cuh"
#include "bt_tc.cuh"

#include <string.h>

#include <algorithm>

#define TC_THREADS 256
#define TC_SMEM (194 * 1024 + 256)

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading (K-direction) and stride
// (row-direction) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

// bounded wait for the given phase parity of an mbarrier; false after the limit
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 24); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_ld32(uint32_t ta, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// x as hi + lo, both TF32 values rounded to nearest (cvt.rna): |x - hi - lo| is
// within 2^-22 |x| (the tensor cores would truncate an unrounded lo)
__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
__device__ __forceinline__ void tc_split(float x, float& hi, float& lo) {
  hi = tc_tf32(x);
  lo = tc_tf32(x - hi);
}

__device__ __forceinline__ int tc_swz(int l) { return l ^ ((l >> 4) & 15); }

__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_pass(float2* __restrict__ psi, const TcPass a,
                                                          int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  float2* E = reinterpret_cast<float2*>(sm);
  unsigned char* Ahi = sm;
  unsigned char* Alo = sm + 65536;
  unsigned char* Bbuf = sm + 131072;  // buffer b at Bbuf + 32768 b: hi, then lo at +16384
  int64_t* runoff = reinterpret_cast<int64_t*>(sm + 196608);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + 196608 + 2048);  // MMA completion
  uint64_t* bbar = mbar + 1;                                        // B buffers 0, 1
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 3);
  int* sflag = reinterpret_cast<int*>(mbar + 3) + 1;
  const int t = threadIdx.x;
  const int M = 13, c = a.c, NP = a.nphase;
  for (int r = t; r < (1 << (M - c)); r += TC_THREADS) {
    int64_t v = 0;
    for (int b = 0; b < M - c; ++b) v |= (int64_t)((r >> b) & 1) << a.tbits[c + b];
    runoff[r] = v;
  }
  if (t == 0) {
    for (int b = 0; b < 3; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(mbar + b)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *sflag = 0;
  }
  if (t < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)), "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc(128, 64);
  const uint32_t bar = tc_smem(mbar);
  uint32_t parity = 0;
  const int64_t per = 1LL << a.lg_tiles, total = per * a.nmem;
  const int cmask = (1 << c) - 1;
  // this thread's row of D in tensor memory: lanes 32 (w % 4) .., columns 64 (w / 4) ..
  const int w = t >> 5;
  const uint32_t drow = tmem + ((uint32_t)(32 * (w & 3)) << 16) + 64 * (w >> 2);
  // this thread's row of A (column t of the tile)
  const int arow = (t >> 3) * 2048 + (t & 7) * 16;
  auto tile_base = [&](int64_t tid) {
    const int64_t mem = a.member_lo + (tid >> a.lg_tiles);
    uint64_t base = (uint64_t)(tid & (per - 1));
    for (int i = 0; i < M; ++i) {
      const int p = a.tbits[i];
      base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
    }
    return psi + (mem << a.nbits) + base;
  };
  // the B operand of phase `ph` into buffer `buf` (thread 0): one 32 KiB bulk copy
  // completing on that buffer's mbarrier
  auto fetch_b = [&](int ph, int buf) {
    const uint32_t bb = tc_smem(bbar + buf);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb), "r"(32768) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            tc_smem(Bbuf + 32768 * buf)),
        "l"(a.bmat + (size_t)ph * 8192), "r"(32768), "r"(bb)
        : "memory");
  };
  uint32_t gph = 0;  // phases this CTA has run: B buffer gph & 1, its use count gph >> 1
  if (t == 0) fetch_b(0, 0);
  bool failed = false;
  for (int64_t tid = blockIdx.x; tid < total && !failed; tid += gridDim.x) {
    float2* g = tile_base(tid);
    // L2 prefetch of this CTA's next tile: one 256-byte run per thread
    if (tid + gridDim.x < total && t < (1 << (M - c))) {
      const float2* gn = tile_base(tid + gridDim.x) + runoff[t];
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(gn), "r"(8 << c) : "memory");
    }
    // the tile into the amplitude-indexed shared tile, 16-byte loads
    {
      float4 buf[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int l = (t + i * TC_THREADS) * 2;
        buf[i] = *reinterpret_cast<const float4*>(g + runoff[l >> c] + (l & cmask));
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int l = (t + i * TC_THREADS) * 2;
        E[tc_swz(l)] = make_float2(buf[i].x, buf[i].y);
        E[tc_swz(l + 1)] = make_float2(buf[i].z, buf[i].w);
      }
    }
    __syncthreads();
    float re[32], im[32];
    for (int p = 0; p < NP && !failed; ++p, ++gph) {
      // column t under this phase: its tile bits outside the block, and the
      // block's register offsets
      int lbase = 0;
      {
        int nb = 0;
        uint32_t rm = 0;
        for (int b = 0; b < 5; ++b) rm |= 1u << a.reg[p][b];
        for (int bit = 0; bit < M; ++bit)
          if (!((rm >> bit) & 1)) {
            if ((t >> nb) & 1) lbase |= 1 << bit;
            ++nb;
          }
      }
      int off[32];
      off[0] = 0;
#pragma unroll
      for (int j = 1; j < 32; ++j) off[j] = off[j & (j - 1)] | (1 << a.reg[p][__ffs(j) - 1]);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const float2 v = E[tc_swz(lbase | off[j])];
        re[j] = v.x;
        im[j] = v.y;
      }
      // the next phase's block (this tile's, or phase 0 of the next tile) into the
      // other buffer, whose last reader (the previous phase's MMAs) has completed
      if (t == 0) {
        if (p + 1 < NP) fetch_b(p + 1, (gph + 1) & 1);
        else if (tid + gridDim.x < total) fetch_b(0, (gph + 1) & 1);
      }
      __syncthreads();  // every thread has read the shared tile before A overwrites it
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float4 h, l;
        tc_split(re[2 * q], h.x, l.x);
        tc_split(im[2 * q], h.y, l.y);
        tc_split(re[2 * q + 1], h.z, l.z);
        tc_split(im[2 * q + 1], h.w, l.w);
        *reinterpret_cast<float4*>(Ahi + arow + q * 128) = h;
        *reinterpret_cast<float4*>(Alo + arow + q * 128) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (t == 0) {
        const int bsel = gph & 1;
        if (!tc_wait(tc_smem(bbar + bsel), (gph >> 1) & 1)) {  // this phase's block has landed
          atomicExch(status, BT_STATUS_TC_TIMEOUT);
          *sflag = 1;
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t ah = tc_smem(Ahi), al = tc_smem(Alo), bh = tc_smem(Bbuf + 32768 * bsel), bl = bh + 16384;
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const uint32_t d = tmem + 64 * half, ar = 32768u * half;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
              const uint32_t ko = 256u * s;
              tc_mma(d, tc_desc(ah + ar + ko, 128, 2048), tc_desc(bh + ko, 128, 2048), idesc, s > 0);
              tc_mma(d, tc_desc(ah + ar + ko, 128, 2048), tc_desc(bl + ko, 128, 2048), idesc, 1);
              tc_mma(d, tc_desc(al + ar + ko, 128, 2048), tc_desc(bh + ko, 128, 2048), idesc, 1);
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                       : "memory");
        }
      }
      __syncthreads();  // thread 0's check of the block copy
      if (*sflag) {
        failed = true;
        break;
      }
      const bool ok = tc_wait(bar, parity);
      parity ^= 1;
      if (!ok) {
        atomicExch(status, BT_STATUS_TC_TIMEOUT);
        *sflag = 1;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (ok) {
        float v[32];
        tc_ld32(drow, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) re[j] = v[2 * j], im[j] = v[2 * j + 1];
        tc_ld32(drow + 32, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) re[16 + j] = v[2 * j], im[16 + j] = v[2 * j + 1];
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      // the column back into the shared tile (A is free: the MMAs have completed)
#pragma unroll
      for (int j = 0; j < 32; ++j) E[tc_swz(lbase | off[j])] = make_float2(re[j], im[j]);
      __syncthreads();
      failed = *sflag != 0;
    }
    if (failed) break;
    // the tile back to global memory, 16-byte stores
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int l = (t + i * TC_THREADS) * 2;
      const float2 u = E[tc_swz(l)], v = E[tc_swz(l + 1)];
      *reinterpret_cast<float4*>(g + runoff[l >> c] + (l & cmask)) = make_float4(u.x, u.y, v.x, v.y);
    }
    __syncthreads();
  }
  if (failed && t == 0) {  // once more for work still in flight: the last MMAs, the prefetched block
    tc_wait(bar, parity ^ 1);
    tc_wait(tc_smem(bbar + ((gph + 1) & 1)), ((gph + 1) >> 1) & 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
}

int bt_launch_tc_pass(bt_ctx* ctx, void* psi, const TcPass& a) {
  static bool attr[64] = {false};
  if (ctx->device < 64 && !attr[ctx->device]) {
    cudaError_t e = cudaFuncSetAttribute(k_tc_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return bt_cuda_check(ctx, e, "tensor-core pass smem attribute");
    attr[ctx->device] = true;
  }
  const int64_t total = (1LL << a.lg_tiles) * a.nmem;
  int64_t grid = ctx->sm_count;
  if (grid > total) grid = total;
  k_tc_pass<<<(unsigned)grid, TC_THREADS, TC_SMEM, ctx->stream>>>((float2*)psi, a, ctx->d_status);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "tensor-core pass launch");
}

// ------------------------------------------------------------------ host side
// x rounded to the nearest TF32 value (ties away from zero, as cvt.rna)
static float tf32_round(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  float y;
  memcpy(&y, &u, 4);
  return y;
}

void bt_tc_block_image(const double* u, float* out) {
  // element (n, k) of a 64 x 64 K-major operand, core matrices 8 x 16 B
  auto at = [](int n, int k) { return ((n / 8) * 2048 + (k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4) / 4; };
  for (int jo = 0; jo < 32; ++jo)
    for (int ji = 0; ji < 32; ++ji) {
      const double ur = u[2 * (jo * 32 + ji)], ui = u[2 * (jo * 32 + ji) + 1];
      const double val[2][2] = {{ur, -ui}, {ui, ur}};  // [c'][c]
      for (int co = 0; co < 2; ++co)
        for (int ci = 0; ci < 2; ++ci) {
          const double x = val[co][ci];
          const float hi = tf32_round((float)x);
          const float lo = tf32_round((float)(x - (double)hi));
          const int e = at(2 * jo + co, 2 * ji + ci);
          out[e] = hi;
          out[4096 + e] = lo;
        }
    }
}

// ------------------------------------------------------------------ TF32 throughput
// Every CTA issues `iters` x 4 MMAs (M = 128, N = 256, K = 8) on fixed operands
// in shared memory into one tensor-memory accumulator; flops = 2 M N K per MMA.
__global__ void __launch_bounds__(128, 1) k_tc_peak(int iters, int* __restrict__ status, float* __restrict__ sink) {
  extern __shared__ __align__(1024) unsigned char sm[];
  float* s = reinterpret_cast<float*>(sm);  // A 128 x 32 (16 KiB), B 256 x 32 (32 KiB)
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + 49152);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 49152 + 8);
  const int t = threadIdx.x;
  for (int e = t; e < 12288; e += blockDim.x) s[e] = 1.0f / (1 + (e & 7));
  if (t == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(mbar)));
  if (t < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)), "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  if (t == 0) {
    const uint32_t sa = tc_smem(s), sb = sa + 16384;
    for (int it = 0; it < iters; ++it)
      for (int k = 0; k < 4; ++k)
        tc_mma(tmem, tc_desc(sa + 256 * k, 128, 1024), tc_desc(sb + 256 * k, 128, 1024), tc_idesc(128, 256),
               (it | k) != 0);
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(mbar))
                 : "memory");
  }
  bool ok = false;
  for (int r = 0; r < 64 && !ok; ++r) ok = tc_wait(tc_smem(mbar), 0);
  if (!ok) atomicExch(status, BT_STATUS_TC_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok && t < 32) {
    uint32_t r0;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r0) : "r"(tmem));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (t == 0) sink[blockIdx.x] = __uint_as_float(r0);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (t < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
}

extern "C" int bt_tc_tf32_peak(bt_ctx* ctx, int iters, double* tflops) {
  if (!ctx || !tflops || iters < 1) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad arguments");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  const int smem = 49152 + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_tc_peak, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return bt_cuda_check(ctx, e, "peak smem attribute");
  float* sink = nullptr;
  if ((rc = bt_cuda_check(ctx, cudaMalloc(&sink, sizeof(float) * ctx->sm_count), "peak sink"))) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_tc_peak<<<ctx->sm_count, 128, smem, ctx->stream>>>(std::min(iters, 64), ctx->d_status, sink);  // warm-up
  cudaEventRecord(e0, ctx->stream);
  k_tc_peak<<<ctx->sm_count, 128, smem, ctx->stream>>>(iters, ctx->d_status, sink);
  cudaEventRecord(e1, ctx->stream);
  e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return bt_cuda_check(ctx, e, "peak run");
  int st = 0;
  if ((rc = bt_cuda_check(ctx, cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status"))) return rc;
  if (st) {
    cudaMemset(ctx->d_status, 0, sizeof(int));
    return bt_fail(ctx, BT_ERR_TIMEOUT, "tensor-core wait timed out");
  }
  *tflops = 2.0 * 128 * 256 * 8 * 4 * (double)iters * ctx->sm_count / (ms * 1e-3) / 1e12;
  return BT_OK;
}
