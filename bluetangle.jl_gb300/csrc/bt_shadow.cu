// Classical-shadow density matrix from snapshots.
//
// The reference (shadow, BlueTangle.jl src/ops.jl:145-185) measures each shot in a
// random basis per qubit (X, Y, Z through H, HSP, I) and adds the snapshot
//   rho_m = (x)_q (3 U_m,q^dagger |b_m,q><b_m,q| U_m,q - I)
// to rho / number_of_experiment.  Here every entry rho[i, j] is one thread summing
// over the snapshots the product over qubits of the 2x2 factor T[code][bit_q(i)]
// [bit_q(j)], code = 2*basis + outcome (6 tables); a factor of a Z-basis qubit is
// diagonal, so most products end at their first mismatching bit.  Sums are FP64;
// the mean divides once at the end.
#include "bt_internal.cuh"

#define BT_SHADOW_TILE 1024  // snapshots staged in shared memory per round

template <typename R>
__global__ void __launch_bounds__(BT_THREADS) k_shadow(typename CT<R>::T* __restrict__ rho, int n, int64_t nsnap,
                                                       const uint8_t* __restrict__ codes, const double* __restrict__ tab,
                                                       double inv_m) {
  __shared__ uint8_t sc[BT_SHADOW_TILE * 16];  // codes of up to 16 qubits per snapshot
  __shared__ double st[6 * 8];
  if (threadIdx.x < 48) st[threadIdx.x] = tab[threadIdx.x];
  const int64_t dim = 1LL << n, total = dim * dim;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // entry i + j * dim
  const bool on = e < total;
  const int64_t i = e & (dim - 1), j = e >> n;
  double sr = 0, si = 0;
  for (int64_t s0 = 0; s0 < nsnap; s0 += BT_SHADOW_TILE) {
    const int cnt = (int)min((int64_t)BT_SHADOW_TILE, nsnap - s0);
    __syncthreads();
    for (int k = threadIdx.x; k < cnt * n; k += blockDim.x) sc[k] = codes[s0 * n + k];
    __syncthreads();
    if (!on) continue;
    for (int s = 0; s < cnt; ++s) {
      double pr = 1, pi = 0;
      const uint8_t* c = sc + s * n;
      bool zero = false;
      for (int q = 0; q < n; ++q) {  // qubit q + 1 is bit n - 1 - q
        const int bi = (int)((i >> (n - 1 - q)) & 1), bj = (int)((j >> (n - 1 - q)) & 1);
        const double* t = st + 8 * c[q] + 2 * (2 * bi + bj);
        const double tr = t[0], ti = t[1];
        if (tr == 0 && ti == 0) {
          zero = true;
          break;
        }
        const double nr = pr * tr - pi * ti;
        pi = pr * ti + pi * tr;
        pr = nr;
      }
      if (!zero) {
        sr += pr;
        si += pi;
      }
    }
  }
  if (on) {
    typename CT<R>::T v;
    v.x = (R)(sr * inv_m);
    v.y = (R)(si * inv_m);
    rho[e] = v;
  }
}

extern "C" int bt_shadow_accumulate(bt_state* rho, int64_t nsnap, const uint8_t* codes, const double* tables) {
  if (!rho) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = rho->ctx;
  if (rho->repr != BT_REPR_DM || rho->batch != 1) return bt_fail(ctx, BT_ERR_BAD_ARG, "need one density matrix");
  if (rho->n > 14) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "shadow density matrices of at most 14 qubits");
  if (nsnap < 1 || !codes || !tables) return bt_fail(ctx, BT_ERR_BAD_ARG, "need snapshots and factor tables");
  const int n = rho->n;
  for (int64_t k = 0; k < nsnap * n; ++k)
    if (codes[k] > 5) return bt_fail(ctx, BT_ERR_BAD_ARG, "snapshot codes are 2*basis + outcome < 6");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  const size_t cb = (size_t)nsnap * n;
  uint8_t* dcodes = nullptr;
  double* dtab = nullptr;
  if ((rc = bt_cuda_check(ctx, cudaMallocAsync((void**)&dcodes, cb + 48 * 8 + 16, ctx->stream), "shadow buffers")))
    return rc;
  dtab = (double*)(((uintptr_t)dcodes + cb + 15) & ~(uintptr_t)15);
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(dcodes, codes, cb, cudaMemcpyHostToDevice, ctx->stream), "codes");
  if (!rc) rc = bt_cuda_check(ctx, cudaMemcpyAsync(dtab, tables, 48 * 8, cudaMemcpyHostToDevice, ctx->stream), "tables");
  if (!rc) {
    const int64_t total = 1LL << (2 * n);
    const unsigned grid = (unsigned)((total + BT_THREADS - 1) / BT_THREADS);
    if (rho->prec == BT_PREC_C64)
      k_shadow<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)rho->d, n, nsnap, dcodes, dtab, 1.0 / nsnap);
    else
      k_shadow<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)rho->d, n, nsnap, dcodes, dtab, 1.0 / nsnap);
    ctx->launches++;
    rc = bt_cuda_check(ctx, cudaGetLastError(), "shadow launch");
  }
  cudaFreeAsync(dcodes, ctx->stream);
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "shadow sync");
  return rc;
}
