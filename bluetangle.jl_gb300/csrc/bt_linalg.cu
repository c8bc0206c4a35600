// Dense linear algebra on density matrices and state preparation:
//   bt_fidelity_dm      fidelity(rho, sigma) = tr(sqrt(sqrt(rho) sigma sqrt(rho)))^2
//                       (BlueTangle.jl src/tensor.jl:222-229)
//   bt_rho_accumulate   rho += w * sum_m |psi_m><psi_m| over the members of a state
//                       (measure's density_matrix option, src/ops.jl:612, :626)
//   bt_state_random     random_state(N) = normalize(rand(ComplexF64, 2^N))
//                       (src/hilbert.jl:882), drawn on the device
//
// The reference computes sqrt of a dense Matrix on the host.  Here both square
// roots come from Hermitian eigendecompositions on the device: with
// rho = V diag(w) V^dagger, sqrt(rho) sigma sqrt(rho) is unitarily similar to
// T = D (V^dagger sigma V) D with D = diag(sqrt(max(w, 0))), so the fidelity is
// (sum_i sqrt(max(mu_i, 0)))^2 over the eigenvalues mu of T.  The eigensolver
// (cuSOLVER zheevd) and the products (cuBLAS zgemm) are library routines loaded
// with dlopen on first use, so the library has no link-time dependency on them.
#include <dlfcn.h>

#include <cmath>
#include <mutex>
#include <vector>

#include <cublas_v2.h>
#include <cusolverDn.h>

#include "bt_internal.cuh"

// ------------------------------------------------------------------ dlopen'ed libraries
struct DenseLibs {
  bool ok = false;
  cusolverStatus_t (*dn_create)(cusolverDnHandle_t*);
  cusolverStatus_t (*dn_destroy)(cusolverDnHandle_t);
  cusolverStatus_t (*dn_set_stream)(cusolverDnHandle_t, cudaStream_t);
  cusolverStatus_t (*heevd_size)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, const cuDoubleComplex*,
                                 int, const double*, int*);
  cusolverStatus_t (*heevd)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int, cuDoubleComplex*, int,
                            double*, cuDoubleComplex*, int, int*);
  cublasStatus_t (*bl_create)(cublasHandle_t*);
  cublasStatus_t (*bl_destroy)(cublasHandle_t);
  cublasStatus_t (*bl_set_stream)(cublasHandle_t, cudaStream_t);
  cublasStatus_t (*zgemm)(cublasHandle_t, cublasOperation_t, cublasOperation_t, int, int, int, const cuDoubleComplex*,
                          const cuDoubleComplex*, int, const cuDoubleComplex*, int, const cuDoubleComplex*,
                          cuDoubleComplex*, int);
};

static void* open_first(const char* const* names) {
  for (const char* const* n = names; *n; ++n)
    if (void* h = dlopen(*n, RTLD_NOW | RTLD_LOCAL)) return h;
  return nullptr;
}

static DenseLibs* dense_libs() {
  static DenseLibs L;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* sv[] = {"libcusolver.so", "libcusolver.so.12", "libcusolver.so.11",
                        "/usr/local/cuda/lib64/libcusolver.so", nullptr};
    const char* bl[] = {"libcublas.so", "libcublas.so.13", "libcublas.so.12", "/usr/local/cuda/lib64/libcublas.so",
                        nullptr};
    void* hs = open_first(sv);
    void* hb = open_first(bl);
    if (!hs || !hb) return;
    L.dn_create = (decltype(L.dn_create))dlsym(hs, "cusolverDnCreate");
    L.dn_destroy = (decltype(L.dn_destroy))dlsym(hs, "cusolverDnDestroy");
    L.dn_set_stream = (decltype(L.dn_set_stream))dlsym(hs, "cusolverDnSetStream");
    L.heevd_size = (decltype(L.heevd_size))dlsym(hs, "cusolverDnZheevd_bufferSize");
    L.heevd = (decltype(L.heevd))dlsym(hs, "cusolverDnZheevd");
    L.bl_create = (decltype(L.bl_create))dlsym(hb, "cublasCreate_v2");
    L.bl_destroy = (decltype(L.bl_destroy))dlsym(hb, "cublasDestroy_v2");
    L.bl_set_stream = (decltype(L.bl_set_stream))dlsym(hb, "cublasSetStream_v2");
    L.zgemm = (decltype(L.zgemm))dlsym(hb, "cublasZgemm_v2");
    L.ok = L.dn_create && L.dn_destroy && L.dn_set_stream && L.heevd_size && L.heevd && L.bl_create && L.bl_destroy &&
           L.bl_set_stream && L.zgemm;
  });
  return L.ok ? &L : nullptr;
}

// device buffers of one call, freed on every return path
struct DevBufs {
  std::vector<void*> p;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T>
  int get(bt_ctx* ctx, size_t count, T** out) {
    void* q = nullptr;
    int rc = bt_cuda_check(ctx, cudaMalloc(&q, count * sizeof(T)), "dense linear algebra workspace");
    if (rc) return rc;
    p.push_back(q);
    *out = (T*)q;
    return BT_OK;
  }
};

// member `m` of a density state as a complex128 column-major d x d matrix (the
// state layout already is column-major: rho[i + j d])
template <typename R>
__global__ void k_to_c128(const typename CT<R>::T* __restrict__ src, double2* __restrict__ dst, int64_t len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    typename CT<R>::T v = src[i];
    dst[i] = make_double2((double)v.x, (double)v.y);
  }
}

static int member_c128(bt_state* s, int64_t m, double2* dst) {
  bt_ctx* ctx = s->ctx;
  const int64_t len = s->member_elems;
  if (s->prec == BT_PREC_C128)
    return bt_cuda_check(ctx, cudaMemcpyAsync(dst, (const double2*)s->d + m * len, len * sizeof(double2),
                                              cudaMemcpyDeviceToDevice, ctx->stream),
                         "member copy");
  k_to_c128<float><<<bt_grid(ctx, len), BT_THREADS, 0, ctx->stream>>>((const float2*)s->d + m * len, dst, len);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "member convert");
}

// T[i, j] *= sqrt(max(w_i, 0)) * sqrt(max(w_j, 0)) (column-major d x d)
__global__ void k_scale_rows_cols(double2* __restrict__ t, const double* __restrict__ w, int d) {
  const int64_t len = (int64_t)d * d;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % d), j = (int)(e / d);
    const double s = sqrt(fmax(w[i], 0.0)) * sqrt(fmax(w[j], 0.0));
    double2 v = t[e];
    t[e] = make_double2(v.x * s, v.y * s);
  }
}

// out = (sum_i sqrt(max(mu_i, 0)))^2 in a fixed order (one thread)
__global__ void k_root_sum_sq(const double* __restrict__ mu, int d, double* __restrict__ out) {
  if (threadIdx.x || blockIdx.x) return;
  double t = 0;
  for (int i = 0; i < d; ++i) t += sqrt(fmax(mu[i], 0.0));
  *out = t * t;
}

static int heevd(bt_ctx* ctx, DenseLibs* L, cusolverDnHandle_t h, DevBufs& bufs, bool vectors, int d, double2* a,
                 double* w, int* info) {
  const cusolverEigMode_t mode = vectors ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
  int lwork = 0;
  if (L->heevd_size(h, mode, CUBLAS_FILL_MODE_LOWER, d, (const cuDoubleComplex*)a, d, w, &lwork) !=
      CUSOLVER_STATUS_SUCCESS)
    return bt_fail(ctx, BT_ERR_DEVICE, "cusolverDnZheevd_bufferSize failed");
  double2* work = nullptr;
  int rc = bufs.get(ctx, (size_t)(lwork > 0 ? lwork : 1), &work);
  if (rc) return rc;
  if (L->heevd(h, mode, CUBLAS_FILL_MODE_LOWER, d, (cuDoubleComplex*)a, d, w, (cuDoubleComplex*)work, lwork, info) !=
      CUSOLVER_STATUS_SUCCESS)
    return bt_fail(ctx, BT_ERR_DEVICE, "cusolverDnZheevd failed");
  return BT_OK;
}

extern "C" {

int bt_fidelity_dm(const bt_state* a_, int64_t am, const bt_state* b_, int64_t bm, double* out) {
  if (!a_ || !b_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* a = const_cast<bt_state*>(a_);
  bt_state* b = const_cast<bt_state*>(b_);
  bt_ctx* ctx = a->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  if (a->repr != BT_REPR_DM || b->repr != BT_REPR_DM || a->n != b->n)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "fidelity(rho, sigma) needs two density matrices of equal size");
  if (am < 0 || am >= a->batch || bm < 0 || bm >= b->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  if (a->n > 14) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "fidelity(rho, sigma) supports n <= 14");
  DenseLibs* L = dense_libs();
  if (!L) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "cuSOLVER / cuBLAS could not be loaded");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  if (b->ctx != ctx) cudaStreamSynchronize(b->ctx->stream);
  const int d = 1 << a->n;
  const size_t dd = (size_t)d * d;
  DevBufs bufs;
  double2 *V, *S, *T;
  double *w, *mu, *res;
  int* info;
  if ((rc = bufs.get(ctx, dd, &V)) || (rc = bufs.get(ctx, dd, &S)) || (rc = bufs.get(ctx, dd, &T)) ||
      (rc = bufs.get(ctx, (size_t)d, &w)) || (rc = bufs.get(ctx, (size_t)d, &mu)) || (rc = bufs.get(ctx, 1, &res)) ||
      (rc = bufs.get(ctx, 2, &info)))
    return rc;
  if ((rc = member_c128(a, am, V)) || (rc = member_c128(b, bm, S))) return rc;
  cusolverDnHandle_t hs = nullptr;
  cublasHandle_t hb = nullptr;
  if (L->dn_create(&hs) != CUSOLVER_STATUS_SUCCESS) return bt_fail(ctx, BT_ERR_DEVICE, "cusolverDnCreate failed");
  if (L->bl_create(&hb) != CUBLAS_STATUS_SUCCESS) {
    L->dn_destroy(hs);
    return bt_fail(ctx, BT_ERR_DEVICE, "cublasCreate failed");
  }
  L->dn_set_stream(hs, ctx->stream);
  L->bl_set_stream(hb, ctx->stream);
  const cuDoubleComplex one = {1.0, 0.0}, zero = {0.0, 0.0};
  // rho = V diag(w) V^dagger
  rc = heevd(ctx, L, hs, bufs, true, d, V, w, info);
  // T = V^dagger (sigma V): S <- sigma V is written into T first, then T <- V^dagger S
  if (!rc && L->zgemm(hb, CUBLAS_OP_N, CUBLAS_OP_N, d, d, d, &one, (const cuDoubleComplex*)S, d,
                      (const cuDoubleComplex*)V, d, &zero, (cuDoubleComplex*)T, d) != CUBLAS_STATUS_SUCCESS)
    rc = bt_fail(ctx, BT_ERR_DEVICE, "cublasZgemm failed");
  if (!rc && L->zgemm(hb, CUBLAS_OP_C, CUBLAS_OP_N, d, d, d, &one, (const cuDoubleComplex*)V, d,
                      (const cuDoubleComplex*)T, d, &zero, (cuDoubleComplex*)S, d) != CUBLAS_STATUS_SUCCESS)
    rc = bt_fail(ctx, BT_ERR_DEVICE, "cublasZgemm failed");
  if (!rc) {
    k_scale_rows_cols<<<bt_grid(ctx, (int64_t)dd), BT_THREADS, 0, ctx->stream>>>(S, w, d);
    ctx->launches++;
    rc = bt_cuda_check(ctx, cudaGetLastError(), "scale launch");
  }
  if (!rc) rc = heevd(ctx, L, hs, bufs, false, d, S, mu, info + 1);
  if (!rc) {
    k_root_sum_sq<<<1, 32, 0, ctx->stream>>>(mu, d, res);
    ctx->launches++;
    rc = bt_cuda_check(ctx, cudaGetLastError(), "fidelity launch");
  }
  int hinfo[2] = {0, 0};
  double h = 0;
  if (!rc)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost, ctx->stream), "info");
  if (!rc) rc = bt_cuda_check(ctx, cudaMemcpyAsync(&h, res, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "res");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "fidelity sync");
  L->bl_destroy(hb);
  L->dn_destroy(hs);
  if (rc) return rc;
  if (hinfo[0] || hinfo[1]) return bt_fail(ctx, BT_ERR_DEVICE, "the Hermitian eigensolver did not converge");
  *out = h;
  return BT_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ rho accumulation
// rho[i + j d] += w * sum_m psi_m[i] conj(psi_m[j]); one thread per entry, members
// summed in order (deterministic), FP64
template <typename R, typename RR>
__global__ void k_rho_acc(typename CT<RR>::T* __restrict__ rho, const typename CT<R>::T* __restrict__ psi, int n,
                          int64_t nmem, double w) {
  const int64_t d = 1LL << n, len = d * d;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e & (d - 1), j = e >> n;
    double re = 0, im = 0;
    for (int64_t m = 0; m < nmem; ++m) {
      const typename CT<R>::T a = psi[(m << n) + i], b = psi[(m << n) + j];
      re += (double)a.x * b.x + (double)a.y * b.y;
      im += (double)a.y * b.x - (double)a.x * b.y;
    }
    typename CT<RR>::T v = rho[e];
    v.x = (RR)((double)v.x + w * re);
    v.y = (RR)((double)v.y + w * im);
    rho[e] = v;
  }
}

// uniform [0, 1) real and imaginary parts from Philox, then scaled to unit norm
template <typename R>
__global__ void k_random_fill(typename CT<R>::T* __restrict__ p, int64_t len, uint64_t key, uint64_t stream) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    typename CT<R>::T v;
    v.x = (R)bt_uniform(key, stream, 2 * (uint64_t)i);
    v.y = (R)bt_uniform(key, stream, 2 * (uint64_t)i + 1);
    p[i] = v;
  }
}

template <typename R>
__global__ void k_scale_by(typename CT<R>::T* __restrict__ p, int64_t len, const double* __restrict__ norm2) {
  const double s = 1.0 / sqrt(*norm2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    typename CT<R>::T v = p[i];
    v.x = (R)((double)v.x * s);
    v.y = (R)((double)v.y * s);
    p[i] = v;
  }
}

extern "C" {

int bt_rho_accumulate(bt_state* rho, int64_t rmember, const bt_state* psi_, double weight) {
  if (!rho || !psi_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* psi = const_cast<bt_state*>(psi_);
  bt_ctx* ctx = rho->ctx;
  if (rho->repr != BT_REPR_DM || psi->repr != BT_REPR_SV || rho->n != psi->n)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "rho must be a density matrix and psi a state vector of the same size");
  if (rmember < 0 || rmember >= rho->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  if (rho->n > 14) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "rho accumulation supports n <= 14");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  if (psi->ctx != ctx) cudaStreamSynchronize(psi->ctx->stream);
  const int64_t len = rho->member_elems;
  const int grid = bt_grid(ctx, len, BT_THREADS, 8);
  const int64_t off = rmember * len;
  const bool f = psi->prec == BT_PREC_C64, rf = rho->prec == BT_PREC_C64;
  if (f && rf) k_rho_acc<float, float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)rho->d + off, (const float2*)psi->d, psi->n, psi->batch, weight);
  else if (f) k_rho_acc<float, double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)rho->d + off, (const float2*)psi->d, psi->n, psi->batch, weight);
  else if (rf) k_rho_acc<double, float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)rho->d + off, (const double2*)psi->d, psi->n, psi->batch, weight);
  else k_rho_acc<double, double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)rho->d + off, (const double2*)psi->d, psi->n, psi->batch, weight);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "rho accumulate launch");
}

int bt_state_clear(bt_state* s, int64_t member) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  if (member < -1 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  const size_t per = (size_t)s->member_elems * elem_bytes(s->prec);
  char* base = (char*)s->d + (member < 0 ? 0 : (size_t)member * per);
  return bt_cuda_check(ctx, cudaMemsetAsync(base, 0, member < 0 ? per * s->batch : per, ctx->stream), "clear");
}

int bt_state_random(bt_state* s, int64_t member, uint64_t seed) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  if (s->repr != BT_REPR_SV) return bt_fail(ctx, BT_ERR_BAD_ARG, "random_state makes state vectors");
  if (member < -1 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  int rc = bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (rc) return rc;
  const int64_t lo = member < 0 ? 0 : member, hi = member < 0 ? s->batch : member + 1;
  double* nrm = nullptr;
  for (int64_t m = lo; m < hi && !rc; ++m) {
    const int64_t len = s->member_elems;
    const int grid = bt_grid(ctx, len);
    // one Philox stream per (seed, member): members differ, and a member's state does
    // not depend on how many members the call fills
    const uint64_t stream = 0x524e440000000000ULL ^ (seed * 0x9E3779B97F4A7C15ULL) ^ (uint64_t)m;
    if (s->prec == BT_PREC_C64) k_random_fill<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d + m * len, len, ctx->seed, stream);
    else k_random_fill<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d + m * len, len, ctx->seed, stream);
    ctx->launches++;
    if ((rc = bt_cuda_check(ctx, cudaGetLastError(), "random fill launch"))) break;
    if (!nrm) {
      void* q = bt_scratch(ctx, 256, &rc);
      if (rc) break;
      nrm = (double*)q;
    }
    if ((rc = bt_launch_norm2(s, m, 1, nrm))) break;
    if (s->prec == BT_PREC_C64) k_scale_by<float><<<grid, BT_THREADS, 0, ctx->stream>>>((float2*)s->d + m * len, len, nrm);
    else k_scale_by<double><<<grid, BT_THREADS, 0, ctx->stream>>>((double2*)s->d + m * len, len, nrm);
    ctx->launches++;
    rc = bt_cuda_check(ctx, cudaGetLastError(), "scale launch");
  }
  return rc;
}

}  // extern "C"
