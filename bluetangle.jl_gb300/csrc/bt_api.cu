// C ABI of the engine (include/btgpu.h): context and state management,
// argument validation with the reference's error behaviour, and the host side
// of each hot-path entry point.  Device work is issued on the context's stream;
// calls that return values to the host synchronise that stream before returning.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "bt_internal.cuh"

static thread_local std::string tl_err;

int bt_fail(bt_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  tl_err = msg;
  return code;
}

int bt_cuda_check(bt_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return BT_OK;
  int code = e == cudaErrorMemoryAllocation ? BT_ERR_OOM : BT_ERR_DEVICE;
  return bt_fail(ctx, code, std::string(what) + ": " + cudaGetErrorString(e));
}

void* bt_scratch(bt_ctx* ctx, size_t bytes, int* rc) {
  *rc = BT_OK;
  if (ctx->scratch_bytes < bytes) {
    if (ctx->scratch) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ctx->scratch);
      ctx->scratch = nullptr;
      ctx->scratch_bytes = 0;
    }
    size_t nb = bytes < (1u << 20) ? (1u << 20) : bytes;
    if (cudaMalloc(&ctx->scratch, nb) != cudaSuccess) {
      *rc = bt_fail(ctx, BT_ERR_OOM, "scratch allocation failed");
      return nullptr;
    }
    ctx->scratch_bytes = nb;
  }
  return ctx->scratch;
}

// carves 256-byte aligned regions out of one scratch allocation
struct Carve {
  size_t total = 0;
  std::vector<size_t> offs;
  int add(size_t bytes) {
    offs.push_back(total);
    total += (bytes + 255) & ~(size_t)255;
    return (int)offs.size() - 1;
  }
  char* base = nullptr;
  int commit(bt_ctx* ctx) {
    int rc;
    base = (char*)bt_scratch(ctx, total ? total : 256, &rc);
    return rc;
  }
  template <typename T> T* at(int i) { return (T*)(base + offs[i]); }
};

static int set_dev(bt_ctx* ctx) {
  return bt_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
}

static int sync_and_status(bt_ctx* ctx, const char* what) {
  int rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), what);
  if (rc) return rc;
  int st = 0;
  rc = bt_cuda_check(ctx, cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
  if (rc) return rc;
  if (st) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (st == 1) return bt_fail(ctx, BT_ERR_BAD_ARG, "measurement outcome with zero probability");
    if (st == 2) return bt_fail(ctx, BT_ERR_NO_BRANCH, "no Kraus branch satisfies u <= cumsum(p)");
    if (st == 16) return bt_fail(ctx, BT_ERR_TIMEOUT, "tensor-core pass: an MMA completion wait ran out");
    return bt_fail(ctx, BT_ERR_BAD_ARG, "Kraus branch with zero norm");
  }
  return BT_OK;
}

// column-major complex (Julia) -> row-major interleaved
static void to_rowmajor(const double* cm, int d, double* rm) {
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      rm[2 * (r * d + c)] = cm[2 * (r + c * d)];
      rm[2 * (r * d + c) + 1] = cm[2 * (r + c * d) + 1];
    }
}

static int members(const bt_state* s, int64_t member, int64_t* lo, int64_t* n) {
  if (member == -1) {
    *lo = 0;
    *n = s->batch;
    return BT_OK;
  }
  if (member < 0 || member >= s->batch) return bt_fail(s->ctx, BT_ERR_BAD_ARG, "member index out of range");
  *lo = member;
  *n = 1;
  return BT_OK;
}

extern "C" {

int bt_abi_version(void) { return BT_ABI_VERSION; }

const char* bt_status_string(int status) {
  switch (status) {
    case BT_OK: return "ok";
    case BT_ERR_BAD_ARG: return "bad argument";
    case BT_ERR_NOT_CPTP: return "not valid kraus operators: not CPTP!";
    case BT_ERR_OOM: return "out of device memory";
    case BT_ERR_DEVICE: return "CUDA device error";
    case BT_ERR_TIMEOUT: return "timeout";
    case BT_ERR_UNSUPPORTED: return "unsupported operation";
    case BT_ERR_NO_BRANCH: return "no Kraus branch selected";
  }
  return "unknown status";
}

int bt_ctx_create(int device, uint64_t seed, bt_ctx** out) {
  if (!out) return bt_fail(nullptr, BT_ERR_BAD_ARG, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return bt_fail(nullptr, BT_ERR_DEVICE, "no CUDA device available");
  if (device < 0 || device >= count) return bt_fail(nullptr, BT_ERR_BAD_ARG, "device index out of range");
  bt_ctx* ctx = new bt_ctx();
  ctx->device = device;
  ctx->seed = seed;
  int rc = set_dev(ctx);
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream create");
  if (!rc) rc = bt_cuda_check(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device), "attr");
  if (!rc) rc = bt_cuda_check(ctx, cudaMalloc(&ctx->d_status, sizeof(int)), "status alloc");
  if (!rc) rc = bt_cuda_check(ctx, cudaMemset(ctx->d_status, 0, sizeof(int)), "status clear");
  if (rc) {
    tl_err = ctx->err;
    bt_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return BT_OK;
}

int bt_ctx_destroy(bt_ctx* ctx) {
  if (!ctx) return BT_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->work) cudaFree(ctx->work);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BT_OK;
}

const char* bt_last_error(const bt_ctx* ctx) { return ctx ? ctx->err.c_str() : tl_err.c_str(); }

int bt_ctx_synchronize(bt_ctx* ctx) {
  if (!ctx) return bt_fail(nullptr, BT_ERR_BAD_ARG, "ctx is NULL");
  int rc = set_dev(ctx);
  if (rc) return rc;
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

int bt_ctx_launch_count(const bt_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL argument");
  *out = ctx->launches;
  return BT_OK;
}

int bt_ctx_stream(const bt_ctx* ctx, void** out) {
  if (!ctx || !out) return bt_fail(nullptr, BT_ERR_BAD_ARG, "NULL argument");
  *out = (void*)ctx->stream;
  return BT_OK;
}

// ------------------------------------------------------------------ state
int bt_state_alloc(bt_ctx* ctx, int n, int repr, int prec, int batch, bt_state** out) {
  if (!ctx || !out) return bt_fail(ctx, BT_ERR_BAD_ARG, "NULL argument");
  *out = nullptr;
  if (repr != BT_REPR_SV && repr != BT_REPR_DM) return bt_fail(ctx, BT_ERR_BAD_ARG, "repr must be SV or DM");
  if (prec != BT_PREC_C128 && prec != BT_PREC_C64) return bt_fail(ctx, BT_ERR_BAD_ARG, "prec must be C128 or C64");
  if (n < 1 || (repr == BT_REPR_SV && n > 34) || (repr == BT_REPR_DM && n > 17))
    return bt_fail(ctx, BT_ERR_BAD_ARG, "qubit count out of range");
  if (batch < 1) return bt_fail(ctx, BT_ERR_BAD_ARG, "batch must be >= 1");
  int rc = set_dev(ctx);
  if (rc) return rc;
  bt_state* s = new bt_state();
  s->ctx = ctx;
  s->n = n;
  s->repr = repr;
  s->prec = prec;
  s->batch = batch;
  s->nbits = repr == BT_REPR_DM ? 2 * n : n;
  s->member_elems = 1LL << s->nbits;
  size_t bytes = (size_t)s->member_elems * elem_bytes(prec) * (size_t)batch;
  cudaError_t e = cudaMalloc(&s->d, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete s;
    return bt_fail(ctx, BT_ERR_OOM, "state allocation of " + std::to_string(bytes) + " bytes failed");
  }
  rc = bt_launch_set_basis(s, 0, batch, 0);
  if (rc) {
    cudaFree(s->d);
    delete s;
    return rc;
  }
  *out = s;
  return BT_OK;
}

int bt_state_free(bt_state* s) {
  if (!s) return BT_OK;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  cudaFree(s->d);
  delete s;
  return BT_OK;
}

int bt_state_info(const bt_state* s, int* n, int* repr, int* prec, int* batch) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  if (n) *n = s->n;
  if (repr) *repr = s->repr;
  if (prec) *prec = s->prec;
  if (batch) *batch = s->batch;
  return BT_OK;
}

void* bt_state_device_ptr(bt_state* s) { return s ? s->d : nullptr; }

int bt_state_set_zero(bt_state* s, int64_t member) { return bt_state_set_basis(s, member, 0); }

int bt_state_set_basis(bt_state* s, int64_t member, uint64_t index) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  int64_t lo, nm;
  int rc = members(s, member, &lo, &nm);
  if (rc) return rc;
  if (index >> s->n) return bt_fail(ctx, BT_ERR_BAD_ARG, "basis index out of range");
  if ((rc = set_dev(ctx))) return rc;
  uint64_t e = s->repr == BT_REPR_DM ? index + (index << s->n) : index;
  return bt_launch_set_basis(s, lo, nm, e);
}

int bt_state_copy(bt_state* dst, int64_t dst_member, const bt_state* src, int64_t src_member) {
  if (!dst || !src) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = dst->ctx;
  if (dst->n != src->n || dst->repr != src->repr || dst->prec != src->prec)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "states differ in n, repr or prec");
  if (src_member < 0 || src_member >= src->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "source member out of range");
  int64_t lo, nm;
  int rc = members(dst, dst_member, &lo, &nm);
  if (rc) return rc;
  if ((rc = set_dev(ctx))) return rc;
  size_t mb = (size_t)dst->member_elems * elem_bytes(dst->prec);
  const char* sp = (const char*)src->d + src_member * mb;
  if (src->ctx != ctx) cudaStreamSynchronize(src->ctx->stream);
  for (int64_t m = lo; m < lo + nm; ++m) {
    char* dp = (char*)dst->d + m * mb;
    if (dp == sp) continue;
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(dp, sp, mb, cudaMemcpyDeviceToDevice, ctx->stream), "state copy");
    if (rc) return rc;
  }
  return BT_OK;
}

static int xfer_check(const bt_state* s, int64_t member, int64_t offset, int64_t len, const void* host) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  if (!host && len > 0) return bt_fail(s->ctx, BT_ERR_BAD_ARG, "host buffer is NULL");
  if (member < 0 || member >= s->batch) return bt_fail(s->ctx, BT_ERR_BAD_ARG, "member out of range");
  if (offset < 0 || len < 0 || offset + len > s->member_elems) return bt_fail(s->ctx, BT_ERR_BAD_ARG, "range out of bounds");
  return BT_OK;
}

int bt_state_upload(bt_state* s, int64_t member, int64_t offset, int64_t len, const double* host) {
  int rc = xfer_check(s, member, offset, len, host);
  if (rc) return rc;
  bt_ctx* ctx = s->ctx;
  if ((rc = set_dev(ctx))) return rc;
  if (s->prec == BT_PREC_C128) {
    double2* dst = (double2*)s->d + member * s->member_elems + offset;
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(dst, host, (size_t)len * 16, cudaMemcpyHostToDevice, ctx->stream), "upload");
    if (rc) return rc;
  } else {
    const int64_t chunk = 1LL << 22;
    double* stage = nullptr;
    rc = bt_work(ctx, (size_t)std::min(len, chunk) * 16, &stage);
    if (rc) return rc;
    for (int64_t o = 0; o < len && !rc; o += chunk) {
      int64_t l = std::min(chunk, len - o);
      rc = bt_cuda_check(ctx, cudaMemcpyAsync(stage, host + 2 * o, (size_t)l * 16, cudaMemcpyHostToDevice, ctx->stream), "upload");
      if (!rc) rc = bt_launch_convert_in(s, member, offset + o, l, stage);
    }
    if (rc) return rc;
  }
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "upload sync");
}

int bt_state_download(const bt_state* s_, int64_t member, int64_t offset, int64_t len, double* host) {
  int rc = xfer_check(s_, member, offset, len, host);
  if (rc) return rc;
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if ((rc = set_dev(ctx))) return rc;
  if (s->prec == BT_PREC_C128) {
    const double2* src = (const double2*)s->d + member * s->member_elems + offset;
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(host, src, (size_t)len * 16, cudaMemcpyDeviceToHost, ctx->stream), "download");
    if (rc) return rc;
  } else {
    const int64_t chunk = 1LL << 22;
    double* stage = nullptr;
    rc = bt_work(ctx, (size_t)std::min(len, chunk) * 16, &stage);
    if (rc) return rc;
    for (int64_t o = 0; o < len && !rc; o += chunk) {
      int64_t l = std::min(chunk, len - o);
      rc = bt_launch_convert_out(s, member, offset + o, l, stage);
      if (!rc) rc = bt_cuda_check(ctx, cudaMemcpyAsync(host + 2 * o, stage, (size_t)l * 16, cudaMemcpyDeviceToHost, ctx->stream), "download");
      if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "download sync");
    }
    if (rc) return rc;
  }
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "download sync");
}

// ------------------------------------------------------------------ gates
static int check_qubits(bt_ctx* ctx, int n, int k, const int32_t* qubits, int nctrl, const int32_t* ctrls) {
  if (k < 1 || !qubits) return bt_fail(ctx, BT_ERR_BAD_ARG, "need at least one target qubit");
  if (nctrl < 0 || (nctrl > 0 && !ctrls)) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad control list");
  uint64_t seen = 0;
  for (int i = 0; i < k + nctrl; ++i) {
    int q = i < k ? qubits[i] : ctrls[i - k];
    if (q < 1 || q > n) return bt_fail(ctx, BT_ERR_BAD_ARG, "N must be larger than qubits");
    if (seen & (1ULL << q)) return bt_fail(ctx, BT_ERR_BAD_ARG, "qubits and controls must differ");
    seen |= 1ULL << q;
  }
  return BT_OK;
}

int bt_apply_matrix(bt_state* s, int k, const int32_t* qubits, const double* mat, int nctrl, const int32_t* ctrls,
                    int64_t member) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  if (!mat) return bt_fail(ctx, BT_ERR_BAD_ARG, "matrix is NULL");
  int rc = check_qubits(ctx, s->n, k, qubits, nctrl, ctrls);
  if (rc) return rc;
  if (k > BT_MAX_K) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "dense gates act on at most 5 qubits");
  int64_t lo, nm;
  if ((rc = members(s, member, &lo, &nm))) return rc;
  if ((rc = set_dev(ctx))) return rc;
  const int d = 1 << k;
  std::vector<double> rm(2 * d * d);
  to_rowmajor(mat, d, rm.data());
  const int n = s->n;
  if (s->repr == BT_REPR_SV) {
    int bits[BT_MAX_K];
    uint64_t cmask = 0;
    for (int i = 0; i < k; ++i) bits[i] = n - qubits[i];
    for (int i = 0; i < nctrl; ++i) cmask |= 1ULL << (n - ctrls[i]);
    return bt_launch_gate(s, k, bits, rm.data(), cmask, lo, nm, nullptr, 0);
  }
  // density matrix: e_op * rho * e_op' acts with U on the row bits (n - q) and
  // conj(U) on the column bits (2n - q) of vec(rho)
  if (nctrl == 0 && 2 * k <= BT_MAX_K) {
    const int dd = d * d;
    std::vector<double> sup(2 * dd * dd);
    for (int ir = 0; ir < d; ++ir)
      for (int ic = 0; ic < d; ++ic)
        for (int jr = 0; jr < d; ++jr)
          for (int jc = 0; jc < d; ++jc) {
            double ar = rm[2 * (ir * d + jr)], ai = rm[2 * (ir * d + jr) + 1];
            double br = rm[2 * (ic * d + jc)], bi = -rm[2 * (ic * d + jc) + 1];
            int r = ir * d + ic, c = jr * d + jc;
            sup[2 * (r * dd + c)] = ar * br - ai * bi;
            sup[2 * (r * dd + c) + 1] = ar * bi + ai * br;
          }
    int bits[2 * BT_MAX_K];
    for (int i = 0; i < k; ++i) {
      bits[i] = n - qubits[i];
      bits[k + i] = 2 * n - qubits[i];
    }
    return bt_launch_gate(s, 2 * k, bits, sup.data(), 0, lo, nm, nullptr, 0);
  }
  int bits[BT_MAX_K];
  uint64_t cmask = 0;
  for (int i = 0; i < k; ++i) bits[i] = n - qubits[i];
  for (int i = 0; i < nctrl; ++i) cmask |= 1ULL << (n - ctrls[i]);
  rc = bt_launch_gate(s, k, bits, rm.data(), cmask, lo, nm, nullptr, 0);
  if (rc) return rc;
  std::vector<double> cj(rm);
  for (int i = 0; i < d * d; ++i) cj[2 * i + 1] = -cj[2 * i + 1];
  cmask = 0;
  for (int i = 0; i < k; ++i) bits[i] = 2 * n - qubits[i];
  for (int i = 0; i < nctrl; ++i) cmask |= 1ULL << (2 * n - ctrls[i]);
  return bt_launch_gate(s, k, bits, cj.data(), cmask, lo, nm, nullptr, 0);
}

// sum_k K^dagger K == I within the tolerance of Julia's isapprox on the matrix
static bool trace_preserving(int d, int nk, const double* kraus_cm) {
  double diff2 = 0;
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      double sr = 0, si = 0;
      for (int i = 0; i < nk; ++i) {
        const double* K = kraus_cm + (size_t)i * 2 * d * d;
        for (int a = 0; a < d; ++a) {
          // conj(K[a, r]) * K[a, c]
          double xr = K[2 * (a + r * d)], xi = -K[2 * (a + r * d) + 1];
          double yr = K[2 * (a + c * d)], yi = K[2 * (a + c * d) + 1];
          sr += xr * yr - xi * yi;
          si += xr * yi + xi * yr;
        }
      }
      sr -= (r == c) ? 1.0 : 0.0;
      diff2 += sr * sr + si * si;
    }
  return sqrt(diff2) <= 1.4901161193847656e-08 * sqrt((double)d);
}

// every K_i^dagger K_i is a multiple of the identity (K_i = c_i U_i)
static bool unitary_mixture(int d, int nk, const double* kraus_cm) {
  for (int i = 0; i < nk; ++i) {
    const double* K = kraus_cm + (size_t)i * 2 * d * d;
    double diag0 = -1;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        double sr = 0, si = 0;
        for (int a = 0; a < d; ++a) {
          double xr = K[2 * (a + r * d)], xi = -K[2 * (a + r * d) + 1];
          double yr = K[2 * (a + c * d)], yi = K[2 * (a + c * d) + 1];
          sr += xr * yr - xi * yi;
          si += xr * yi + xi * yr;
        }
        if (r == c) {
          if (diag0 < 0) diag0 = sr;
          if (fabs(sr - diag0) > 1e-12 || fabs(si) > 1e-12) return false;
        } else if (fabs(sr) > 1e-12 || fabs(si) > 1e-12) {
          return false;
        }
      }
  }
  return true;
}

int bt_apply_matrix_members(bt_state* s, int k, const int32_t* qubits, const double* mats, int nctrl,
                            const int32_t* ctrls) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  if (!mats) return bt_fail(ctx, BT_ERR_BAD_ARG, "matrices are NULL");
  if (s->repr != BT_REPR_SV) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "per-member matrices need state vectors");
  int rc = check_qubits(ctx, s->n, k, qubits, nctrl, ctrls);
  if (rc) return rc;
  if (k > BT_MAX_K) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "dense gates act on at most 5 qubits");
  if ((rc = set_dev(ctx))) return rc;
  const int d = 1 << k;
  const int64_t B = s->batch;
  const size_t per = 2 * (size_t)d * d;
  const bool f = s->prec == BT_PREC_C64;
  Carve cv;
  int iM = cv.add((size_t)B * per * (f ? 4 : 8));
  if ((rc = cv.commit(ctx))) return rc;
  std::vector<float> hf(f ? B * per : 0);
  std::vector<double> hd(f ? 0 : B * per);
  for (int64_t m = 0; m < B; ++m) {
    const double* cm = mats + (size_t)m * per;
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c)
        for (int z = 0; z < 2; ++z) {
          const double v = cm[2 * (r + c * d) + z];
          if (f) hf[m * per + 2 * (r * d + c) + z] = (float)v;
          else hd[m * per + 2 * (r * d + c) + z] = v;
        }
  }
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<void>(iM), f ? (const void*)hf.data() : (const void*)hd.data(),
                                          (size_t)B * per * (f ? 4 : 8), cudaMemcpyHostToDevice, ctx->stream),
                     "matrix upload");
  if (rc) return rc;
  int bits[BT_MAX_K];
  uint64_t cmask = 0;
  for (int i = 0; i < k; ++i) bits[i] = s->n - qubits[i];
  for (int i = 0; i < nctrl; ++i) cmask |= 1ULL << (s->n - ctrls[i]);
  // a copy from pageable memory has left the host vectors once cudaMemcpyAsync returns
  return bt_launch_gate(s, k, bits, nullptr, cmask, 0, B, cv.at<void>(iM), (int64_t)per);
}

int bt_apply_kraus(bt_state* s, int k, const int32_t* qubits, int nk, const double* kraus, int mode,
                   const double* uniforms, const int32_t* forced, int32_t* branch_out, double* probs_out) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  int rc = check_qubits(ctx, s->n, k, qubits, 0, nullptr);
  if (rc) return rc;
  if (k > 3) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "Noise models are available only for up to 3 qubits!");
  if (nk < 1 || !kraus) return bt_fail(ctx, BT_ERR_BAD_ARG, "need at least one Kraus operator");
  const int d = 1 << k;
  if (!trace_preserving(d, nk, kraus)) return bt_fail(ctx, BT_ERR_NOT_CPTP, "not valid kraus operators: not CPTP!");
  const int flags = mode & ~0xff;
  mode &= 0xff;
  if ((rc = set_dev(ctx))) return rc;
  const int n = s->n;
  std::vector<double> rm((size_t)nk * 2 * d * d);
  for (int i = 0; i < nk; ++i) to_rowmajor(kraus + (size_t)i * 2 * d * d, d, rm.data() + (size_t)i * 2 * d * d);

  if (mode == BT_KRAUS_SUM) {
    if (s->repr != BT_REPR_DM) return bt_fail(ctx, BT_ERR_BAD_ARG, "a Kraus sum needs a density matrix");
    if (2 * k > BT_MAX_K) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "density-matrix channels act on at most 2 qubits");
    // superoperator sum_i K_i (x) conj(K_i) on (row bits, column bits): one pass
    const int dd = d * d;
    std::vector<double> sup(2 * (size_t)dd * dd, 0.0);
    for (int i = 0; i < nk; ++i) {
      const double* K = rm.data() + (size_t)i * 2 * d * d;
      for (int ir = 0; ir < d; ++ir)
        for (int ic = 0; ic < d; ++ic)
          for (int jr = 0; jr < d; ++jr)
            for (int jc = 0; jc < d; ++jc) {
              double ar = K[2 * (ir * d + jr)], ai = K[2 * (ir * d + jr) + 1];
              double br = K[2 * (ic * d + jc)], bi = -K[2 * (ic * d + jc) + 1];
              int r = ir * d + ic, c = jr * d + jc;
              sup[2 * (r * dd + c)] += ar * br - ai * bi;
              sup[2 * (r * dd + c) + 1] += ar * bi + ai * br;
            }
    }
    int bits[2 * 2];
    for (int i = 0; i < k; ++i) {
      bits[i] = n - qubits[i];
      bits[k + i] = 2 * n - qubits[i];
    }
    return bt_launch_gate(s, 2 * k, bits, sup.data(), 0, 0, s->batch, nullptr, 0);
  }
  if (mode != BT_KRAUS_TRAJ) return bt_fail(ctx, BT_ERR_BAD_ARG, "unknown Kraus mode");
  if (s->repr != BT_REPR_SV) return bt_fail(ctx, BT_ERR_BAD_ARG, "trajectory branches need a state vector");
  const int64_t B = s->batch;
  Carve cv;
  int iK = cv.add(rm.size() * sizeof(double));
  int iU = uniforms ? cv.add(B * sizeof(double)) : -1;
  int iF = forced ? cv.add(B * sizeof(int)) : -1;
  int iR = cv.add(B * 2 * d * d * sizeof(double));
  int iB = cv.add(B * sizeof(int));
  int iP = cv.add(B * nk * sizeof(double));
  int iM = cv.add(B * 2 * d * d * elem_bytes(s->prec) / 2);
  if ((rc = cv.commit(ctx))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iK), rm.data(), rm.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "kraus upload");
  if (!rc && uniforms) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iU), uniforms, B * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "uniform upload");
  if (!rc && forced) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<int>(iF), forced, B * sizeof(int), cudaMemcpyHostToDevice, ctx->stream), "forced upload");
  if (rc) return rc;
  int bits[3];
  for (int i = 0; i < k; ++i) bits[i] = n - qubits[i];
  const bool umix = (flags & BT_KRAUS_UNITARY_MIX) != 0;
  if (umix && !unitary_mixture(d, nk, kraus))
    return bt_fail(ctx, BT_ERR_BAD_ARG, "BT_KRAUS_UNITARY_MIX needs Kraus operators that are multiples of unitaries");
  if (!umix && (rc = bt_launch_rdm(s, k, bits, 0, B, cv.at<double>(iR)))) return rc;
  bt_kraus_desc kd;
  kd.k = k;
  kd.nk = nk;
  kd.ref_perm = (flags & BT_KRAUS_REF_ORDER) && k == 2 && qubits[0] > qubits[1];
  uint64_t stream = 0x4b52000000000000ULL ^ ctx->rng_calls++;
  rc = bt_launch_decide_kraus(s, kd, B, umix ? nullptr : cv.at<double>(iR), cv.at<double>(iK),
                              uniforms ? cv.at<double>(iU) : nullptr,
                              forced ? cv.at<int>(iF) : nullptr, stream, cv.at<int>(iB), cv.at<double>(iP),
                              cv.at<void>(iM));
  if (rc) return rc;
  if ((rc = bt_launch_gate(s, k, bits, nullptr, 0, 0, B, cv.at<void>(iM), 2 * d * d))) return rc;
  if (branch_out)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(branch_out, cv.at<int>(iB), B * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "branch download");
  if (!rc && probs_out)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(probs_out, cv.at<double>(iP), B * nk * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "probs download");
  if (rc) return rc;
  return sync_and_status(ctx, "kraus");
}

// ------------------------------------------------------------------ measurement
int bt_measure_z(bt_state* s, int qubit, const double* uniforms, const int32_t* forced, int32_t* outcome, double* p0) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  int rc = check_qubits(ctx, s->n, 1, &qubit, 0, nullptr);
  if (rc) return rc;
  if ((rc = set_dev(ctx))) return rc;
  const int64_t B = s->batch;
  const int b = s->n - qubit;
  if (s->repr == BT_REPR_DM) {
    Carve cv;
    int iS = cv.add(B * 36 * sizeof(double));
    if ((rc = cv.commit(ctx))) return rc;
    if (p0) {
      if ((rc = bt_launch_bitsums(s, 0, B, cv.at<double>(iS)))) return rc;
    }
    if ((rc = bt_launch_dephase(s, b, 0, B))) return rc;
    if (p0) {
      std::vector<double> h(B * 36);
      rc = bt_cuda_check(ctx, cudaMemcpyAsync(h.data(), cv.at<double>(iS), h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "p0 download");
      if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "measure sync");
      if (rc) return rc;
      for (int64_t m = 0; m < B; ++m) p0[m] = h[m * 36] - h[m * 36 + 1 + b];
    }
    return BT_OK;
  }
  Carve cv;
  int iU = uniforms ? cv.add(B * sizeof(double)) : -1;
  int iF = forced ? cv.add(B * sizeof(int)) : -1;
  int iR = cv.add(B * 8 * sizeof(double));
  int iO = cv.add(B * sizeof(int));
  int iS = cv.add(B * sizeof(double));
  int iP = cv.add(B * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  if (uniforms) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iU), uniforms, B * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "uniform upload");
  if (!rc && forced) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<int>(iF), forced, B * sizeof(int), cudaMemcpyHostToDevice, ctx->stream), "forced upload");
  if (rc) return rc;
  if ((rc = bt_launch_rdm(s, 1, &b, 0, B, cv.at<double>(iR)))) return rc;
  uint64_t stream = 0x4d5a000000000000ULL ^ ctx->rng_calls++;
  rc = bt_launch_decide_measure(ctx, B, cv.at<double>(iR), uniforms ? cv.at<double>(iU) : nullptr,
                                forced ? cv.at<int>(iF) : nullptr, stream, cv.at<int>(iO), cv.at<double>(iS),
                                cv.at<double>(iP));
  if (rc) return rc;
  if ((rc = bt_launch_collapse(s, b, cv.at<int>(iO), cv.at<double>(iS), 0, B))) return rc;
  if (outcome)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(outcome, cv.at<int>(iO), B * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "outcome download");
  if (!rc && p0)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(p0, cv.at<double>(iP), B * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "p0 download");
  if (rc) return rc;
  return sync_and_status(ctx, "measure");
}

int bt_measure_z2(bt_state* s, int q1, int q2, const double* uniforms, const int32_t* forced, int32_t* outcome,
                  double* probs) {
  if (!s) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_ctx* ctx = s->ctx;
  const int32_t qs[2] = {q1, q2};
  int rc = check_qubits(ctx, s->n, 2, qs, 0, nullptr);
  if (rc) return rc;
  if (s->repr != BT_REPR_SV)
    return bt_fail(ctx, BT_ERR_UNSUPPORTED, "the two-qubit Born measurement acts on state vectors");
  if ((rc = set_dev(ctx))) return rc;
  const int64_t B = s->batch;
  const int bits[2] = {s->n - q1, s->n - q2};
  Carve cv;
  int iU = uniforms ? cv.add(B * sizeof(double)) : -1;
  int iF = forced ? cv.add(B * sizeof(int)) : -1;
  int iR = cv.add(B * 32 * sizeof(double));
  int iO = cv.add(B * sizeof(int));
  int iS = cv.add(B * sizeof(double));
  int iP = cv.add(B * 4 * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  if (uniforms) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iU), uniforms, B * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "uniform upload");
  if (!rc && forced) rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<int>(iF), forced, B * sizeof(int), cudaMemcpyHostToDevice, ctx->stream), "forced upload");
  if (rc) return rc;
  if ((rc = bt_launch_rdm(s, 2, bits, 0, B, cv.at<double>(iR)))) return rc;
  uint64_t stream = 0x4d5a320000000000ULL ^ ctx->rng_calls++;
  rc = bt_launch_decide_measure2(ctx, B, cv.at<double>(iR), uniforms ? cv.at<double>(iU) : nullptr,
                                 forced ? cv.at<int>(iF) : nullptr, stream, cv.at<int>(iO), cv.at<double>(iS),
                                 cv.at<double>(iP));
  if (rc) return rc;
  if ((rc = bt_launch_collapse2(s, bits[0], bits[1], cv.at<int>(iO), cv.at<double>(iS), 0, B))) return rc;
  if (outcome)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(outcome, cv.at<int>(iO), B * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "outcome download");
  if (!rc && probs)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(probs, cv.at<double>(iP), B * 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "probs download");
  if (rc) return rc;
  return sync_and_status(ctx, "measure2");
}

int bt_reduced_dm(const bt_state* s_, int k, const int32_t* qubits, int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  if (s->repr != BT_REPR_SV) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "reduced matrices are computed from state vectors");
  int rc = check_qubits(ctx, s->n, k, qubits, 0, nullptr);
  if (rc) return rc;
  if (k > 3) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "at most 3 kept qubits");
  if (member < 0 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  if ((rc = set_dev(ctx))) return rc;
  const int d = 1 << k;
  Carve cv;
  int iR = cv.add(2 * d * d * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  int bits[3];
  for (int i = 0; i < k; ++i) bits[i] = s->n - qubits[i];
  if ((rc = bt_launch_rdm(s, k, bits, member, 1, cv.at<double>(iR)))) return rc;
  std::vector<double> h(2 * d * d);
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(h.data(), cv.at<double>(iR), h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "rdm download");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "rdm sync");
  if (rc) return rc;
  for (int a = 0; a < d; ++a)
    for (int b = 0; b < d; ++b) {
      out[2 * (a + b * d)] = h[2 * (a * d + b)];
      out[2 * (a + b * d) + 1] = h[2 * (a * d + b) + 1];
    }
  return BT_OK;
}

// ------------------------------------------------------------------ sampling
int bt_sample(const bt_state* s_, int64_t member, int64_t shots, const double* uniforms, uint64_t seed, int64_t* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (shots < 0 || (shots > 0 && !out)) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad shots/out");
  if (member < 0 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  if (shots == 0) return BT_OK;
  int rc = set_dev(ctx);
  if (rc) return rc;
  Carve cv;
  int iU = uniforms ? cv.add(shots * sizeof(double)) : -1;
  int iO = cv.add(shots * sizeof(int64_t));
  if ((rc = cv.commit(ctx))) return rc;
  if (uniforms)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iU), uniforms, shots * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "uniform upload");
  if (rc) return rc;
  uint64_t stream = seed ^ 0x53414d5000000000ULL;
  if ((rc = bt_launch_sample(s, member, shots, uniforms ? cv.at<double>(iU) : nullptr, stream, cv.at<int64_t>(iO)))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(out, cv.at<int64_t>(iO), shots * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream), "shots download");
  if (rc) return rc;
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sample sync");
}

int bt_sample_members(const bt_state* s_, const double* uniforms, uint64_t seed, int64_t* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  int rc = set_dev(ctx);
  if (rc) return rc;
  const int64_t B = s->batch;
  Carve cv;
  int iU = uniforms ? cv.add(B * sizeof(double)) : -1;
  int iO = cv.add(B * sizeof(int64_t));
  if ((rc = cv.commit(ctx))) return rc;
  if (uniforms)
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iU), uniforms, B * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "uniform upload");
  if (rc) return rc;
  uint64_t stream = seed ^ 0x53414d4500000000ULL;
  if ((rc = bt_launch_sample_each(s, uniforms ? cv.at<double>(iU) : nullptr, stream, cv.at<int64_t>(iO)))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(out, cv.at<int64_t>(iO), B * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream), "shots download");
  if (rc) return rc;
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sample sync");
}

int bt_probabilities(const bt_state* s_, int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  if (member < 0 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  int rc = set_dev(ctx);
  if (rc) return rc;
  const int64_t len = 1LL << s->n;
  const int64_t chunk = 1LL << 23;
  Carve cv;
  int iO = cv.add((size_t)std::min(len, chunk) * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  for (int64_t o = 0; o < len && !rc; o += chunk) {
    int64_t l = std::min(chunk, len - o);
    rc = bt_launch_probs(s, member, o, l, cv.at<double>(iO));
    if (!rc) rc = bt_cuda_check(ctx, cudaMemcpyAsync(out + o, cv.at<double>(iO), l * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "probs download");
    if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "probs sync");
  }
  return rc;
}

// ------------------------------------------------------------------ observables
int bt_expect_pauli(const bt_state* s_, int nterms, const uint64_t* xmask, const uint64_t* zmask, const double* coef,
                    int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (nterms < 0 || (nterms > 0 && (!xmask || !zmask || !out))) return bt_fail(ctx, BT_ERR_BAD_ARG, "bad term arrays");
  const uint64_t valid = s->n >= 64 ? ~0ULL : ((1ULL << s->n) - 1);
  for (int t = 0; t < nterms; ++t)
    if ((xmask[t] | zmask[t]) & ~valid) return bt_fail(ctx, BT_ERR_BAD_ARG, "Pauli mask names a qubit beyond n");
  int64_t lo, nm;
  int rc = members(s, member, &lo, &nm);
  if (rc) return rc;
  if (nterms == 0) return BT_OK;
  if ((rc = set_dev(ctx))) return rc;
  std::map<uint64_t, std::vector<int>> groups;
  for (int t = 0; t < nterms; ++t) groups[xmask[t]].push_back(t);
  if (s->repr == BT_REPR_SV && s->nbits >= 8 && groups.size() >= 3) {
    // many x-masks: tiles of M bits holding the x-bits of up to
    // BT_PAULI_TILE_TERMS strings each, one read of the state per tile group
    const int c = s->prec == BT_PREC_C64 ? 5 : 4;
    const int M = std::min(s->prec == BT_PREC_C64 ? 13 : 12, s->nbits);
    std::vector<int> order;
    for (auto& g : groups)
      for (int t : g.second) order.push_back(t);  // equal x-masks adjacent: they share products
    std::vector<std::pair<uint64_t, std::vector<int>>> tg;  // (tile mask, terms)
    std::vector<char> used(nterms, 0);
    for (size_t start = 0; start < order.size();) {
      uint64_t Q = (1ULL << c) - 1;
      std::vector<int> ts;
      for (size_t k = start; k < order.size() && (int)ts.size() < BT_PAULI_TILE_TERMS; ++k) {
        const int t = order[k];
        if (used[t] || __builtin_popcountll(Q | xmask[t]) > M) continue;
        Q |= xmask[t];
        ts.push_back(t);
        used[t] = 1;
      }
      for (int b = 0; b < s->nbits && __builtin_popcountll(Q) < M; ++b) Q |= 1ULL << b;
      tg.push_back({Q, ts});
      while (start < order.size() && used[order[start]]) ++start;
    }
    Carve cv;
    const int W = BT_PAULI_TILE_TERMS;
    int iR = cv.add(tg.size() * nm * W * sizeof(double));
    if ((rc = cv.commit(ctx))) return rc;
    double* res = cv.at<double>(iR);
    for (size_t gi = 0; gi < tg.size() && !rc; ++gi) {
      uint64_t xs[BT_PAULI_TILE_TERMS], zs[BT_PAULI_TILE_TERMS];
      const auto& ts = tg[gi].second;
      for (size_t j = 0; j < ts.size(); ++j) xs[j] = xmask[ts[j]], zs[j] = zmask[ts[j]];
      rc = bt_launch_pauli_tile(s, M, tg[gi].first, (int)ts.size(), xs, zs, lo, nm, res + gi * nm * W);
    }
    if (rc) return rc;
    std::vector<double> h(tg.size() * nm * W);
    rc = bt_cuda_check(ctx, cudaMemcpyAsync(h.data(), res, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "expect download");
    if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "expect sync");
    if (rc) return rc;
    for (size_t gi = 0; gi < tg.size(); ++gi) {
      const auto& ts = tg[gi].second;
      for (int64_t m = 0; m < nm; ++m)
        for (size_t j = 0; j < ts.size(); ++j)
          out[m * nterms + ts[j]] = (coef ? coef[ts[j]] : 1.0) * h[(gi * nm + m) * W + j];
    }
    return BT_OK;
  }
  // few x-masks: one read pass per group of <= 8 strings sharing an x-mask
  std::vector<std::pair<uint64_t, std::vector<int>>> batches;
  for (auto& g : groups)
    for (size_t i = 0; i < g.second.size(); i += 8)
      batches.push_back({g.first, std::vector<int>(g.second.begin() + i, g.second.begin() + std::min(g.second.size(), i + 8))});
  Carve cv;
  int iR = cv.add(batches.size() * nm * 8 * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  double* res = cv.at<double>(iR);
  for (size_t bi = 0; bi < batches.size() && !rc; ++bi) {
    uint64_t z[8];
    const auto& ts = batches[bi].second;
    for (size_t j = 0; j < ts.size(); ++j) z[j] = zmask[ts[j]];
    rc = bt_launch_pauli(s, batches[bi].first, (int)ts.size(), z, lo, nm, res + bi * nm * 8);
  }
  if (rc) return rc;
  std::vector<double> h(batches.size() * nm * 8);
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(h.data(), res, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "expect download");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "expect sync");
  if (rc) return rc;
  for (size_t bi = 0; bi < batches.size(); ++bi) {
    const auto& ts = batches[bi].second;
    for (int64_t m = 0; m < nm; ++m)
      for (size_t j = 0; j < ts.size(); ++j) {
        double c = coef ? coef[ts[j]] : 1.0;
        out[m * nterms + ts[j]] = c * h[(bi * nm + m) * 8 + j];
      }
  }
  return BT_OK;
}

int bt_expect_z_all(const bt_state* s_, int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  int64_t lo, nm;
  int rc = members(s, member, &lo, &nm);
  if (rc) return rc;
  if ((rc = set_dev(ctx))) return rc;
  Carve cv;
  int iR = cv.add(nm * 36 * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  if ((rc = bt_launch_bitsums(s, lo, nm, cv.at<double>(iR)))) return rc;
  std::vector<double> h(nm * 36);
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(h.data(), cv.at<double>(iR), h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "expect download");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "expect sync");
  if (rc) return rc;
  for (int64_t m = 0; m < nm; ++m)
    for (int q = 1; q <= s->n; ++q) out[m * s->n + q - 1] = h[m * 36] - 2.0 * h[m * 36 + 1 + (s->n - q)];
  return BT_OK;
}

int bt_expect_matrix(const bt_state* s_, int k, const int32_t* qubits, const double* mat, int nctrl,
                     const int32_t* ctrls, int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!mat || !out) return bt_fail(ctx, BT_ERR_BAD_ARG, "NULL argument");
  if (s->repr != BT_REPR_SV) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "expect_matrix needs a state vector");
  int rc = check_qubits(ctx, s->n, k, qubits, nctrl, ctrls);
  if (rc) return rc;
  if (k > 2) return bt_fail(ctx, BT_ERR_UNSUPPORTED, "expect_matrix supports k <= 2");
  if (member < 0 || member >= s->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  if ((rc = set_dev(ctx))) return rc;
  const int d = 1 << k;
  std::vector<double> rm(2 * d * d);
  to_rowmajor(mat, d, rm.data());
  Carve cv;
  int iM = cv.add(rm.size() * sizeof(double));
  int iR = cv.add(sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(cv.at<double>(iM), rm.data(), rm.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "matrix upload");
  if (rc) return rc;
  int bits[2];
  uint64_t cmask = 0;
  for (int i = 0; i < k; ++i) bits[i] = s->n - qubits[i];
  for (int i = 0; i < nctrl; ++i) cmask |= 1ULL << (s->n - ctrls[i]);
  if ((rc = bt_launch_expect_matrix(s, k, bits, cv.at<double>(iM), cmask, member, cv.at<double>(iR)))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(out, cv.at<double>(iR), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "expect download");
  if (rc) return rc;
  return bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "expect sync");
}

int bt_norm2(const bt_state* s_, int64_t member, double* out) {
  if (!s_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* s = const_cast<bt_state*>(s_);
  bt_ctx* ctx = s->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  int64_t lo, nm;
  int rc = members(s, member, &lo, &nm);
  if (rc) return rc;
  if ((rc = set_dev(ctx))) return rc;
  Carve cv;
  int iR = cv.add(nm * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  if ((rc = bt_launch_norm2(s, lo, nm, cv.at<double>(iR)))) return rc;
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(out, cv.at<double>(iR), nm * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "norm download");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "norm sync");
  return rc;
}

int bt_fidelity(const bt_state* a_, int64_t am, const bt_state* b_, int64_t bm, double* out) {
  if (!a_ || !b_) return bt_fail(nullptr, BT_ERR_BAD_ARG, "state is NULL");
  bt_state* a = const_cast<bt_state*>(a_);
  bt_state* b = const_cast<bt_state*>(b_);
  bt_ctx* ctx = a->ctx;
  if (!out) return bt_fail(ctx, BT_ERR_BAD_ARG, "out is NULL");
  if (a->n != b->n || a->repr != BT_REPR_SV || b->repr != BT_REPR_SV)
    return bt_fail(ctx, BT_ERR_BAD_ARG, "fidelity needs two state vectors of equal size");
  if (am < 0 || am >= a->batch || bm < 0 || bm >= b->batch) return bt_fail(ctx, BT_ERR_BAD_ARG, "member out of range");
  int rc = set_dev(ctx);
  if (rc) return rc;
  if (b->ctx != ctx) cudaStreamSynchronize(b->ctx->stream);
  Carve cv;
  int iR = cv.add(2 * sizeof(double));
  if ((rc = cv.commit(ctx))) return rc;
  if ((rc = bt_launch_inner(a, am, b, bm, cv.at<double>(iR)))) return rc;
  double h[2];
  rc = bt_cuda_check(ctx, cudaMemcpyAsync(h, cv.at<double>(iR), sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "fidelity download");
  if (!rc) rc = bt_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "fidelity sync");
  if (rc) return rc;
  *out = h[0] * h[0] + h[1] * h[1];
  return BT_OK;
}

}  // extern "C"
