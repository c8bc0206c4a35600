// Internal declarations of the btgpu engine (sm_103a).
//
// Data layout in HBM: one state is `batch` members stored back to back; a
// member is 2^nbits complex numbers (nbits = n for a state vector, 2n for a
// density matrix viewed as vec(rho) with rho[i, j] at i + j*2^n), interleaved
// (re, im) as double2 (c128) or float2 (c64).  Amplitude index bit b belongs
// to qubit n - b (qubit 1 is the most significant bit), as in the reference.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/btgpu.h"

#define BT_MAX_K 5        // dense matrices passed by value in kernel parameters
#define BT_THREADS 256    // threads per block for sweep and reduction kernels

struct bt_ctx {
  int device = 0;
  int sm_count = 152;
  cudaStream_t stream = nullptr;
  uint64_t seed = 0;
  uint64_t rng_calls = 0;  // distinct Philox counter block per RNG-consuming call
  std::string err;
  void* scratch = nullptr;  // device scratch, grown on demand (reductions, tables)
  size_t scratch_bytes = 0;
  void* work = nullptr;     // device workspace of reduction partials
  size_t work_bytes = 0;
  int* d_status = nullptr;  // device-side status word (decide kernels report here)
  int64_t launches = 0;
};

struct bt_state {
  bt_ctx* ctx = nullptr;
  int n = 0, repr = 0, prec = 0, batch = 1;
  int nbits = 0;             // bits per member: n (SV) or 2n (DM)
  int64_t member_elems = 0;  // 2^nbits complex numbers
  void* d = nullptr;
};

// ---------------------------------------------------------------- helpers
template <typename R> struct CT;
template <> struct CT<double> { typedef double2 T; };
template <> struct CT<float> { typedef float2 T; };

static inline size_t elem_bytes(int prec) { return prec == BT_PREC_C64 ? 8 : 16; }

// status handling (bt_api.cu)
int bt_fail(bt_ctx* ctx, int code, const std::string& msg);
int bt_cuda_check(bt_ctx* ctx, cudaError_t e, const char* what);
void* bt_scratch(bt_ctx* ctx, size_t bytes, int* rc);  // reuses/grows ctx->scratch (API-level tables)
int bt_work(bt_ctx* ctx, size_t bytes, double** out);  // reuses/grows ctx->work (kernel partials)

// ---------------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11): 10 rounds of two 32x32->64 multiplies
// with the published multipliers and Weyl key increments.
struct bt_u4 { uint32_t x, y, z, w; };

__host__ __device__ inline bt_u4 bt_philox(bt_u4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    bt_u4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// uniform double in [0, 1) with 53 random bits, for draw `index` of stream (s0, s1)
__host__ __device__ inline double bt_uniform(uint64_t key, uint64_t stream, uint64_t index) {
  bt_u4 c = {(uint32_t)index, (uint32_t)(index >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
  bt_u4 r = bt_philox(c, (uint32_t)key, (uint32_t)(key >> 32));
  uint64_t b = ((uint64_t)r.x << 21) ^ (uint64_t)(r.y >> 11);
  return (double)(b & ((1ULL << 53) - 1)) * (1.0 / 9007199254740992.0);
}

// insert a zero bit at each position of the ascending list pos[0..k-1]
__host__ __device__ inline uint64_t bt_insert_zeros(uint64_t g, int k, const int* pos) {
  for (int i = 0; i < k; ++i) {
    int p = pos[i];
    uint64_t lo = g & ((1ULL << p) - 1);
    g = ((g >> p) << (p + 1)) | lo;
  }
  return g;
}

// ---------------------------------------------------------------- launchers
// Gate sweep: dense k-qubit matrix on bit positions `bits` (bits[0] = MSB of the
// matrix index), all bits of cmask must read 1.  `m` is a row-major interleaved
// complex128 matrix (host).  per_member (device, precision R, row-major
// interleaved, pm_stride reals apart) replaces m when not null.
// active (device, one byte per member, optional): members with 0 are left untouched
int bt_launch_gate(bt_state* s, int k, const int* bits, const double* m_rowmajor, uint64_t cmask,
                   int64_t mem_lo, int64_t nmem, const void* per_member, int64_t pm_stride,
                   const int8_t* active = nullptr);

// Reductions write FP64 results per member into `out` (device), member-major.
// reduced density matrix (k <= 3) on bits: out[mem][2*D*D] row-major interleaved
// (active as for bt_launch_gate: members with 0 are not read and get zeros)
int bt_launch_rdm(bt_state* s, int k, const int* bits, int64_t mem_lo, int64_t nmem, double* out,
                  const int8_t* active = nullptr);
// Pauli terms sharing one xmask (<= 8 zmasks): out[mem][T] = Re <P_t>
int bt_launch_pauli(bt_state* s, uint64_t x, int T, const uint64_t* z, int64_t mem_lo, int64_t nmem,
                    double* out);
// up to BT_PAULI_TILE_TERMS strings whose x-masks lie inside one tile of M bits
// (tilemask, containing the lowest 5 (c64) / 4 (c128) bits), state vectors only:
// out[mem][BT_PAULI_TILE_TERMS], term t at index t
#define BT_PAULI_TILE_TERMS 24
int bt_launch_pauli_tile(bt_state* s, int M, uint64_t tilemask, int T, const uint64_t* x, const uint64_t* z,
                         int64_t mem_lo, int64_t nmem, double* out);
// per-bit weights: out[mem][0] = sum p, out[mem][1 + b] = sum_{bit b set} p (SV: p=|a|^2,
// DM: p = Re rho[i,i]); b over the n system bits
int bt_launch_bitsums(bt_state* s, int64_t mem_lo, int64_t nmem, double* out);
// out[mem] = sum |psi|^2 (state) or Re tr(rho) (density), FP64-accurate for every precision
int bt_launch_norm2(bt_state* s, int64_t mem_lo, int64_t nmem, double* out);
// out[mem][0..1] = <a_mem | b_mem'> (complex), one member each
int bt_launch_inner(bt_state* a, int64_t am, bt_state* b, int64_t bm, double* out);
// Re <psi| M |psi> for k <= 2 with controls
int bt_launch_expect_matrix(bt_state* s, int k, const int* bits, const double* m_rowmajor, uint64_t cmask,
                            int64_t mem, double* out);

// collapse: member m keeps amplitudes whose `bit` equals outcome[m] scaled by scale[m]
int bt_launch_collapse(bt_state* s, int bit, const int* d_outcome, const double* d_scale, int64_t mem_lo,
                       int64_t nmem);
// two-qubit collapse: member m keeps amplitudes whose bits (b1, b2) match outcome[m]
// (1..4: q1 = (o-1)&1, q2 = (o-1)>>1, the reference's order), scaled by scale[m]
int bt_launch_collapse2(bt_state* s, int b1, int b2, const int* d_outcome, const double* d_scale, int64_t mem_lo,
                        int64_t nmem);
// DM dephasing on one qubit: zero rho[i, j] where bit b of i differs from bit b of j
int bt_launch_dephase(bt_state* s, int b, int64_t mem_lo, int64_t nmem);

// device-side decisions (one thread per member)
int bt_launch_decide_measure(bt_ctx* ctx, int64_t nmem, const double* rdm /*[mem][8]*/, const double* u,
                             const int* forced, uint64_t rng_stream, int* outcome, double* scale,
                             double* p0);
// two-qubit measurement from the 4x4 reduced matrix [mem][32]: outcome 1..4, probs [mem][4]
int bt_launch_decide_measure2(bt_ctx* ctx, int64_t nmem, const double* rdm, const double* u, const int* forced,
                              uint64_t rng_stream, int* outcome, double* scale, double* probs);
struct bt_kraus_desc {
  int k, nk, ref_perm;  // ref_perm: probabilities from the pair permuted to ascending order
};
int bt_launch_decide_kraus(bt_state* s, bt_kraus_desc kd, int64_t nmem, const double* rdm,
                           const double* kraus_rowmajor, const double* u, const int* forced,
                           uint64_t rng_stream, int* branch, double* probs, void* per_member_out);

// sampling
int bt_launch_sample(bt_state* s, int64_t mem, int64_t shots, const double* d_u, uint64_t seed_stream,
                     int64_t* d_out);
int bt_launch_probs(bt_state* s, int64_t mem, int64_t offset, int64_t len, double* d_out);
// one shot per member: d_out[m] from member m's weights (d_u[m] or Philox draw m)
int bt_launch_sample_each(bt_state* s, const double* d_u, uint64_t seed_stream, int64_t* d_out);
// bt_plan_run_members on members [0, nmem) of s only (bt_plan.cu)
int bt_plan_run_members_n(bt_plan* p, bt_state* s, int64_t nmem, int count, const int64_t* add_index,
                          const double* mats);

// state maintenance
int bt_launch_set_basis(bt_state* s, int64_t mem_lo, int64_t nmem, uint64_t index);
int bt_launch_convert_in(bt_state* s, int64_t mem, int64_t offset, int64_t len, const double* d_src);
int bt_launch_convert_out(bt_state* s, int64_t mem, int64_t offset, int64_t len, double* d_dst);
int bt_launch_broadcast(bt_state* dst, const bt_state* src, int64_t src_mem);

static inline int bt_grid(const bt_ctx* ctx, int64_t work, int per_block = BT_THREADS, int waves = 16) {
  int64_t b = (work + per_block - 1) / per_block;
  int64_t cap = (int64_t)ctx->sm_count * waves;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}
