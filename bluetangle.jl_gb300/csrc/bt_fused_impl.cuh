// Fused tile pass: many 1- and 2-qubit gates per HBM round trip.
//
// A CTA owns a tile of 2^M amplitudes (M = 13 for complex64, 12 for complex128;
// 64 KiB of shared memory): the amplitudes whose M "tile bits" vary while every
// other bit is fixed.  The tile bits always include the lowest global bits, so the
// tile is 2^(M-c) contiguous 256-byte runs, loaded and stored with 16-byte
// accesses.  The pass program (from the planner in bt_plan.cu) is a list of
// register phases: in a phase each of the 256 threads gathers the 2^RB amplitudes
// that differ in the phase's RB register bits (RB = 5 / 4) from the swizzled
// shared-memory tile, applies the phase's gates with compile-time register
// indices, and scatters them back.  One pass therefore costs one read and one
// write of the state however many gates it holds; it replaces that many separate
// sweeps (each an HBM round trip) of the reference's per-gate operator products
// (BlueTangle.jl src/hilbert.jl:505, :517-553).
//
// This header holds the kernel templates (the generic pass interprets its op list
// at run time; plans normally run specialised kernels, bt_jit.cu).
#pragma once
#include <atomic>

#include "bt_fused.cuh"

template <typename R>
__device__ __forceinline__ int swz(int l) {
  // XOR the bank-selecting low bits with the next bits: conflict-free 8/16-byte
  // accesses for threads that differ in those next bits
  if constexpr (sizeof(R) == 4) return l ^ ((l >> 4) & 15);
  else return l ^ ((l >> 3) & 7);
}

template <int J>
struct LowBit { static constexpr int v = (J & 1) ? 0 : 1 + LowBit<(J >> 1)>::v; };
template <>
struct LowBit<0> { static constexpr int v = 0; };

// ---------------------------------------------------------------- register ops
template <typename R, int NB, int B>
__device__ __forceinline__ void op_g1(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B < NB) {
    const R m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3];
    const R m10r = m[4], m10i = m[5], m11r = m[6], m11i = m[7];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      xr[j] = fma(m00r, ar, fma(-m00i, ai, fma(m01r, br, -m01i * bi)));
      xi[j] = fma(m00r, ai, fma(m00i, ar, fma(m01r, bi, m01i * br)));
      xr[k] = fma(m10r, ar, fma(-m10i, ai, fma(m11r, br, -m11i * bi)));
      xi[k] = fma(m10r, ai, fma(m10i, ar, fma(m11r, bi, m11i * br)));
    }
  }
}

template <typename R, int NB, int B>
__device__ __forceinline__ void op_d1(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B < NB) {
    const R d0r = m[0], d0i = m[1], d1r = m[2], d1i = m[3];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      const R dr = (j & (1 << B)) ? d1r : d0r, di = (j & (1 << B)) ? d1i : d0i;
      const R ar = xr[j], ai = xi[j];
      xr[j] = fma(dr, ar, -di * ai);
      xi[j] = fma(dr, ai, di * ar);
    }
  }
}

// matrix index r = 2*bit(B0) + bit(B1)
template <typename R, int NB, int B0, int B1>
__device__ __forceinline__ void op_g2(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B0 < NB && B1 < NB && B0 != B1) {
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & ((1 << B0) | (1 << B1))) continue;
      const int q[4] = {j, j | (1 << B1), j | (1 << B0), j | (1 << B0) | (1 << B1)};
      R ar[4], ai[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) { ar[c] = xr[q[c]]; ai[c] = xi[q[c]]; }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        R yr = 0, yi = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const R mr = m[2 * (4 * r + c)], mi = m[2 * (4 * r + c) + 1];
          yr = fma(mr, ar[c], fma(-mi, ai[c], yr));
          yi = fma(mr, ai[c], fma(mi, ar[c], yi));
        }
        xr[q[r]] = yr;
        xi[q[r]] = yi;
      }
    }
  }
}

template <typename R, int NB, int B0, int B1>
__device__ __forceinline__ void op_d2(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B0 < NB && B1 < NB && B0 != B1) {
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      const int r = ((j >> B0) & 1) * 2 + ((j >> B1) & 1);
      const R dr = m[2 * r], di = m[2 * r + 1];
      const R ar = xr[j], ai = xi[j];
      xr[j] = fma(dr, ar, -di * ai);
      xi[j] = fma(dr, ai, di * ar);
    }
  }
}

template <typename R>
__device__ __forceinline__ R sel4(int p, R a, R b, R c, R d) {
  return p == 0 ? a : (p == 1 ? b : (p == 2 ? c : d));
}

// out[r] = ph[r] * in[perm[r]]
template <typename R, int NB, int B0, int B1>
__device__ __forceinline__ void op_p2(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m, int perm,
                                      int unit) {
  if constexpr (B0 < NB && B1 < NB && B0 != B1) {
    const int p0 = perm & 3, p1 = (perm >> 2) & 3, p2 = (perm >> 4) & 3, p3 = (perm >> 6) & 3;
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & ((1 << B0) | (1 << B1))) continue;
      const int q[4] = {j, j | (1 << B1), j | (1 << B0), j | (1 << B0) | (1 << B1)};
      const R ar[4] = {xr[q[0]], xr[q[1]], xr[q[2]], xr[q[3]]};
      const R ai[4] = {xi[q[0]], xi[q[1]], xi[q[2]], xi[q[3]]};
      const int pp[4] = {p0, p1, p2, p3};
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const R vr = sel4(pp[r], ar[0], ar[1], ar[2], ar[3]);
        const R vi = sel4(pp[r], ai[0], ai[1], ai[2], ai[3]);
        if (unit) {
          xr[q[r]] = vr;
          xi[q[r]] = vi;
        } else {
          const R dr = m[2 * r], di = m[2 * r + 1];
          xr[q[r]] = fma(dr, vr, -di * vi);
          xi[q[r]] = fma(dr, vi, di * vr);
        }
      }
    }
  }
}

// CNOT with control register bit BC and target BT: swap the pair where the control is 1
template <typename R, int NB, int BC, int BT>
__device__ __forceinline__ void op_cx(R (&xr)[1 << NB], R (&xi)[1 << NB]) {
  if constexpr (BC < NB && BT < NB && BC != BT) {
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (!(j & (1 << BC)) || (j & (1 << BT))) continue;
      const int k = j | (1 << BT);
      const R tr = xr[j], ti = xi[j];
      xr[j] = xr[k];
      xi[j] = xi[k];
      xr[k] = tr;
      xi[k] = ti;
    }
  }
}

template <typename R, int NB, int B0, int B1>
__device__ __forceinline__ void op_sw(R (&xr)[1 << NB], R (&xi)[1 << NB]) {
  if constexpr (B0 < NB && B1 < NB && B0 != B1) {
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (!(j & (1 << B0)) || (j & (1 << B1))) continue;
      const int k = (j & ~(1 << B0)) | (1 << B1);
      const R tr = xr[j], ti = xi[j];
      xr[j] = xr[k];
      xi[j] = xi[k];
      xr[k] = tr;
      xi[k] = ti;
    }
  }
}

// out0 = p0 * in1, out1 = p1 * in0
template <typename R, int NB, int B>
__device__ __forceinline__ void op_x1(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m, int unit) {
  if constexpr (B < NB) {
    const R p0r = m[0], p0i = m[1], p1r = m[2], p1i = m[3];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      if (unit) {
        xr[j] = br; xi[j] = bi; xr[k] = ar; xi[k] = ai;
      } else {
        xr[j] = fma(p0r, br, -p0i * bi);
        xi[j] = fma(p0r, bi, p0i * br);
        xr[k] = fma(p1r, ar, -p1i * ai);
        xi[k] = fma(p1r, ai, p1i * ar);
      }
    }
  }
}

// real 2x2 matrix [[a, b], [c, d]]
template <typename R, int NB, int B>
__device__ __forceinline__ void op_r1(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B < NB) {
    const R a = m[0], b = m[1], c = m[2], d = m[3];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      xr[j] = fma(a, ar, b * br);
      xi[j] = fma(a, ai, b * bi);
      xr[k] = fma(c, ar, d * br);
      xi[k] = fma(c, ai, d * bi);
    }
  }
}

// [[a, i b], [i b, a]]: out0 = a in0 + i b in1, out1 = i b in0 + a in1
template <typename R, int NB, int B>
__device__ __forceinline__ void op_rx1(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m) {
  if constexpr (B < NB) {
    const R a = m[0], b = m[1];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      xr[j] = fma(a, ar, -b * bi);
      xi[j] = fma(a, ai, b * br);
      xr[k] = fma(a, br, -b * ai);
      xi[k] = fma(a, bi, b * ar);
    }
  }
}

// diag(1, q), or diag(q, 1) when lo (the factored scalar is folded elsewhere in
// the pass); code 2: q = -1, 3: q = i, 4: q = -i
template <typename R, int NB, int B>
__device__ __forceinline__ void op_dh(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m, int code,
                                      int lo) {
  if constexpr (B < NB) {
    const R qr = m[0], qi = m[1];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (((j >> B) & 1) == lo) continue;
      const R ar = xr[j], ai = xi[j];
      if (code == 2) {
        xr[j] = -ar; xi[j] = -ai;
      } else if (code == 3) {
        xr[j] = -ai; xi[j] = ar;
      } else if (code == 4) {
        xr[j] = ai; xi[j] = -ar;
      } else {
        xr[j] = fma(qr, ar, -qi * ai);
        xi[j] = fma(qr, ai, qi * ar);
      }
    }
  }
}

// butterfly [[1, s01], [s10, s11]] with s = -1 where bits 0, 1, 2 of fl are set
template <typename R, int NB, int B>
__device__ __forceinline__ void op_hb(R (&xr)[1 << NB], R (&xi)[1 << NB], int fl) {
  if constexpr (B < NB) {
    const R s01 = (fl & 1) ? R(-1) : R(1), s10 = (fl & 2) ? R(-1) : R(1), s11 = (fl & 4) ? R(-1) : R(1);
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      xr[j] = fma(s01, br, ar);
      xi[j] = fma(s01, bi, ai);
      xr[k] = fma(s11, br, s10 * ar);
      xi[k] = fma(s11, bi, s10 * ai);
    }
  }
}

// real [[1, p], [q, s]] (flags bit 1 clear) or [[p, 1], [s, q]] (set), s = -1 if flags bit 0
template <typename R, int NB, int B>
__device__ __forceinline__ void op_rn(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m, int fl) {
  if constexpr (B < NB) {
    const R p = m[0], q = m[1], sg = (fl & 1) ? R(-1) : R(1);
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      if (!(fl & 2)) {
        xr[j] = fma(p, br, ar); xi[j] = fma(p, bi, ai);
        xr[k] = fma(q, ar, sg * br); xi[k] = fma(q, ai, sg * bi);
      } else {
        xr[j] = fma(p, ar, br); xi[j] = fma(p, ai, bi);
        xr[k] = fma(q, br, sg * ar); xi[k] = fma(q, bi, sg * ai);
      }
    }
  }
}

// [[1, it], [it, 1]] (flags bit 1 clear) or [[-it, 1], [1, -it]] (set)
template <typename R, int NB, int B>
__device__ __forceinline__ void op_rxn(R (&xr)[1 << NB], R (&xi)[1 << NB], const R* __restrict__ m, int fl) {
  if constexpr (B < NB) {
    const R t = m[0];
#pragma unroll
    for (int j = 0; j < (1 << NB); ++j) {
      if (j & (1 << B)) continue;
      const int k = j | (1 << B);
      const R ar = xr[j], ai = xi[j], br = xr[k], bi = xi[k];
      if (!(fl & 2)) {
        xr[j] = fma(-t, bi, ar); xi[j] = fma(t, br, ai);
        xr[k] = fma(-t, ai, br); xi[k] = fma(t, ar, bi);
      } else {
        xr[j] = fma(t, ai, br); xi[j] = fma(-t, ar, bi);
        xr[k] = fma(t, bi, ar); xi[k] = fma(-t, br, ai);
      }
    }
  }
}

#define BT_PAIRS(X)                                                                                     \
  X(0, 1) X(0, 2) X(0, 3) X(0, 4) X(1, 0) X(1, 2) X(1, 3) X(1, 4) X(2, 0) X(2, 1) X(2, 3) X(2, 4) X(3, 0) \
  X(3, 1) X(3, 2) X(3, 4) X(4, 0) X(4, 1) X(4, 2) X(4, 3)

template <typename R, int NB>
__device__ __forceinline__ void apply_op(R (&xr)[1 << NB], R (&xi)[1 << NB], const FOp o, const R* __restrict__ mat) {
  const R* m = mat + o.moff;
  switch (o.type) {
    case FOP_G1:
      switch (o.b0) {
        case 0: op_g1<R, NB, 0>(xr, xi, m); break;
        case 1: op_g1<R, NB, 1>(xr, xi, m); break;
        case 2: op_g1<R, NB, 2>(xr, xi, m); break;
        case 3: op_g1<R, NB, 3>(xr, xi, m); break;
        case 4: op_g1<R, NB, 4>(xr, xi, m); break;
      }
      break;
    case FOP_D1:
      switch (o.b0) {
        case 0: op_d1<R, NB, 0>(xr, xi, m); break;
        case 1: op_d1<R, NB, 1>(xr, xi, m); break;
        case 2: op_d1<R, NB, 2>(xr, xi, m); break;
        case 3: op_d1<R, NB, 3>(xr, xi, m); break;
        case 4: op_d1<R, NB, 4>(xr, xi, m); break;
      }
      break;
    case FOP_G2:
      switch (o.b0 * 8 + o.b1) {
#define X(a, b) case a * 8 + b: op_g2<R, NB, a, b>(xr, xi, m); break;
        BT_PAIRS(X)
#undef X
      }
      break;
    case FOP_D2:
      switch (o.b0 * 8 + o.b1) {
#define X(a, b) case a * 8 + b: op_d2<R, NB, a, b>(xr, xi, m); break;
        BT_PAIRS(X)
#undef X
      }
      break;
    case FOP_P2:
      switch (o.b0 * 8 + o.b1) {
#define X(a, b) case a * 8 + b: op_p2<R, NB, a, b>(xr, xi, m, o.flags, o.unit); break;
        BT_PAIRS(X)
#undef X
      }
      break;
    case FOP_CX:
      switch (o.b0 * 8 + o.b1) {
#define X(a, b) case a * 8 + b: op_cx<R, NB, a, b>(xr, xi); break;
        BT_PAIRS(X)
#undef X
      }
      break;
    case FOP_SW:
      switch (o.b0 * 8 + o.b1) {
#define X(a, b) case a * 8 + b: op_sw<R, NB, a, b>(xr, xi); break;
        BT_PAIRS(X)
#undef X
      }
      break;
#define ONE(FN, ...)                             \
  switch (o.b0) {                                \
    case 0: FN<R, NB, 0>(xr, xi, ##__VA_ARGS__); break; \
    case 1: FN<R, NB, 1>(xr, xi, ##__VA_ARGS__); break; \
    case 2: FN<R, NB, 2>(xr, xi, ##__VA_ARGS__); break; \
    case 3: FN<R, NB, 3>(xr, xi, ##__VA_ARGS__); break; \
    case 4: FN<R, NB, 4>(xr, xi, ##__VA_ARGS__); break; \
  }
    case FOP_X1: ONE(op_x1, m, o.unit) break;
    case FOP_R1: ONE(op_r1, m) break;
    case FOP_RX1: ONE(op_rx1, m) break;
    case FOP_DH: ONE(op_dh, m, o.unit, o.flags & 1) break;
    case FOP_HB: ONE(op_hb, o.flags) break;
    case FOP_RN: ONE(op_rn, m, o.flags) break;
    case FOP_RXN: ONE(op_rxn, m, o.flags) break;
#undef ONE
  }
}

// offsets of the 2^NB register amplitudes: off[j] = XOR of s[b] over the set bits b
// of j.  The swizzle is XOR-linear on disjoint bit sets (swz(a|b) = swz(a)^swz(b)),
// so with s[b] = swz(1 << reg[b]) the shared-memory index of amplitude j is
// swz(lbase) ^ off[j]: one XOR per access.
template <typename R, int NB, int J>
struct Offs {
  static __device__ __forceinline__ void fill(int (&off)[1 << NB], const int (&s)[NB]) {
    if constexpr (J < (1 << NB)) {
      off[J] = off[J & (J - 1)] ^ s[LowBit<J>::v];
      Offs<R, NB, J + 1>::fill(off, s);
    }
  }
};

template <typename R, int M, int NB>
__global__ void __launch_bounds__(1 << (M - NB), 2) k_fused(typename CT<R>::T* __restrict__ psi,
                                                              const FusedArgs<R> a) {
  typedef typename CT<R>::T C2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* tile = reinterpret_cast<C2*>(smem_raw);
  int64_t* runoff = reinterpret_cast<int64_t*>(smem_raw + (sizeof(C2) << M));
  const int c = a.c;
  const int nruns = 1 << (M - c);
  for (int r = threadIdx.x; r < nruns; r += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < M - c; ++b)
      if ((r >> b) & 1) o |= 1LL << a.tbits[c + b];
    runoff[r] = o;
  }
  __syncthreads();
  constexpr int V = 16 / sizeof(C2);
  constexpr int NCHUNK = (1 << M) / V;
  const int64_t per = 1LL << a.lg_tiles;
  const int64_t total = per * a.nmem;
  const int cmask = (1 << c) - 1;
  for (int64_t tid = blockIdx.x; tid < total; tid += gridDim.x) {
    const int64_t mem = a.member_lo + (tid >> a.lg_tiles);
    uint64_t base = (uint64_t)(tid & (per - 1));
    for (int i = 0; i < M; ++i) {
      const int p = a.tbits[i];
      base = ((base >> p) << (p + 1)) | (base & ((1ULL << p) - 1));
    }
    C2* g = psi + (mem << a.nbits) + base;
    // every 16-byte load of the tile in flight at once (NPT per thread), then to smem
    constexpr int T = 1 << (M - NB);
    constexpr int NPT = NCHUNK / T;
    {
      float4 buf[NPT];
#pragma unroll
      for (int i = 0; i < NPT; ++i) {
        const int l = (threadIdx.x + i * T) * V;
        buf[i] = __ldcs(reinterpret_cast<const float4*>(g + runoff[l >> c] + (l & cmask)));
      }
#pragma unroll
      for (int i = 0; i < NPT; ++i) {
        const int l = (threadIdx.x + i * T) * V;
        if constexpr (V == 2) {
          tile[swz<R>(l)] = make_float2(buf[i].x, buf[i].y);
          tile[swz<R>(l + 1)] = make_float2(buf[i].z, buf[i].w);
        } else {
          *reinterpret_cast<float4*>(&tile[swz<R>(l)]) = buf[i];
        }
      }
    }
    __syncthreads();
    for (int p = 0; p < a.nphase; ++p) {
      const FPhase ph = a.ph[p];
      uint32_t regmask = 0;
      int s[NB];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        regmask |= 1u << ph.reg[b];
        s[b] = swz<R>(1 << ph.reg[b]);
      }
      int lbase = 0;
      {
        int nb = 0;
        const int t = threadIdx.x;
        for (int bit = 0; bit < M; ++bit)
          if (!((regmask >> bit) & 1)) {
            if ((t >> nb) & 1) lbase |= 1 << bit;
            ++nb;
          }
      }
      const int sbase = swz<R>(lbase);
      R xr[1 << NB], xi[1 << NB];
      {
        int off[1 << NB];
        off[0] = 0;
        Offs<R, NB, 1>::fill(off, s);
#pragma unroll
        for (int j = 0; j < (1 << NB); ++j) {
          const C2 v = tile[sbase ^ off[j]];
          xr[j] = v.x;
          xi[j] = v.y;
        }
      }
      for (int o = ph.op0; o < ph.op0 + ph.nop; ++o) apply_op<R, NB>(xr, xi, a.op[o], a.mat);
      // the offsets are recomputed rather than kept live across the op loop
#pragma unroll
      for (int b = 0; b < NB; ++b) asm volatile("" : "+r"(s[b]));
      {
        int off[1 << NB];
        off[0] = 0;
        Offs<R, NB, 1>::fill(off, s);
#pragma unroll
        for (int j = 0; j < (1 << NB); ++j) {
          C2 v;
          v.x = xr[j];
          v.y = xi[j];
          tile[sbase ^ off[j]] = v;
        }
      }
      __syncthreads();
    }
    {
      float4 buf[NPT];
#pragma unroll
      for (int i = 0; i < NPT; ++i) {
        const int l = (threadIdx.x + i * T) * V;
        if constexpr (V == 2) {
          const C2 v0 = tile[swz<R>(l)], v1 = tile[swz<R>(l + 1)];
          buf[i] = make_float4(v0.x, v0.y, v1.x, v1.y);
        } else {
          buf[i] = *reinterpret_cast<const float4*>(&tile[swz<R>(l)]);
        }
      }
#pragma unroll
      for (int i = 0; i < NPT; ++i) {
        const int l = (threadIdx.x + i * T) * V;
        __stcs(reinterpret_cast<float4*>(g + runoff[l >> c] + (l & cmask)), buf[i]);
      }
    }
    __syncthreads();
  }
}

template <typename R, int M, int NB>
static int launch_fused(bt_ctx* ctx, void* psi, const FusedArgs<R>& a) {
  typedef typename CT<R>::T C2;
  const size_t smem = (sizeof(C2) << M) + sizeof(int64_t) * (1 << (M - a.c));
  // one value per kernel (its largest tile), set once per device; contexts on
  // other threads may launch meanwhile
  static std::atomic<bool> attr_set[64] = {};
  if (ctx->device < 64 && !attr_set[ctx->device].load()) {
    cudaError_t e = cudaFuncSetAttribute(k_fused<R, M, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)((sizeof(C2) << M) + 8 * (1 << M)));
    if (e != cudaSuccess) return bt_cuda_check(ctx, e, "fused smem attribute");
    attr_set[ctx->device].store(true);
  }
  int64_t total = (1LL << a.lg_tiles) * a.nmem;
  int64_t grid = (int64_t)ctx->sm_count * 2 * 4;
  if (grid > total) grid = total;
  k_fused<R, M, NB><<<(unsigned)grid, 1 << (M - NB), smem, ctx->stream>>>((C2*)psi, a);
  ctx->launches++;
  return bt_cuda_check(ctx, cudaGetLastError(), "fused kernel launch");
}

// tiles smaller than the default hold a whole small state (2^(M-RB) threads per CTA)
// the launchers that instantiate these templates are bt_fused_c64.cu and
// bt_fused_c128.cu (two translation units, compiled in parallel)
