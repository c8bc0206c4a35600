// Shared declarations of the fused tile pass (bt_fused_impl.cuh, bt_jit.cu) and its
// planner (bt_plan.cu).
#pragma once
#include "bt_internal.cuh"

#define BT_FUSED_MAX_PHASES 48
#define BT_FUSED_MAX_OPS 192
#define BT_FUSED_MAX_REALS_F 4096  // float matrix entries per pass (16 KiB)
#define BT_FUSED_MAX_REALS_D 2048  // double matrix entries per pass (16 KiB)

// tile geometry: M tile bits held in shared memory (64 KiB), RB register bits per thread
#define BT_TILE_M_C64 13
#define BT_TILE_RB_C64 5
#define BT_TILE_M_C128 12
#define BT_TILE_RB_C128 4
#define BT_TILE_LOW_C64 5   // the lowest global bits always in a tile: 256-byte contiguous runs
#define BT_TILE_LOW_C128 4
#define BT_TILE_THREADS 256

enum {
  FOP_G1 = 1,  // general 2x2: m00 m01 m10 m11 (8 reals)
  FOP_D1 = 2,  // diagonal 2x2: d0 d1 (4 reals)
  FOP_G2 = 3,  // general 4x4 on (b0 = high bit, b1 = low bit) (32 reals)
  FOP_D2 = 4,  // diagonal 4x4 (8 reals)
  FOP_P2 = 5,  // monomial 4x4: out[r] = ph[r] * in[perm[r]]; perm packed in flags, phases 8 reals
  FOP_CX = 6,  // CNOT, control register bit b0, target b1 (register renaming, no arithmetic)
  FOP_SW = 7,  // SWAP of register bits b0, b1
  FOP_X1 = 8,  // anti-diagonal 2x2: out0 = p0*in1, out1 = p1*in0 (4 reals); unit: plain swap
  FOP_R1 = 9,  // real 2x2 (4 reals): H, RY, ...
  FOP_RX1 = 10,  // [[a, ib], [ib, a]] with a, b real (2 reals): RX
  FOP_DH = 11,   // diag(1, q), or diag(q, 1) when flags bit 0 is set (2 reals);
                 // unit 2: q = -1, 3: q = i, 4: q = -i (no arithmetic)
  FOP_HB = 12,   // butterfly [[1, s01], [s10, s11]], signs -1 where flags bits 0, 1, 2 are set (no reals)
  FOP_RN = 13,   // real [[1, p], [q, s]] (flags bit 1 clear) or [[p, 1], [s, q]] (set); s = -1 if
                 // flags bit 0 (2 reals p, q): a rotation with its larger entry factored out
  FOP_RXN = 14,  // [[1, it], [it, 1]] (flags bit 1 clear) or [[-it, 1], [1, -it]] (set) (1 real t)
};

struct FOp {
  uint8_t type, b0, b1, flags;  // flags for P2: perm[r] = (flags >> 2r) & 3
  uint16_t moff, unit;          // unit: P2 phases are all exactly 1
};

struct FPhase {
  uint8_t reg[6];  // tile-local bits held in registers (ascending), register bit b = reg[b] (b < nreg)
  uint8_t nreg;
  uint16_t op0, nop;
};

template <typename R>
struct FusedArgs {
  int nbits, M, c, nphase;
  int packed;               // specialised complex64 code in two-lane arithmetic (bt_jit.cu)
  int permem;               // specialised code reading entries from a per-member table (bt_jit.cu)
  int pbit;                 // lane bit (tile-local) of the pair-lane complex64 form, or -1: every
                            // phase holds it as its last register bit (bt_plan.cu, bt_jit.cu)
  int tbits[16];            // tile-local bit -> global bit (ascending; tbits[i] = i for i < c)
  int64_t member_lo, nmem;  // members processed
  int lg_tiles;             // log2(tiles per member) = nbits - M
  FPhase ph[BT_FUSED_MAX_PHASES];
  FOp op[BT_FUSED_MAX_OPS];
  R mat[sizeof(R) == 4 ? BT_FUSED_MAX_REALS_F : BT_FUSED_MAX_REALS_D];
};

int bt_launch_fused_f(bt_ctx* ctx, void* psi, const FusedArgs<float>& a);
int bt_launch_fused_d(bt_ctx* ctx, void* psi, const FusedArgs<double>& a);
