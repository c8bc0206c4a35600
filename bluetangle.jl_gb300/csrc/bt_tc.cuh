// Tensor-core fused passes (bt_tc.cu): the planner's fused tile passes with every
// register phase applied as one dense 32 x 32 complex block by tcgen05.mma
// (kind::tf32, three TF32 products, FP32 accumulation); complex64 states, tiles of
// 2^13 amplitudes, 5 register bits per phase.
#pragma once
#include "bt_fused.cuh"

// device status word set when an MMA completion wait runs out (the kernel then
// stops, frees its tensor memory and returns)
#define BT_STATUS_TC_TIMEOUT 16

struct TcPass {
  int nbits, c, nphase, lg_tiles;
  int64_t member_lo, nmem;
  int tbits[16];                         // tile-local bit -> global bit (13 tile bits)
  uint8_t reg[BT_FUSED_MAX_PHASES][5];   // per phase: the block's tile-local bits, bit b of the block index
  const float* bmat;                     // device: per phase 8192 floats (B hi, B lo; bt_tc_block_image)
};

int bt_launch_tc_pass(bt_ctx* ctx, void* psi, const TcPass& a);
// the MMA operand image (TF32 hi then lo, 2 x 4096 floats in the K-major core layout)
// of the real form of a 32 x 32 complex matrix u (row-major interleaved complex128)
void bt_tc_block_image(const double* u, float* out);
