// Plan specialisation with NVRTC (bt_jit.cu).
#pragma once
#include <string>
#include <vector>

#include "bt_fused.cuh"

bool bt_jit_available();
int bt_jit_min_blocks();  // CTAs per SM the specialised passes are compiled for (BTGPU_JIT_MINB, default 2)
int bt_jit_max_ops();     // gates per specialised pass at most (BTGPU_PLAN_MAX_OPS, default 96)
int bt_tile_rb(bool c64); // register bits per thread of a fused pass (complex64: BTGPU_TILE_RB, 4 or 5)
bool bt_jit_packed_default();  // complex64 specialised passes in two-lane arithmetic (BTGPU_JIT_PACKED)
// compiles (once per distinct pass structure) and returns one kernel entry per pass
int bt_jit_prepare_f(bt_ctx* ctx, std::vector<const FusedArgs<float>*>& passes, std::vector<void*>& out);
int bt_jit_prepare_d(bt_ctx* ctx, std::vector<const FusedArgs<double>*>& passes, std::vector<void*>& out);
int bt_jit_launch_f(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<float>& a);
int bt_jit_launch_d(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<double>& a);
// kernels compiled with a.permem: member member_lo + m reads row m of the device
// table mm (mstride reals per row)
int bt_jit_launch_members_f(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<float>& a, const float* mm,
                            int64_t mstride);
int bt_jit_launch_members_d(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<double>& a, const double* mm,
                            int64_t mstride);
