// Generic fused tile passes for complex64 states (templates in bt_fused_impl.cuh).
// One tile size per translation unit (this file: 2^13; bt_fused_c64_m1x.cu the
// smaller tiles) so that the build compiles them in parallel.
#include "bt_fused_impl.cuh"

int bt_fused_f12(bt_ctx* ctx, void* psi, const FusedArgs<float>& a);
int bt_fused_f11(bt_ctx* ctx, void* psi, const FusedArgs<float>& a);
int bt_fused_f10(bt_ctx* ctx, void* psi, const FusedArgs<float>& a);

int bt_launch_fused_f(bt_ctx* ctx, void* psi, const FusedArgs<float>& a) {
  if (a.nphase > 0 && a.ph[0].nreg != BT_TILE_RB_C64)
    return bt_fail(ctx, BT_ERR_UNSUPPORTED, "a pass of 4 register bits runs only as a specialised kernel");
  switch (a.M) {
    case 13: return launch_fused<float, 13, BT_TILE_RB_C64>(ctx, psi, a);
    case 12: return bt_fused_f12(ctx, psi, a);
    case 11: return bt_fused_f11(ctx, psi, a);
    case 10: return bt_fused_f10(ctx, psi, a);
  }
  return bt_fail(ctx, BT_ERR_BAD_ARG, "fused pass: unsupported tile size");
}
