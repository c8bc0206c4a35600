// Generic fused tile passes for complex128 states (templates in bt_fused_impl.cuh).
#include "bt_fused_impl.cuh"

int bt_launch_fused_d(bt_ctx* ctx, void* psi, const FusedArgs<double>& a) {
  switch (a.M) {
    case 12: return launch_fused<double, 12, BT_TILE_RB_C128>(ctx, psi, a);
    case 11: return launch_fused<double, 11, BT_TILE_RB_C128>(ctx, psi, a);
    case 10: return launch_fused<double, 10, BT_TILE_RB_C128>(ctx, psi, a);
    case 9: return launch_fused<double, 9, BT_TILE_RB_C128>(ctx, psi, a);
  }
  return bt_fail(ctx, BT_ERR_BAD_ARG, "fused pass: unsupported tile size");
}
