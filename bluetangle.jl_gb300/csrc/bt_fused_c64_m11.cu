// Generic fused tile pass, complex64, tiles of 2^11 amplitudes (bt_fused_impl.cuh).
#include "bt_fused_impl.cuh"

int bt_fused_f11(bt_ctx* ctx, void* psi, const FusedArgs<float>& a) {
  return launch_fused<float, 11, BT_TILE_RB_C64>(ctx, psi, a);
}
