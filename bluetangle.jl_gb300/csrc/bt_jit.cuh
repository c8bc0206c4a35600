// Plan specialisation with NVRTC (bt_jit.cu).
#pragma once
#include <string>
#include <vector>

#include "bt_fused.cuh"

bool bt_jit_available();
// compiles (once per distinct pass structure) and returns one kernel entry per pass
int bt_jit_prepare_f(bt_ctx* ctx, std::vector<const FusedArgs<float>*>& passes, std::vector<void*>& out);
int bt_jit_prepare_d(bt_ctx* ctx, std::vector<const FusedArgs<double>*>& passes, std::vector<void*>& out);
int bt_jit_launch_f(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<float>& a);
int bt_jit_launch_d(bt_ctx* ctx, void* entry, void* psi, const FusedArgs<double>& a);
