// Per-order launch entry: resolves precision and summation order to one
// instantiation of the fused stage kernels.
#pragma once

#include "sdg_stage.cuh"
#include "sdg_stage_emu.cuh"
#include "sdg_stage_emu_eo.cuh"
#include "sdg_stage_elem.cuh"
#include "sdg_stage_eo.cuh"
#include "sdg_stage_warp.cuh"

namespace sdg {

template <int P>
int launch_stage_order(int prec, int opt, const StageArgs& a, cudaStream_t st) {
  constexpr bool kCanSplit = (P > 7);
  // EVENODD: the even-odd bodies (FP64, FP32 and emulated FP64)
  const bool split = kCanSplit && (opt != SDG_OPT_GENERAL);
  if (prec == SDG_PREC_FP64_EMU) {
    if (opt == SDG_OPT_EVENODD) return launch_stage_emu_eo_impl<P>(a, st);
    return launch_stage_emu_impl<P>(a, st);
  }
  if (opt == SDG_OPT_EVENODD) {
    if (prec == SDG_PREC_FP64) return launch_stage_eo_impl<P, double>(a, st);
    // p = 1: one thread an element (same bits as the block body): 129.7
    // against 48.2 GDOF-updates/s at 128^3 on GB300
    if constexpr (P == 1) return launch_stage_elem_impl<P>(a, st);
    // p = 2, 3: one warp an element (same bits as the block body)
    if constexpr (P == 2 || P == 3) return launch_stage_warp_impl<P>(a, st);
    return launch_stage_eo_impl<P, float>(a, st);
  }
  if (prec == SDG_PREC_FP64) {
    if (split) return launch_stage_impl<P, double, double, kCanSplit>(a, st);
    return launch_stage_impl<P, double, double, false>(a, st);
  }
  if (split) return launch_stage_impl<P, float, float, kCanSplit>(a, st);
  return launch_stage_impl<P, float, float, false>(a, st);
}

}  // namespace sdg
