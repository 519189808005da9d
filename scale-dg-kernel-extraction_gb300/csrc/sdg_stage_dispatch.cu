// Runtime dispatch of the fused stage kernel on the polynomial order (the
// C++ template replaces the reference's ERB-generated per-order kernels and
// the select case of mod_dg_optr_kernel.f90:87-133).
#include "sdg_stage.cuh"

namespace sdg {

#define SDG_DECL_ORDER(p) \
  int launch_stage_p##p(int prec, int opt, const StageArgs& a, cudaStream_t st);
SDG_DECL_ORDER(1) SDG_DECL_ORDER(2) SDG_DECL_ORDER(3) SDG_DECL_ORDER(4)
SDG_DECL_ORDER(5) SDG_DECL_ORDER(6) SDG_DECL_ORDER(7) SDG_DECL_ORDER(8)
SDG_DECL_ORDER(9) SDG_DECL_ORDER(10) SDG_DECL_ORDER(11) SDG_DECL_ORDER(12)
SDG_DECL_ORDER(13) SDG_DECL_ORDER(14) SDG_DECL_ORDER(15)
#undef SDG_DECL_ORDER

int launch_stage(int p, int prec, int opt, const StageArgs& a, cudaStream_t st) {
  if (prec != SDG_PREC_FP64 && prec != SDG_PREC_FP32 && prec != SDG_PREC_FP64_EMU)
    return fail(SDG_ERR_INVALID_ARG, "unknown precision %d", prec);
  if (opt != SDG_OPT_GENERAL && opt != SDG_OPT_OPT1 && opt != SDG_OPT_EVENODD)
    return fail(SDG_ERR_BAD_OPTTYPE, "unknown DGOptrKernel type %d", opt);
  switch (p) {
    case 1: return launch_stage_p1(prec, opt, a, st);
    case 2: return launch_stage_p2(prec, opt, a, st);
    case 3: return launch_stage_p3(prec, opt, a, st);
    case 4: return launch_stage_p4(prec, opt, a, st);
    case 5: return launch_stage_p5(prec, opt, a, st);
    case 6: return launch_stage_p6(prec, opt, a, st);
    case 7: return launch_stage_p7(prec, opt, a, st);
    case 8: return launch_stage_p8(prec, opt, a, st);
    case 9: return launch_stage_p9(prec, opt, a, st);
    case 10: return launch_stage_p10(prec, opt, a, st);
    case 11: return launch_stage_p11(prec, opt, a, st);
    case 12: return launch_stage_p12(prec, opt, a, st);
    case 13: return launch_stage_p13(prec, opt, a, st);
    case 14: return launch_stage_p14(prec, opt, a, st);
    case 15: return launch_stage_p15(prec, opt, a, st);
    default:
      return fail(SDG_ERR_UNSUPPORTED_ORDER, "PolyOrder %d outside 1..15", p);
  }
}

}  // namespace sdg
