// PsOps of PsLambert, PsLambertTex.
#include "swr_ps_impl.cuh"

namespace swr {

const PsOps* ps_ops_lambert(int id) {
  static const PsOps kPsLambert = make_ps<PsLambert>();
  static const PsOps kPsLambertTex = make_ps<PsLambertTex>();
  switch (id) {
    case SWR_PS_LAMBERT: return &kPsLambert;
    case SWR_PS_LAMBERT_TEX: return &kPsLambertTex;
    default: return nullptr;
  }
}

}  // namespace swr
