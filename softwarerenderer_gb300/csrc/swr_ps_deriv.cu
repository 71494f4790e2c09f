// PsOps of PsDiff, PsPerspDeriv.
#include "swr_ps_impl.cuh"

namespace swr {

const PsOps* ps_ops_deriv(int id) {
  static const PsOps kPsDiff = make_ps<PsDiff>();
  static const PsOps kPsPerspDeriv = make_ps<PsPerspDeriv>();
  switch (id) {
    case SWR_PS_DIFF: return &kPsDiff;
    case SWR_PS_PERSP_DERIV: return &kPsPerspDeriv;
    default: return nullptr;
  }
}

}  // namespace swr
