// PsOps of PsVColor, PsVColorAffine.
#include "swr_ps_impl.cuh"

namespace swr {

const PsOps* ps_ops_color(int id) {
  static const PsOps kPsVColor = make_ps<PsVColor>();
  static const PsOps kPsVColorAffine = make_ps<PsVColorAffine>();
  switch (id) {
    case SWR_PS_VCOLOR: return &kPsVColor;
    case SWR_PS_VCOLOR_AFFINE: return &kPsVColorAffine;
    default: return nullptr;
  }
}

}  // namespace swr
