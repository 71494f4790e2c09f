// PsOps of PsTexNearest, PsTexMip.
#include "swr_ps_impl.cuh"

namespace swr {

const PsOps* ps_ops_tex(int id) {
  static const PsOps kPsTexNearest = make_ps<PsTexNearest>();
  static const PsOps kPsTexMip = make_ps<PsTexMip>();
  switch (id) {
    case SWR_PS_TEX_NEAREST: return &kPsTexNearest;
    case SWR_PS_TEX_MIP: return &kPsTexMip;
    default: return nullptr;
  }
}

}  // namespace swr
