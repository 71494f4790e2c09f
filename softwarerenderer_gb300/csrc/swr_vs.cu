// Vertex-stage kernels of the built-in vertex shaders.
#include "swr_vs_impl.cuh"

namespace swr {
namespace {

const VsOps kPosUV = make_vs<VsPosUV>();
const VsOps kPosNrmUV = make_vs<VsPosNrmUV>();
const VsOps kPosRGB = make_vs<VsPosRGB>();
const VsOps kPosRGBAffine = make_vs<VsPosRGBAffine>();
const VsOps kPosRGBUV = make_vs<VsPosRGBUV>();

}  // namespace

const VsOps* vs_ops(int id) {
  switch (id) {
    case SWR_VS_POS_UV: return &kPosUV;
    case SWR_VS_POS_NRM_UV: return &kPosNrmUV;
    case SWR_VS_POS_RGB: return &kPosRGB;
    case SWR_VS_POS_RGB_AFFINE: return &kPosRGBAffine;
    case SWR_VS_POS_RGB_UV: return &kPosRGBUV;
    default: return nullptr;
  }
}

}  // namespace swr
