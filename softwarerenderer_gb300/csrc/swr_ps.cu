// Pixel-shader registry: id -> PsOps (the shaders are instantiated in swr_ps_*.cu).
#include "swr_ops.h"

namespace swr {

const PsOps* ps_ops_lambert(int id);
const PsOps* ps_ops_color(int id);
const PsOps* ps_ops_tex(int id);
const PsOps* ps_ops_deriv(int id);

const PsOps* ps_ops(int id) {
  if (const PsOps* o = ps_ops_lambert(id)) return o;
  if (const PsOps* o = ps_ops_color(id)) return o;
  if (const PsOps* o = ps_ops_tex(id)) return o;
  if (const PsOps* o = ps_ops_deriv(id)) return o;
  return nullptr;
}

}  // namespace swr
