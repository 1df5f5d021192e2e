// Mixed-precision kernels (FP32 reconstruction/flux, FP64 state and update).
#include "fvh_mixed.h"

namespace fvh {
namespace mixed {

struct workspace {};

fvh_status create(const fvh_mesh_view &, const fvh_params &, workspace **out) {
  *out = nullptr;
  return FVH_ERR_UNSUPPORTED;
}

void destroy(workspace *w) { delete w; }

cudaError_t step(workspace *, const fvh_mesh_view &, const fvh_params &,
                 const fvh_state_view &, double *, double *, double *, int,
                 fvh_device_status *, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace mixed
}  // namespace fvh
