// kern2d64.cu -- instantiations of the photon-pool kernel for the Walk2D64 walker:
// continuous-wave / frequency-domain x (Philox, replay tape).  A separate translation
// unit per walker so the build compiles them in parallel.
#include "pool.cuh"

namespace vmc {

const void *kernel_2d64(bool fd, bool tape, bool /*one: FP32 walks only*/) {
  if (fd) {
    if (tape) return reinterpret_cast<const void *>(&pool_kernel<Walk2D64<true, TapeRng>, TapeRng>);
    return reinterpret_cast<const void *>(&pool_kernel<Walk2D64<true, PhiloxRng>, PhiloxRng>);
  }
  if (tape) return reinterpret_cast<const void *>(&pool_kernel<Walk2D64<false, TapeRng>, TapeRng>);
  return reinterpret_cast<const void *>(&pool_kernel<Walk2D64<false, PhiloxRng>, PhiloxRng>);
}

}  // namespace vmc
