// kern3d32.cu -- instantiations of the photon-pool kernel for the Walk3D32 walker:
// continuous-wave / frequency-domain x (Philox of a one-job launch, Philox per job,
// replay tape).  A separate translation unit per walker so the build compiles them in
// parallel.
#include "pool.cuh"

namespace vmc {

const void *kernel_3d32(bool fd, bool tape, bool one) {
  if (fd) {
    if (tape) return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<true, TapeRng>, TapeRng>);
    if (one) return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<true, PhiloxOne>, PhiloxOne>);
    return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<true, PhiloxRng>, PhiloxRng>);
  }
  if (tape) return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<false, TapeRng>, TapeRng>);
  if (one) return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<false, PhiloxOne>, PhiloxOne>);
  return reinterpret_cast<const void *>(&pool_kernel<Walk3D32<false, PhiloxRng>, PhiloxRng>);
}

}  // namespace vmc
