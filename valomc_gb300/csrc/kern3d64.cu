// kern3d64.cu -- instantiations of the photon-pool kernel for the Walk3D64 walker:
// continuous-wave / frequency-domain x (Philox, replay tape).  A separate translation
// unit per walker so the build compiles them in parallel.
#include "pool.cuh"

namespace vmc {

namespace {
template <class F> const void *K(F *f) { return reinterpret_cast<const void *>(f); }
template <bool FD, class R> const void *per_job(bool tab) {
  return tab ? K(&pool_kernel<Walk3D64<FD, R>, R, true>) : K(&pool_kernel<Walk3D64<FD, R>, R, false>);
}
}  // namespace

const void *kernel_3d64(bool fd, bool tape, bool /*one: FP32 walks only*/, bool tab) {
  if (tape) return fd ? per_job<true, TapeRng>(tab) : per_job<false, TapeRng>(tab);
  return fd ? per_job<true, PhiloxRng>(tab) : per_job<false, PhiloxRng>(tab);
}

}  // namespace vmc
