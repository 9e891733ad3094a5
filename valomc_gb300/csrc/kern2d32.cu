// kern2d32.cu -- instantiations of the photon-pool kernel for the Walk2D32 walker:
// continuous-wave / frequency-domain x (Philox of a one-job launch, Philox per job,
// replay tape).  A separate translation unit per walker so the build compiles them in
// parallel.
#include "pool.cuh"

namespace vmc {

namespace {
template <class F> const void *K(F *f) { return reinterpret_cast<const void *>(f); }
template <bool FD, class R> const void *per_job(bool tab) {
  return tab ? K(&pool_kernel<Walk2D32<FD, R>, R, true>) : K(&pool_kernel<Walk2D32<FD, R>, R, false>);
}
}  // namespace

const void *kernel_2d32(bool fd, bool tape, bool one, bool tab) {
  if (one) return fd ? K(&pool_kernel<Walk2D32<true, PhiloxOne>, PhiloxOne, false>)
                     : K(&pool_kernel<Walk2D32<false, PhiloxOne>, PhiloxOne, false>);
  if (tape) return fd ? per_job<true, TapeRng>(tab) : per_job<false, TapeRng>(tab);
  return fd ? per_job<true, PhiloxRng>(tab) : per_job<false, PhiloxRng>(tab);
}

}  // namespace vmc
