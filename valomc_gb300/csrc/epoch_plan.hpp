// epoch_plan.hpp -- the serving loop's rules for the size of an epoch and its slices (host
// code, no CUDA), apart from the loop so that they are tested on the CPU.
#pragma once
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

namespace vmc {

// Photons in the next epoch.  `fixed` > 0 is taken as it is.  Otherwise the size follows the
// load: at least 50 ms of work at the measured rate (and 2e5 photons) while the backlog is
// small, for latency; up to the backlog and at most max_ms of work (0: 500 ms) as it grows,
// since every launch ends in a drain and larger epochs pay it less often.
inline int64_t epoch_photons(int64_t fixed, double rate, int32_t max_ms, int64_t backlog) {
  if (fixed > 0) return fixed;
  const double max_s = (max_ms > 0 ? max_ms : 500) * 1e-3;
  const int64_t lo = std::max<int64_t>(200000, (int64_t)(rate * 0.05));
  const int64_t hi = std::max<int64_t>(lo, (int64_t)(rate * max_s));
  return std::min(hi, std::max(lo, backlog));
}

// Slices of one epoch over the open requests, left[i] > 0 photons of request i not yet
// issued; slice i is at most left[i].
//
// Shortest remaining first: every request gets a floor of a quarter of an equal share (at
// least 1 photon), so none starves, and the rest of the epoch goes to the requests with the
// fewest photons left, in that order, so that small and medium requests finish within one
// epoch instead of sharing it equally with the largest.
//
// Water-filling: a request with fewer photons left than an equal share of what remains gets
// all of them, and the others split the rest equally (at least 1 photon each).
//
// Both fill the epoch as far as the open requests allow: equal shares left the small
// requests' unused share idle (underfilled epochs, a lower measured rate and smaller epochs
// after them).  Requests with equal photon counts keep their order.
inline std::vector<int64_t> epoch_slices(const std::vector<int64_t> &left, int64_t epoch, bool shortest_first) {
  const size_t n = left.size();
  std::vector<int64_t> slice(n, 0);
  if (n == 0) return slice;
  std::vector<size_t> order(n);
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return left[a] < left[b]; });
  int64_t rest = epoch;
  if (shortest_first) {
    const int64_t floor_share = std::max<int64_t>(1, epoch / (4 * (int64_t)n));
    for (size_t i : order) {
      slice[i] = std::min(floor_share, left[i]);
      rest -= slice[i];
    }
    for (size_t i : order) {
      if (rest <= 0) break;
      const int64_t extra = std::min(rest, left[i] - slice[i]);
      slice[i] += extra;
      rest -= extra;
    }
  } else {
    size_t k = 0;
    for (; k < n; k++) {
      const size_t i = order[k];
      const int64_t s = rest / (int64_t)(n - k);
      if (left[i] > s) break;
      slice[i] = left[i];
      rest -= slice[i];
    }
    const int64_t s = k < n ? std::max<int64_t>(1, rest / (int64_t)(n - k)) : 0;
    for (; k < n; k++) slice[order[k]] = std::min(s, left[order[k]]);
  }
  return slice;
}

}  // namespace vmc
