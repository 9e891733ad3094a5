"""The serving loop's epoch rules (valomc_gb300/csrc/epoch_plan.hpp) on the CPU: the header is
compiled with g++ into a small driver, which the tests feed cases and whose answers they check
against the rules as the header states them."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "valomc_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <iostream>
#include <string>
#include "epoch_plan.hpp"
int main() {
  std::string op;
  while (std::cin >> op) {
    if (op == "E") {
      long long fixed, backlog; double rate; int max_ms;
      std::cin >> fixed >> rate >> max_ms >> backlog;
      std::printf("%lld\n", (long long)vmc::epoch_photons(fixed, rate, max_ms, backlog));
    } else {
      int sf; long long epoch; size_t n;
      std::cin >> sf >> epoch >> n;
      std::vector<int64_t> left(n);
      for (auto &x : left) { long long v; std::cin >> v; x = v; }
      for (int64_t s : vmc::epoch_slices(left, epoch, sf != 0)) std::printf("%lld ", (long long)s);
      std::printf("\n");
    }
  }
}
"""


@pytest.fixture(scope="module")
def driver():
    with tempfile.TemporaryDirectory() as td:
        src, exe = os.path.join(td, "plan.cpp"), os.path.join(td, "plan")
        with open(src, "w") as fp:
            fp.write(DRIVER)
        subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", CSRC, src, "-o", exe],
                       check=True, capture_output=True, text=True)

        def run(lines):
            out = subprocess.run([exe], input="\n".join(lines) + "\n", check=True, capture_output=True,
                                 text=True, timeout=60).stdout.splitlines()
            return out
        yield run


def epoch(driver, fixed, rate, max_ms, backlog):
    return int(driver([f"E {fixed} {rate} {max_ms} {backlog}"])[0])


def slices(driver, shortest_first, ep, left):
    return [int(x) for x in driver([f"S {int(shortest_first)} {ep} {len(left)} " + " ".join(map(str, left))])[0].split()]


def test_epoch_size_follows_the_load(driver):
    rate = 1.3e8
    assert epoch(driver, 7000, rate, 0, 10**9) == 7000                       # fixed size as given
    assert epoch(driver, 0, rate, 0, 10**5) == int(rate * 0.05)              # small backlog: 50 ms of work
    assert epoch(driver, 0, rate, 0, 3 * 10**7) == 3 * 10**7                 # the backlog, when between
    assert epoch(driver, 0, rate, 0, 10**10) == int(rate * 0.5)              # capped at 0.5 s of work
    assert epoch(driver, 0, rate, 150, 10**10) == int(rate * 0.15)           # epoch_max_ms
    assert epoch(driver, 0, 0.0, 0, 10) == 200000                            # no rate yet: 2e5 photons


@pytest.mark.parametrize("shortest_first", [True, False])
@pytest.mark.parametrize("case", [
    (10**7, [10**5, 3 * 10**6, 10**7, 2 * 10**5]),
    (10**6, [10**5, 3 * 10**6, 10**7, 2 * 10**5]),
    (5, [7, 9, 11]),
    (10**6, [500]),
    (10**8, [10**5, 10**6]),
])
def test_slices_stay_within_the_requests_and_fill_the_epoch(driver, shortest_first, case):
    ep, left = case
    s = slices(driver, shortest_first, ep, left)
    assert len(s) == len(left)
    assert all(1 <= x <= l for x, l in zip(s, left))                         # none starves, none overdrawn
    if sum(left) <= ep:
        assert s == left                                                     # everything fits: all of it
    else:
        floor = max(1, ep // (4 * len(left))) if shortest_first else 1
        assert sum(s) <= max(ep, floor * len(left))
        assert sum(s) >= min(ep, sum(left)) - len(left)                      # the epoch is filled


def test_shortest_first_finishes_small_requests(driver):
    left = [10**7, 10**5, 3 * 10**6, 2 * 10**5]
    ep = 10**6
    s = slices(driver, True, ep, left)
    floor = ep // (4 * len(left))                                            # 62500
    assert s[1] == 10**5 and s[3] == 2 * 10**5                               # the two small ones finish
    assert s[0] == floor                                                     # the largest gets its floor
    assert s[2] == ep - 10**5 - 2 * 10**5 - floor                            # the next smallest the rest
    assert sum(s) == ep


def test_water_filling_splits_the_rest_equally(driver):
    left = [10**7, 10**5, 3 * 10**6, 2 * 10**5]
    ep = 10**6
    s = slices(driver, False, ep, left)
    assert s[1] == 10**5 and s[3] == 2 * 10**5                               # below an equal share: all
    share = (ep - 3 * 10**5) // 2
    assert s[0] == share and s[2] == share                                   # the others split the rest


def test_equal_requests_keep_their_order(driver):
    s = slices(driver, True, 10, [100, 100, 100])
    assert s == [8, 1, 1]                                                    # floor 1 each, the rest to the first
