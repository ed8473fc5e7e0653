// Adaptive shape of the serving kernel, host side: the arrival-rate estimate
// and the shape a launch of the persistent kernel takes
// (sigops_server_set_adaptive).  Plain C++ with no CUDA, so the CPU tests
// drive the same code with simulated arrivals.
#pragma once
#include <stdint.h>

namespace sg {

struct ShapePolicy {
  // 10 ms samples averaged with weight 1/4: a step reaches two thirds of its
  // height in about 40 ms (a low shape under overload builds a backlog
  // meanwhile), and the scatter of single samples (about 7% at half load, with
  // requests of 1..2048 items) is averaged down to about 3%.  The same weight
  // serves rises and falls: a faster rise would follow the samples' upward
  // scatter and sit above the mean.
  static constexpr double kSampleS = 0.01;
  static constexpr double kWeight = 0.25;
  static constexpr double kDownFraction = 0.8;  // back to the low shape below this share of the switch rate

  int low = 0, high = 0;
  double switch_rate = 0;   // items/s; 0 = no adaptive choice
  double rate = 0;          // arrival-rate estimate, items/s
  double sample_t = 0;      // time of the last sample (s; 0 = none yet)
  uint64_t sample_items = 0;  // items accepted up to that sample

  // t: now (s); items_in: items accepted so far.  Called as often as liked;
  // takes a sample every kSampleS.
  void observe(double t, uint64_t items_in) {
    if (t - sample_t < kSampleS) return;
    const double inst = sample_t > 0 ? (double)(items_in - sample_items) / (t - sample_t) : 0.0;
    rate += kWeight * (inst - rate);
    sample_t = t;
    sample_items = items_in;
  }

  // the shape the next launch takes: `fixed` without an adaptive choice, and
  // `running` while the rate lies between the two thresholds
  int wanted(int fixed, int running) const {
    if (switch_rate <= 0) return fixed;
    if (rate >= switch_rate) return high;
    if (rate < kDownFraction * switch_rate) return low;
    return running;
  }
};

}  // namespace sg
