// Host half of the reference's RayTracingFeedbackExtractor
// (rayt/GPU_renderer/ray-tracing-feedback-extractor.cpp:100-185): decoding a
// pass's sorted unique feedback array into fault blocks and (duplicate) hit
// blocks, shared by the per-frame renderer and the server.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace rayt {

class FeedbackDecoder {
 public:
  std::vector<int> faults;    // tree block IDs, in the array's order (descending)
  std::vector<int> hits;      // cache blocks hit
  std::vector<int> dup_hits;  // cache blocks hit through a duplicated node

  // ProcessUnique + AdjustExpectedFaults (:108-185): every fault, read in
  // chunks that double from expected_faults (ending with the chunk that
  // reaches the first non-fault), then a window of at most 4000 hits starting
  // at rand() % (hits left), wrapping around.
  void Decode(const int32_t* u, int count, LibcRand& rand) {
    faults.clear();
    hits.clear();
    dup_hits.clear();
    auto add_hit = [this](int32_t v) {
      if (v & 1) dup_hits.push_back((v >> 1) - 1);
      else hits.push_back((v >> 1) - 1);
    };
    int stride = expected_faults_, size = 0;
    while (size < count && (size == 0 || u[size - 1] < 0)) {
      stride = std::min(stride, count - size);
      for (int i = size; i < size + stride; ++i) {
        if (u[i] < 0) faults.push_back(-u[i] - 1);
        else if (u[i] != kNoHit) add_hit(u[i]);
      }
      size += stride;
      stride *= 2;
    }
    if (size < count) {
      const int len = count - size;
      const int start = rand.Next() % len;
      const int take = std::min(kHitsToExtract, len);
      int seg[2][2];
      int nseg = 0;
      if (start + take <= len) {
        seg[nseg][0] = start, seg[nseg][1] = take, ++nseg;
      } else {
        seg[nseg][0] = 0, seg[nseg][1] = start + take - len, ++nseg;
        seg[nseg][0] = start, seg[nseg][1] = len - start, ++nseg;
      }
      for (int k = 0; k < nseg; ++k)
        for (int i = 0; i < seg[k][1]; ++i) {
          const int32_t v = u[size + seg[k][0] + i];
          if (v != kNoHit) add_hit(v);
        }
    }
    if (expected_faults_ > 1 && (int)faults.size() < expected_faults_) expected_faults_ /= 2;
    else if ((int)faults.size() > expected_faults_) expected_faults_ *= 2;
  }

 private:
  static constexpr int kHitsToExtract = 4000;  // ray-tracing-feedback-extractor.cpp:22-23
  int expected_faults_ = 1 << 16;
};

}  // namespace rayt
