// Error reporting and the glibc-compatible rand() stream.
#include "internal.h"
#include <cstdio>

namespace rayt {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return RAYT_E_CUDA;
}

// Seeding: r[0] = seed (0 becomes 1), r[i] = 16807 * r[i-1] mod (2^31 - 1)
// by Schrage's method for i = 1..30, r[31..33] = r[0..2]; every later term is
// r[i] = r[i-3] + r[i-31] (mod 2^32) and the output is that term shifted right
// by one; the terms for i = 34..343 are discarded.
void LibcRand::Seed(uint32_t seed) {
  int32_t r[34];
  r[0] = (int32_t)(seed == 0 ? 1u : seed);
  for (int i = 1; i < 31; ++i) {
    int32_t hi = r[i - 1] / 127773;
    int32_t lo = r[i - 1] % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = word;
  }
  for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
  for (int i = 0; i < 34; ++i) r_[i] = r[i];
  i_ = 34;
  for (int k = 34; k < 344; ++k) Next();
}

int LibcRand::Next() {
  // ring of the last 34 terms, r_[k % 34] holds term k
  uint32_t v = (uint32_t)r_[(i_ - 31) % 34] + (uint32_t)r_[(i_ - 3) % 34];
  r_[i_ % 34] = (int32_t)v;
  ++i_;
  if (i_ >= 34 * 1000000) i_ -= 34 * 999999;  // keep the index bounded, same residues
  return (int)(v >> 1);
}

}  // namespace rayt

extern "C" {
const char* rayt_last_error(void) { return rayt::g_last_error.c_str(); }
const char* rayt_version(void) { return "rayt_gb300 0.1 (sm_103a)"; }
}

namespace rayt {

size_t pixel_coords_count(int w, int h) { return (size_t)w + (w + 1) + h + (h + 1); }

void pixel_coords(int w, int h, float* out) {
  const float W = (float)w, H = (float)h;
  for (int x = 0; x < w; ++x) *out++ = (x + 0.5f) / W * 2 - 1;
  for (int x = 0; x <= w; ++x) *out++ = (float)x / W * 2 - 1;
  for (int y = 0; y < h; ++y) *out++ = (y + 0.5f) / H * 2 - 1;
  for (int y = 0; y <= h; ++y) *out++ = (float)y / H * 2 - 1;
}

void view_origin(const float* m, float* origin) {
  origin[0] = m[2] / m[14];
  origin[1] = m[6] / m[14];
  origin[2] = m[10] / m[14];
  origin[3] = 0.0f / m[14];
}

}  // namespace rayt
