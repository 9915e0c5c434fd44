// The library's host G1 sum (msm_small in host_g1.hpp, compiled here as it is
// in the library) over cases read from standard input: a line "n", then n
// lines of a 64-byte point and a 32-byte canonical scalar in hex; prints the
// 64-byte result in hex, one line a case.
#include <cstdio>
#include <string>
#include <vector>

#include "host_g1.hpp"

using namespace apg::host;

static bool unhex(const char* s, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    unsigned v;
    if (sscanf(s + 2 * i, "%2x", &v) != 1) return false;
    out[i] = (uint8_t)v;
  }
  return true;
}

int main() {
  size_t n;
  while (scanf("%zu", &n) == 1) {
    std::vector<uint8_t> pts(64 * n);
    std::vector<F> ks(n);
    char p[129], k[65];
    for (size_t j = 0; j < n; ++j) {
      if (scanf("%128s %64s", p, k) != 2 || !unhex(p, &pts[64 * j], 64)) return 2;
      uint8_t kb[32];
      if (!unhex(k, kb, 32) || !from_bytes(kb, ks[j])) return 3;
    }
    uint8_t out[64];
    g1::msm_small(pts.data(), ks.data(), n, out);
    for (int i = 0; i < 64; ++i) printf("%02x", out[i]);
    printf("\n");
  }
  return 0;
}
