// The library's field inversion (inverse_divsteps in field.cuh, the device
// code compiled for the host) against a slow shift-and-add modular product:
// x must satisfy a x = 1 mod m and 0 <= x < m, for random inputs of both
// fields and edge values (small, powers of two, m - 1, m - 2).
#include <cstdio>
#include <random>
#include "field.cuh"
using namespace apg;
typedef unsigned __int128 u128;
static void mulmod(const uint32_t a[8], const uint32_t b[8], const uint32_t m[8], uint32_t out[8]) {
  // schoolbook then reduce by shift-subtract (slow, test only)
  uint64_t acc[5] = {0};
  uint64_t M[5] = {0}, B[5] = {0};
  for (int i = 0; i < 8; ++i) { M[i / 2] |= (uint64_t)m[i] << (32 * (i % 2)); B[i / 2] |= (uint64_t)b[i] << (32 * (i % 2)); }
  auto ge = [](const uint64_t* x, const uint64_t* y) { for (int k = 4; k >= 0; --k) if (x[k] != y[k]) return x[k] > y[k]; return true; };
  auto add = [](uint64_t* x, const uint64_t* y) { u128 c = 0; for (int k = 0; k < 5; ++k) { u128 t = (u128)x[k] + y[k] + c; x[k] = (uint64_t)t; c = t >> 64; } };
  auto sub = [](uint64_t* x, const uint64_t* y) { uint64_t br = 0; for (int k = 0; k < 5; ++k) { u128 t = (u128)x[k] - y[k] - br; x[k] = (uint64_t)t; br = (uint64_t)(t >> 127) & 1; } };
  for (int bit = 255; bit >= 0; --bit) {
    add(acc, acc); while (ge(acc, M)) sub(acc, M);
    if ((a[bit / 32] >> (bit % 32)) & 1) { add(acc, B); while (ge(acc, M)) sub(acc, M); }
  }
  for (int i = 0; i < 8; ++i) out[i] = (uint32_t)(acc[i / 2] >> (32 * (i % 2)));
}
int main() {
  const uint32_t FR[8] = {FrConsts::P0, FrConsts::P1, FrConsts::P2, FrConsts::P3, FrConsts::P4, FrConsts::P5, FrConsts::P6, FrConsts::P7};
  const uint32_t FQ[8] = {FqConsts::P0, FqConsts::P1, FqConsts::P2, FqConsts::P3, FqConsts::P4, FqConsts::P5, FqConsts::P6, FqConsts::P7};
  std::mt19937_64 rng(11);
  int bad = 0, n = 0;
  for (int which = 0; which < 2; ++which) {
    const uint32_t* m = which ? FQ : FR;
    for (int t = 0; t < 20000; ++t) {
      uint32_t a[8];
      for (int i = 0; i < 8; ++i) a[i] = (uint32_t)rng();
      a[7] &= 0x3fffffff;
      if (t < 40) { for (int i = 0; i < 8; ++i) a[i] = 0; a[0] = t + 1; if (t >= 20) a[t % 8] = 1u << (t % 31); }
      if (t == 40) { for (int i = 0; i < 8; ++i) a[i] = m[i]; a[0] -= 1; }
      if (t == 41) { for (int i = 0; i < 8; ++i) a[i] = m[i]; a[0] -= 2; }
      bool g = true; for (int i = 7; i >= 0; --i) if (a[i] != m[i]) { g = a[i] > m[i]; break; }
      if (g) { int64_t b = 0; for (int i = 0; i < 8; ++i) { b += (int64_t)a[i] - m[i]; a[i] = (uint32_t)b; b >>= 32; } }
      bool z = true; for (int i = 0; i < 8; ++i) z &= a[i] == 0; if (z) continue;
      uint32_t x[8], one[8];
      bool ok = inverse_divsteps(a, m, x);
      mulmod(a, x, m, one);
      bool isone = one[0] == 1; for (int i = 1; i < 8; ++i) isone &= one[i] == 0;
      bool below = false; for (int i = 7; i >= 0; --i) if (x[i] != m[i]) { below = x[i] < m[i]; break; }
      ++n;
      if (!ok || !isone || !below) { if (bad < 5) printf("bad: field %d t %d ok %d one %d below %d\n", which, t, ok, isone, below); ++bad; }
    }
  }
  printf("%d inverses, %d bad\n", n, bad);
  return bad != 0;
}
