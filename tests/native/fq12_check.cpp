// Replays the reference's Fq12 known answers (fq12_kats.txt) through the
// library's host tower (host_pairing.hpp): for every fq12_ops line a + b,
// a - b, a b, a^2, 1/a (or "none" for a = 0), the conjugate and a^q, a^(q^2),
// a^(q^3) (as plain powers); for every fq12_final_exp line the exact final
// exponent (q^12 - 1)/r. Prints "<ops> <final_exp>" agreeing counts and
// exits non-zero on any disagreement.
#include <cstdio>
#include <cstring>

#include "host_pairing.hpp"

using namespace apg::host::pairing;

static int hexval(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }

static bool read12(const char* h, F12& out) {
  if (strlen(h) != 768) return false;
  uint8_t b[384];
  for (int i = 0; i < 384; ++i) b[i] = (uint8_t)(hexval(h[2 * i]) * 16 + hexval(h[2 * i + 1]));
  F6* halves[2] = {&out.c0, &out.c1};
  for (int i = 0; i < 2; ++i) {
    F2* t[3] = {&halves[i]->c0, &halves[i]->c1, &halves[i]->c2};
    for (int j = 0; j < 3; ++j) {
      uint64_t w0[4], w1[4];
      memcpy(w0, b + 192 * i + 64 * j, 32);
      memcpy(w1, b + 192 * i + 64 * j + 32, 32);
      if (apg::host::g1::QConsts::geq_q(w0) || apg::host::g1::QConsts::geq_q(w1)) return false;
      t[j]->c0 = apg::host::g1::q_from_canonical(w0);
      t[j]->c1 = apg::host::g1::q_from_canonical(w1);
    }
  }
  return true;
}

static bool zero12(const F12& a) { return f12eq(a, F12{f6zero(), f6zero()}); }

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* f = fopen(argv[1], "r");
  if (!f) return 2;
  static char line[1 << 14];
  static char tok[12][800];
  int ops = 0, fexp = 0, bad = 0;
  const Big& q = pc().q;
  const Big q2 = big_mul(q, q), q3 = big_mul(q2, q);
  while (fgets(line, sizeof line, f)) {
    if (!strncmp(line, "fq12_ops ", 9)) {
      if (sscanf(line + 9, "%799s %799s %799s %799s %799s %799s %799s %799s %799s %799s %799s", tok[0], tok[1], tok[2],
                 tok[3], tok[4], tok[5], tok[6], tok[7], tok[8], tok[9], tok[10]) != 11)
        return 2;
      F12 a, b, w[9];
      bool ok = read12(tok[0], a) && read12(tok[1], b);
      const bool no_inv = !strcmp(tok[6], "none");
      for (int i = 0; ok && i < 9; ++i) ok = (i == 4 && no_inv) || read12(tok[2 + i], w[i]);
      if (ok) {
        const F12 sum{f6add(a.c0, b.c0), f6add(a.c1, b.c1)}, diff{f6sub(a.c0, b.c0), f6sub(a.c1, b.c1)};
        ok = f12eq(sum, w[0]) && f12eq(diff, w[1]) && f12eq(f12mul(a, b), w[2]) && f12eq(f12sqr(a), w[3]) &&
             (no_inv ? zero12(a) : f12eq(f12inv(a), w[4])) && f12eq(F12{a.c0, f6neg(a.c1)}, w[5]) &&
             f12eq(f12pow(a, q), w[6]) && f12eq(f12pow(a, q2), w[7]) && f12eq(f12pow(a, q3), w[8]);
      }
      ok ? ++ops : ++bad;
    } else if (!strncmp(line, "fq12_final_exp ", 15)) {
      if (sscanf(line + 15, "%799s %799s", tok[0], tok[1]) != 2) return 2;
      F12 a, want;
      const bool ok = read12(tok[0], a) && read12(tok[1], want) && f12eq(final_exponentiation(a), want);
      ok ? ++fexp : ++bad;
    }
  }
  printf("%d %d\n", ops, fexp);
  return bad ? 1 : 0;
}
