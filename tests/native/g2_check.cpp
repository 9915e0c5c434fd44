// Replays the reference's G2 known answers (g2_kats.txt) through the
// library's host G2 arithmetic (host_pairing.hpp): for every g2_ops line
// P + Q, 2P, kP and -P; every g2_reject encoding refused; the generator's
// bytes accepted and written back unchanged. Prints "<ops> <rejects> <gen>"
// counts of agreeing lines and exits non-zero on any disagreement.
#include <cstdio>
#include <cstring>
#include <string>

#include "host_pairing.hpp"

using namespace apg::host::pairing;

static int hexval(char c) { return c <= '9' ? c - '0' : c - 'a' + 10; }
static bool unhex(const char* h, uint8_t* out, size_t n) {
  if (strlen(h) != 2 * n) return false;
  for (size_t i = 0; i < n; ++i) out[i] = (uint8_t)(hexval(h[2 * i]) * 16 + hexval(h[2 * i + 1]));
  return true;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* f = fopen(argv[1], "r");
  if (!f) return 2;
  static char line[1 << 14];
  int ops = 0, rejects = 0, gens = 0, bad = 0;
  while (fgets(line, sizeof line, f)) {
    char a[7][300];
    if (!strncmp(line, "g2_ops ", 7)) {
      if (sscanf(line + 7, "%299s %299s %299s %299s %299s %299s %299s", a[0], a[1], a[2], a[3], a[4], a[5], a[6]) != 7)
        return 2;
      uint8_t p[128], q[128], k[32], want[4][128], got[128];
      bool ok = unhex(a[0], p, 128) && unhex(a[1], q, 128) && unhex(a[2], k, 32);
      for (int i = 0; i < 4; ++i) ok = ok && unhex(a[3 + i], want[i], 128);
      G2 P, Qp;
      ok = ok && g2from_bytes(p, P) && g2from_bytes(q, Qp);
      Big kb(4);
      memcpy(kb.data(), k, 32);
      big_trim(kb);
      const G2 res[4] = {g2add(P, Qp), g2add(P, P), g2mul(P, kb), g2neg(P)};
      for (int i = 0; ok && i < 4; ++i) {
        g2to_bytes(res[i], got);
        ok = memcmp(got, want[i], 128) == 0;
      }
      ok ? ++ops : ++bad;
    } else if (!strncmp(line, "g2_reject ", 10)) {
      uint8_t p[128];
      G2 P;
      if (sscanf(line + 10, "%299s", a[0]) != 1 || !unhex(a[0], p, 128)) return 2;
      g2from_bytes(p, P) ? ++bad : ++rejects;
    } else if (!strncmp(line, "g2_generator ", 13)) {
      uint8_t p[128], back[128];
      G2 P;
      if (sscanf(line + 13, "%299s", a[0]) != 1 || !unhex(a[0], p, 128)) return 2;
      bool ok = g2from_bytes(p, P);
      if (ok) {
        g2to_bytes(P, back);
        ok = memcmp(back, p, 128) == 0;
      }
      ok ? ++gens : ++bad;
    }
  }
  printf("%d %d %d\n", ops, rejects, gens);
  return bad ? 1 : 0;
}
