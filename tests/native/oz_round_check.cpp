// Host driver for the CPU test of slepc_gb300/csrc/oz_round.h: reads "x H R sc" (round X 2^sc, X = H 2^42 + R) or
// "f BITS" (the integer of an integer-valued float given by its bits) per line, prints the result per line.
#include <cinttypes>
#include <cstdio>
#include <cstring>

#include "../../slepc_gb300/csrc/oz_round.h"

int main() {
  char op[4];
  while (std::scanf("%3s", op) == 1) {
    if (op[0] == 'x') {
      long long H, R;
      int sc;
      if (std::scanf("%lld %lld %d", &H, &R, &sc) != 3) return 1;
      double d = 0.0;
      const bool ok = oz_round_x(H, R, sc, &d);
      uint64_t b;
      std::memcpy(&b, &d, 8);
      std::printf("%d %016" PRIx64 "\n", ok ? 1 : 0, b);
    } else {
      unsigned u;
      if (std::scanf("%x", &u) != 1) return 1;
      float f;
      std::memcpy(&f, &u, 4);
      std::printf("%d\n", (int)oz_f2i_exact(f));
    }
  }
  return 0;
}
