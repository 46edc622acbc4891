// Neighbour slot codes on the host: every lattice translation T within +-4096 cells per axis
// survives pack_code -> code_t_full given any floor difference within +-200 cells of T (the
// rounding of Cell::diff and the image shell move T by a few cells at most), the
// minimum-image bit is independent of the translation, and code_t alone is exact for |T| < 512.
#include <cstdio>

#include "common.cuh"

using namespace nnpgpu;

int main() {
  long long checked = 0;
  for (int t = -4096; t <= 4096; ++t)
    for (int r = -200; r <= 200; r += 7)
      for (int mn = 0; mn < 2; ++mn) {
        const int c = pack_code(t, -t, t / 3, mn != 0);
        if (code_min(c) != (mn != 0)) { std::printf("min bit t=%d\n", t); return 1; }
        const int got[3] = {code_t_full(c, 0, t + r), code_t_full(c, 1, -t + r), code_t_full(c, 2, t / 3 - r)};
        if (got[0] != t || got[1] != -t || got[2] != t / 3) {
          std::printf("t=%d r=%d: %d %d %d\n", t, r, got[0], got[1], got[2]);
          return 1;
        }
        if (t >= -512 && t < 512 && (code_t(c, 0) != t || code_t(c, 1) != (-t == 512 ? -512 : -t))) {
          std::printf("code_t t=%d\n", t);
          return 1;
        }
        ++checked;
      }
  std::printf("ok %lld\n", checked);
  return 0;
}
