// Host check of the cell-record index arithmetic the kernels use
// (birp_cpp_gb300/csrc/cell_index.h): every cell -1..n-1 maps inside the
// record array, the map is the build kernel's enumeration order, and a walk
// of unit steps stays inside. Exit code = number of failures.
#include <cstdio>
#include <random>

#include "../../birp_cpp_gb300/csrc/cell_index.h"

using namespace birp;

int main() {
  int fails = 0;
  const int dims[][3] = {{2, 2, 2}, {3, 5, 7}, {64, 64, 64}, {96, 320, 144}, {256, 256, 256}, {513, 385, 385}};
  for (auto& d : dims) {
    const int nx = d[0], ny = d[1], nz = d[2];
    const long long cx = nx + 1, cxy = (long long)(nx + 1) * (ny + 1), cnt = record_count(nx, ny, nz);
    // enumeration order of the record build: r = c*cxy + b*cx + a, cell = (a-1, b-1, c-1)
    if (nx * ny * nz <= 64 * 64 * 64) {
      long long r = 0;
      for (int c = 0; c <= nz; ++c)
        for (int b = 0; b <= ny; ++b)
          for (int a = 0; a <= nx; ++a, ++r)
            if (record_index(cx, cxy, a - 1, b - 1, c - 1) != r) ++fails;
      if (r != cnt) ++fails;
    }
    // extreme cells are inside
    const int ks[] = {-1, 0};
    for (int kx : {-1, 0, nx - 2, nx - 1})
      for (int ky : {-1, 0, ny - 2, ny - 1})
        for (int kz : {-1, 0, nz - 2, nz - 1}) {
          long long i = record_index(cx, cxy, kx, ky, kz);
          if (i < 0 || i >= cnt) ++fails;
        }
    (void)ks;
    // random walks: start in [0, n-2], unit steps confined to [-1, n-1]
    std::mt19937 rng(7 + nx);
    for (int w = 0; w < 200; ++w) {
      int k[3] = {(int)(rng() % (nx - 1)), (int)(rng() % (ny - 1)), (int)(rng() % (nz - 1))};
      const int n[3] = {nx, ny, nz};
      long long q = 2 * record_index(cx, cxy, k[0], k[1], k[2]);  // float4 index
      for (int s = 0; s < 2000; ++s) {
        int a = rng() % 3, dir = (rng() & 1) ? 1 : -1;
        if (k[a] + dir < -1 || k[a] + dir > n[a] - 1) continue;  // sentinel stops the walk
        k[a] += dir;
        q += 2 * dir * record_stride(cx, cxy, a);
        if (q != 2 * record_index(cx, cxy, k[0], k[1], k[2])) ++fails;
        if (q < 0 || q + 1 >= 2 * cnt) ++fails;
      }
    }
  }
  std::printf("%d failures\n", fails);
  return fails;
}
