// Index arithmetic of the cell-record layout (birp_internal.h), shared by the
// kernels and checked on the host by tests/cpp/cell_index_test.cpp.
//
// Cells -1..n-1 per axis; record (kx, ky, kz) is at
// ((kz+1) * cxy + (ky+1) * cx + (kx+1)) with cx = nx+1, cxy = (nx+1)(ny+1),
// i.e. in [0, (nx+1)(ny+1)(nz+1)) for every cell in range. A record is two
// float4, so its first float4 is at 2 * record index.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define BIRP_HD __host__ __device__ __forceinline__
#else
#define BIRP_HD inline
#endif

namespace birp {

BIRP_HD long long record_index(long long cx, long long cxy, int kx, int ky, int kz) {
  return (long long)(kz + 1) * cxy + (long long)(ky + 1) * cx + (kx + 1);
}

// Records between neighbouring cells along axis a (0, 1, 2).
BIRP_HD long long record_stride(long long cx, long long cxy, int a) { return a == 0 ? 1 : (a == 1 ? cx : cxy); }

BIRP_HD long long record_count(int nx, int ny, int nz) {
  return ((long long)nx + 1) * ((long long)ny + 1) * ((long long)nz + 1);
}

}  // namespace birp
