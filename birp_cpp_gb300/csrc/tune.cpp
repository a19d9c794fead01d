// Tile-shape choice (lanes per ray, warp-block width, warps across a tile)
// from the committed tuning tables (tune_table.inc): one for a request
// rendered alone, one for a request inside a batch (where other requests
// already fill the GPU).
#include <cstdint>

#include "birp_host.h"

namespace birp {

struct TuneRow {
  int64_t max_pixels;
  int max_samples;
  int kind;
  int trilinear;
  int seg_log2;
  int wbx_l2;  // -1: the default warp-block width for seg_log2
  int wgx_l2;  // -1: 2 warps across the tile
};

#include "tune_table.inc"

TunedShape tuned_shape(int64_t pixels, int n_samples, int kind, int trilinear, bool batched) {
  const TuneRow* rows = batched ? kTuneRowsBatch : kTuneRowsPlain;
  const size_t n = batched ? sizeof(kTuneRowsBatch) / sizeof(TuneRow) : sizeof(kTuneRowsPlain) / sizeof(TuneRow);
  for (size_t i = 0; i < n; ++i) {
    const TuneRow& r = rows[i];
    if (pixels > r.max_pixels || n_samples > r.max_samples) continue;
    if (r.kind >= 0 && r.kind != kind) continue;
    if (r.trilinear >= 0 && r.trilinear != (trilinear ? 1 : 0)) continue;
    return {r.seg_log2, r.wbx_l2, r.wgx_l2};
  }
  return {0, -1, -1};
}

}  // namespace birp
