// Lookup into the committed autotune table (tune_table.inc, written by the
// package's autotune.py from timings on a GB300).  Each row gives the best
// fused-kernel tile shape measured for a (mode, kernel size, channels) key and
// an image-size class; sizes between measured classes use the nearest class
// at or below the request.
#pragma once

#include <stdint.h>

namespace kcv {

struct TuneRow {
  int mode, ksize, channels;
  long min_row_bytes;  // source bytes per row at or above which the row applies
  int min_rows;        // destination rows at or above which the row applies
  int threads, tile_rows, stage_rows, stages;
};

static const TuneRow kTuneTable[] = {
#include "tune_table.inc"
    {-1, 0, 0, 0, 0, 0, 0, 0, 0}};

inline bool lookup_tile_shape(int mode, int ksize, int channels, long row_bytes, int rows,
                              int *threads, int *tile_rows, int *stage_rows, int *stages) {
  const TuneRow *best = nullptr;
  for (const TuneRow &r : kTuneTable) {
    if (r.mode != mode || r.ksize != ksize || r.channels != channels) continue;
    if (row_bytes < r.min_row_bytes || rows < r.min_rows) continue;
    if (!best || r.min_row_bytes > best->min_row_bytes ||
        (r.min_row_bytes == best->min_row_bytes && r.min_rows > best->min_rows))
      best = &r;
  }
  if (!best) return false;
  *threads = best->threads;
  *tile_rows = best->tile_rows;
  *stage_rows = best->stage_rows;
  *stages = best->stages;
  return true;
}

}  // namespace kcv
