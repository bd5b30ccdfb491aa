// sg_fused2d_host.h -- host entry points of the fused Nin = 2 path (sg_fused2d.cu).
#pragma once

#include <vector>

#include "sg_fused2d.cuh"

namespace sg {

// Uniform tilings of one grid.  slots > 0: the grid runs alone (one launch over its
// units, `slots` of them resident at once): the block counts minimize
// waves x (unit + set-up).  slots = 0 (the batch, many grids): units of about `target`
// values of eval (forward) or of the cotangent (adjoint; target <= 0: the whole axis 1
// per tile).  Adjoint tiles span axis 0 whole when its samples x the tile's channels fit
// `np` pairs, else chunks of axis-0 control points with one channel each (rows of
// `align`-element multiples).  False when the grid does not fit the fused path.
bool f2_forward_tiling(int64_t ns0, int64_t ns1, int nch, int64_t target, int slots, F2Tiling &t);
// Forward tiles (sorted axis-1 samples, lb1: its support table): 128 samples x a block
// of rows whose columns span at most `cols` (kF2TileCols of the value type).
bool f2_forward_tile_tiling(const int32_t *lb1, int64_t n1, int d1, int64_t ns0, int64_t ns1, int nch,
                            int cols, int64_t target, int slots, F2Tiling &t);
// First axis-1 column and column count of the forward tile over rows [b_lo, b_lo + b_len)
// of a sorted axis (lb1: its support table).
void f2_tile_columns(const int32_t *lb1, int64_t n1, int d1, int64_t b_lo, int64_t b_len, int32_t &cb,
                     int32_t &ncol);
// Columns of a forward tile's intermediate for the value type.
inline int f2_tile_cols(int dtype) { return dtype == SG_F64 ? kF2TileCols<double>() : kF2TileCols<float>(); }
bool f2_adjoint_tiling(const int32_t *lb0, int64_t n0, int d0, int64_t ns0, int64_t n1, int d1,
                       int64_t ns1, int nch, int np, int align, int64_t target, int slots, F2Tiling &t);

// Values of the type per 16 bytes (the row alignment chunked adjoint tiles need).
inline int f2_align_elems(int dtype) { return dtype == SG_F64 ? 2 : 4; }

// Batch unit sizes: forward warp tasks of about this many eval values; adjoint tiles
// span axis 1 whole (no cotangent row is read twice).
constexpr int64_t kF2BatchFwdTarget = 1 << 14;
constexpr int64_t kF2BatchAdjTarget = 0;

// Resident forward warp tasks (kind 0) / adjoint CTAs (kind 1) / forward tile CTAs
// (kind 2) on the current device.
int f2_slots(int dtype, int kind);

// (sample, channel) pairs of one adjoint tile for the value type (axis 0's samples times
// the tile's channels)
int64_t f2_pairs_per_tile(int dtype);

// One evaluate! (kind 0: warp tasks, kind 2: tiles) or evaluate_adjoint! (kind 1) of one
// grid: one launch over the units of `t`.  dtype SG_BF16_F32 reads bfloat16 control points (forward only).
// status: device word where a bounded wait of the adjoint that gives up records
// SG_ERR_TIMEOUT.
int f2_launch_grid(int dtype, const F2Grid &g, const F2Tiling &t, int kind, int *status, cudaStream_t s);

// The batch kernels over a device list of units of one kind (grids: device descriptors
// indexed by F2Tile::grid).  Forward: one warp per unit (kind 0) or one CTA per tile
// (kind 2); adjoint: persistent CTAs that take tiles with an atomic on `head` (zero
// before the launch).
int f2_launch_batch(int dtype, int kind, const F2Grid *grids, const F2Tile *tiles, int64_t n_tiles,
                    unsigned long long *head, int *status, cudaStream_t s);

// Test hooks of the adjoint kernels' bounded waits: the consumers' wait budget in SM
// cycles (<= 0: the default, about a second), and whether the producer withholds its
// arrival on every CTA's first stage (the stage never completes; the waits run out).
int f2_set_wait_cycles(int64_t cycles);
int f2_set_withhold_first_stage(bool on);

// off[c] = sum over c' < c of (lb0[c' + 1 + d] - lb0[c']) for c in [0, n]: where control
// point c's weights start in the adjoint's axis-0 weight list (lb0: the support table
// lb[c + d], n + d + 1 values).
inline std::vector<int32_t> f2_weight_offsets(const int32_t *lb0, int64_t n, int d) {
    std::vector<int32_t> off((size_t)n + 1, 0);
    for (int64_t c = 0; c < n; ++c) off[c + 1] = off[c] + (lb0[c + 1 + d] - lb0[c]);
    return off;
}

// Whether a grid's sizes fit the fused path's 32-bit element offsets.
inline bool f2_offsets_fit(int64_t ns0, int64_t ns1, int64_t n0, int64_t n1, int64_t nch) {
    const int64_t lim = 0x7fffffffLL;
    return ns0 * ns1 * nch < lim && n0 * n1 * nch < lim;
}

}  // namespace sg
