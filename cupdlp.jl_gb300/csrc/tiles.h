// tiles.h — the work decomposition of the step kernels: warp tiles grouped into CTAs.
//
// A tile is one warp's share of a CSR matrix: consecutive rows holding at most
// TileTraits<T>::kNnz nonzeros and at most kTileRows rows, or one row of up to kWarpShare
// nonzeros streamed by the warp in rounds. A longer row is a group tile: W = 2, 4 or 8
// warps (about kWarpShare nonzeros each) split it and combine their sums in shared memory,
// 8 / W such rows to a CTA; a row longer than kCtaNnz is cut into 8-warp pieces of kCtaNnz
// whose partial sums meet in a carry array. Consecutive tiles of one instance form a CTA's
// work (8 to 96 tiles, dealt to its 8 warps in turn, or 8 / W group tiles), so every CTA
// belongs to exactly one instance and the per-instance step decision can count CTAs. An
// instance with few tiles gets one tile per warp (most CTAs in flight), a large one as many
// as make its CTAs a single wave over the GPU (no ragged last wave, and fewer partial sums
// for the step decision to reduce). The decomposition depends only on the instance's own
// row lengths, never on where the instance sits in a packed batch.
//
// Lane-interleaved copy: lane l of a warp tile owns the tile's nonzeros [l E, (l + 1) E)
// (consecutive, so that rows are summed with one FMA per nonzero and few shuffles). Read
// from the CSR, the j-th load of every lane would hit 32 addresses E elements apart. The plan
// therefore keeps a copy of every warp tile's columns and values in which the lane's nonzeros
// come in 16-byte groups of G = 16 / (element size) (4 columns or FP32 values, 2 FP64 values):
// the lane's j-th element sits at data_begin + 32 G (j / G) + G l + j % G (interleaved_slot), so
// that each group is one 128-bit load of the lane and each such load of the warp is one
// coalesced 512-byte access. Tiles with E < G keep one element per load (slot data_begin +
// 32 j + l). Slots past the tile's nonzeros hold column 0 and value 0 and are loaded with the
// lane's run but never gathered. Long rows (warp-streamed, group and split) already stream the
// CSR coalesced and have no copy.
#pragma once

#include <vector>

#include "problem.h"

namespace gpdhg {

constexpr int kTileRows = 31;     // rows per tile: rows + 1 row offsets fit in 32 lanes
// Nonzeros per lane (at most) and per tile: FP64 tiles are half as long, which keeps a
// lane's values and gathered entries in registers at the FP64 kernels' occupancy.
template <class T>
struct TileTraits {
  static constexpr int kEMax = sizeof(T) == 8 ? 4 : 8;
  static constexpr int kNnz = 32 * kEMax;
};
constexpr int kWarpShare = 512;   // nonzeros per warp of a long row
constexpr int kCtaNnz = 16384;    // longest row (piece) one CTA sums
constexpr int kLongRound = 8;     // (column, value) loads per lane and round of a long row
constexpr int kTilesPerCtaMin = 8;   // tiles per CTA: one per warp for small instances,
constexpr int kTilesPerCtaMax = 96;  // up to twelve per warp for large ones
// Resident CTAs per SM of the step kernels (their __launch_bounds__ minimum): a large
// instance gets one CTA per resident slot of the GPU's 152 SMs, so its CTAs run as one wave
// with no partly filled last wave.
template <class T>
constexpr int kPrimalCtasPerSm = sizeof(T) == 8 ? 4 : 4;
constexpr int kDualCtasPerSm = 4;

// Slot of lane `lane`'s j-th element in a warp tile's interleaved copy of `bytes`-byte
// elements (E = 2^e_log2 per lane): 16-byte groups when E fills one.
__host__ __device__ constexpr long long interleaved_slot(int data_begin, int e_log2, int lane, int j, int bytes) {
  return (16 / bytes <= (1 << e_log2))
             ? (long long)data_begin + 32LL * (16 / bytes) * (j / (16 / bytes)) + (16 / bytes) * lane + j % (16 / bytes)
             : (long long)data_begin + 32LL * j + lane;
}

constexpr int kWarpLong = -1;  // Tile::e_log2 of a row streamed by one warp
// Tile::e_log2 of a row summed by 2^g warps (g = 1, 2, 3)
__host__ __device__ constexpr int group_code(int g) { return -1 - g; }
__host__ __device__ constexpr int group_log2(int e_log2) { return -1 - e_log2; }

struct Tile {
  int32_t row_begin;  // first row (packed numbering)
  int32_t rows;       // rows of the tile (1 for a piece of a split row, 0 for an empty instance)
  int32_t nnz_begin;  // first nonzero in the CSR
  int32_t nnz;        // nonzeros of the tile
  int32_t e_log2;     // log2 of the nonzeros per lane; kWarpLong: one row streamed by the
                      // warp; group_code(g): one row (or piece) summed by 2^g warps
  int32_t split;      // -1, or the split row this piece belongs to
  int32_t piece;      // piece index within the split row
  int32_t pieces;     // pieces of the split row
  int32_t carry;      // first carry slot of the split row
  int32_t aux;        // tiles of A: first inequality row of the instance (packed numbering)
  int32_t data_begin; // warp tiles: first slot of the tile in the lane-interleaved copy
};

// Device view of a tile plan.
template <class T>
struct TileView {
  const Tile* tiles;
  const int32_t* cta_tile_begin;    // first tile of each CTA (ctas + 1)
  const int32_t* cta_inst;          // instance of each CTA
  const int32_t* inst_cta_begin;    // first CTA of each instance (instances + 1)
  const int32_t* inst_split_begin;  // first split row of each instance (instances + 1)
  T* carry;                         // one partial row sum per piece of every split row
  unsigned* counter;                // pieces finished per split row (back to 0 after each launch)
  const int32_t* cta_map;           // launched CTA -> plan CTA (NULL: the identity); a batch
                                    // launches only the CTAs of instances still running
  const int32_t* icol;              // lane-interleaved columns of the warp tiles
  const T* ival;                    // lane-interleaved values of the warp tiles
  int32_t num_ctas;
  int32_t num_splits;
};

template <class T>
struct TilePlan {
  DBuf<Tile> tiles;
  DBuf<int32_t> cta_tile_begin, cta_inst, inst_cta_begin, inst_split_begin;
  DBuf<T> carry;
  DBuf<unsigned> counter;
  DBuf<int32_t> icol;
  DBuf<T> ival;
  int32_t num_tiles = 0, num_ctas = 0, num_splits = 0;
  long long interleaved_slots = 0;
  TileView<T> view() const {
    return TileView<T>{tiles.get(),      cta_tile_begin.get(), cta_inst.get(), inst_cta_begin.get(),
                       inst_split_begin.get(), carry.get(),     counter.get(),  nullptr,
                       icol.get(),       ival.get(),            num_ctas,       num_splits};
  }
};

// Plan parameters of one instance's tiles. The kernels take any values within the limits
// below; choose_tile_config picks them per instance from its row-length histogram.
struct TileConfig {
  int32_t tile_nnz;   // nonzeros per warp tile at most (<= 32 * kEMax); longer rows up to
                      // kWarpShare are warp-streamed
  int32_t e_floor;    // a lane's run is at least min(ceil(nnz / rows), e_floor) nonzeros (about
                      // one row per lane when rows are short; 1 turns the rule off)
  int32_t tpc_max;    // tiles per CTA at most (kTilesPerCtaMin..kTilesPerCtaMax)
};
constexpr int kTileSideAt = 0;   // the primal kernel's plan (rows of A')
constexpr int kTileSideA = 1;    // the dual kernel's plan (rows of A)
// Row-length histogram of an instance: the share of its nonzeros in rows of length
// [2^b, 2^(b+1)) for b = 0..kHistBins-2 (the last bin takes longer rows), then
// log2(nonzeros) / 32 as a size feature.
constexpr int kHistBins = 16;
constexpr int kHistLen = kHistBins + 1;
void row_histogram(const int32_t* rp, int32_t r0, int32_t r1, float* h);
// Instances (and table entries) with fewer than 2^20 nonzeros use the default parameters.
constexpr float kTileTableMinSize = 20.0f / 32.0f;
template <class T>
TileConfig default_tile_config();
// The measured table's entry nearest (L1 distance over the histogram) to the instance's,
// for the plan's precision and side, among entries of at least 2^20 nonzeros; the default for
// smaller instances or when the table has none. A process-wide override (set_tile_override,
// used by the tuning sweep) takes precedence.
template <class T>
TileConfig choose_tile_config(const int32_t* rp, int32_t r0, int32_t r1, int side);
// precision: GPDHG_PRECISION_FP64 or GPDHG_PRECISION_FP32; cfg NULL clears the override.
void set_tile_override(int precision, int side, const TileConfig* cfg);

// Appends the tiles of rows [r0, r1) of a CSR with row pointer rp (instance inst). An empty
// range still gets one empty tile (the instance's step decision runs in its CTA).
void list_tiles(const int32_t* rp, int32_t r0, int32_t r1, int32_t inst, int32_t aux, int tile_nnz, int e_max,
                std::vector<Tile>& out, int32_t& splits, int32_t& carries);

// Plan of rows [bounds[k], bounds[k + 1]) for every instance k of matrix M (Tile::aux =
// aux[k], or 0 when aux is empty), with the lane-interleaved copy of M's precision-T values
// (M.view<T>() must hold them).
template <class T>
void build_tile_plan(TilePlan<T>& plan, const DeviceMatrix& M, const std::vector<int32_t>& bounds,
                     const std::vector<int32_t>& aux, int ctas_per_sm, int side, cudaStream_t s);

}  // namespace gpdhg
