// tile_table.h — measured tile plan parameters by row-length histogram.
//
// Written by cupdlp.jl_gb300/tune_tiles.py from a sweep of the plan parameters on one
// GB300: for each tuning matrix, precision and kernel side, the histogram of its rows
// (row_histogram) and the parameters with the lowest measured kernel time. The planner
// takes the entry nearest to an instance's histogram (choose_tile_config).
#pragma once

#include <cstdint>

namespace gpdhg {

struct TileTableEntry {
  const char* name;
  bool fp64;
  int side;
  float hist[17];
  int32_t tile_nnz, e_floor, tpc_max;
};

inline constexpr TileTableEntry kTileTable[] = {
    {"none", false, -1, {}, 0, 0, 0},   // placeholder: no measured entries yet
};

}  // namespace gpdhg
