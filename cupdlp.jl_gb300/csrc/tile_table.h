// tile_table.h — measured tile plan parameters by row-length histogram.
//
// Written by cupdlp.jl_gb300/tune_tiles.py from a sweep of the plan parameters on one
// GB300: for each tuning matrix, precision and kernel side, the histogram of its rows
// (row_histogram) and the parameters with the lowest measured kernel time. The planner
// takes the entry nearest to an instance's histogram (choose_tile_config).
// Kernel times: microseconds per launch over 200 iterations, best vs default parameters;
// the best replaces the default where it is at least 3% faster.
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
    // powerlaw_full FP32 side 0: 113.6 us (default 113.7 us; measured best (256, 1, 96))
    {"powerlaw_full", false, 0, {0.0762f, 0.0152f, 0.0194f, 0.0264f, 0.0373f, 0.0528f, 0.0734f, 0.1023f, 0.5971f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.7605f}, 256, 8, 96},
    // powerlaw_full FP32 side 1: 130.6 us (default 130.9 us; measured best (256, 1, 96))
    {"powerlaw_full", false, 1, {0.0000f, 0.0001f, 0.0125f, 0.2513f, 0.3833f, 0.1825f, 0.0871f, 0.0423f, 0.0211f, 0.0104f, 0.0052f, 0.0024f, 0.0013f, 0.0005f, 0.0000f, 0.0000f, 0.7605f}, 256, 8, 96},
    // powerlaw_full FP64 side 0: 143.0 us (default 143.0 us; measured best (128, 4, 96))
    {"powerlaw_full", true, 0, {0.0762f, 0.0152f, 0.0194f, 0.0264f, 0.0373f, 0.0528f, 0.0734f, 0.1023f, 0.5971f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.7605f}, 128, 4, 96},
    // powerlaw_full FP64 side 1: 203.3 us (default 203.6 us; measured best (128, 1, 96))
    {"powerlaw_full", true, 1, {0.0000f, 0.0001f, 0.0125f, 0.2513f, 0.3833f, 0.1825f, 0.0871f, 0.0423f, 0.0211f, 0.0104f, 0.0052f, 0.0024f, 0.0013f, 0.0005f, 0.0000f, 0.0000f, 0.7605f}, 128, 4, 96},
    // powerlaw_mid FP32 side 0: 33.4 us (default 42.7 us; measured best (128, 1, 24))
    {"powerlaw_mid", false, 0, {0.0762f, 0.0152f, 0.0199f, 0.0270f, 0.0381f, 0.0527f, 0.0722f, 0.1017f, 0.5970f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6878f}, 128, 1, 24},
    // powerlaw_mid FP32 side 1: 36.9 us (default 40.4 us; measured best (256, 8, 24))
    {"powerlaw_mid", false, 1, {0.0000f, 0.0002f, 0.0124f, 0.2521f, 0.3859f, 0.1810f, 0.0875f, 0.0422f, 0.0209f, 0.0097f, 0.0054f, 0.0028f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6878f}, 256, 8, 24},
    // powerlaw_mid FP64 side 0: 40.7 us (default 44.9 us; measured best (128, 4, 24))
    {"powerlaw_mid", true, 0, {0.0762f, 0.0152f, 0.0199f, 0.0270f, 0.0381f, 0.0527f, 0.0722f, 0.1017f, 0.5970f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6878f}, 128, 4, 24},
    // powerlaw_mid FP64 side 1: 57.6 us (default 57.6 us; measured best (128, 4, 96))
    {"powerlaw_mid", true, 1, {0.0000f, 0.0002f, 0.0124f, 0.2521f, 0.3859f, 0.1810f, 0.0875f, 0.0422f, 0.0209f, 0.0097f, 0.0054f, 0.0028f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6878f}, 128, 4, 96},
    // transportation FP32 side 0: 21.6 us (default 21.6 us; measured best (256, 8, 96))
    {"transportation", false, 0, {0.0000f, 1.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 256, 8, 96},
    // transportation FP32 side 1: 21.4 us (default 21.5 us; measured best (256, 1, 96))
    {"transportation", false, 1, {0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5000f, 0.0000f, 0.5000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 256, 8, 96},
    // transportation FP64 side 0: 27.4 us (default 27.5 us; measured best (64, 4, 96))
    {"transportation", true, 0, {0.0000f, 1.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 128, 4, 96},
    // transportation FP64 side 1: 26.0 us (default 26.2 us; measured best (64, 1, 96))
    {"transportation", true, 1, {0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5000f, 0.0000f, 0.5000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 128, 4, 96},
    // uniform FP32 side 0: 18.4 us (default 18.4 us; measured best (256, 8, 96))
    {"uniform", false, 0, {0.0000f, 0.0028f, 0.1274f, 0.7866f, 0.0831f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 256, 8, 96},
    // uniform FP32 side 1: 26.6 us (default 26.7 us; measured best (256, 8, 24))
    {"uniform", false, 1, {0.0000f, 0.0000f, 0.0003f, 0.1044f, 0.8817f, 0.0136f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 256, 8, 96},
    // uniform FP64 side 0: 28.2 us (default 28.2 us; measured best (128, 4, 96))
    {"uniform", true, 0, {0.0000f, 0.0028f, 0.1274f, 0.7866f, 0.0831f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 128, 4, 96},
    // uniform FP64 side 1: 33.9 us (default 33.9 us; measured best (128, 4, 96))
    {"uniform", true, 1, {0.0000f, 0.0000f, 0.0003f, 0.1044f, 0.8817f, 0.0136f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.6541f}, 128, 4, 96},
    // small FP32 side 0: 9.7 us (default 10.2 us; measured best (128, 1, 96))
    {"small", false, 0, {0.0001f, 0.0029f, 0.1268f, 0.7874f, 0.0829f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5191f}, 128, 1, 96},
    // small FP32 side 1: 15.3 us (default 16.0 us; measured best (128, 1, 24))
    {"small", false, 1, {0.0000f, 0.0000f, 0.0001f, 0.1051f, 0.8807f, 0.0140f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5191f}, 128, 1, 24},
    // small FP64 side 0: 10.3 us (default 10.5 us; measured best (128, 4, 24))
    {"small", true, 0, {0.0001f, 0.0029f, 0.1268f, 0.7874f, 0.0829f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5191f}, 128, 4, 96},
    // small FP64 side 1: 17.2 us (default 17.6 us; measured best (128, 1, 24))
    {"small", true, 1, {0.0000f, 0.0000f, 0.0001f, 0.1051f, 0.8807f, 0.0140f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.5191f}, 128, 4, 96},
};

}  // namespace gpdhg
