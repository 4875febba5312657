// tiles.cu — host builder of the tile plans of the step kernels.
#include <algorithm>
#include <atomic>
#include <exception>
#include <thread>
#include <cmath>
#include <mutex>

#include "tile_table.h"
#include "tiles.h"

namespace gpdhg {

namespace {
int ceil_log2(long long v) {
  int l = 0;
  while ((1LL << l) < v) ++l;
  return l;
}

// One warp per warp tile: lane l's j-th nonzero (CSR position nnz_begin + l E + j) goes to
// its interleaved_slot in the column and the value copy; slots past the tile's nonzeros get
// column 0 and value 0.
template <class T>
__global__ void __launch_bounds__(256) interleave_tiles_kernel(const Tile* __restrict__ tiles, int ntiles,
                                                              const int32_t* __restrict__ col,
                                                              const T* __restrict__ val, int32_t* icol, T* ival) {
  const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= ntiles) return;
  const Tile t = tiles[w];
  if (t.e_log2 < 0) return;
  const int E = 1 << t.e_log2;
  for (int j = 0; j < E; ++j) {
    const int k = lane * E + j;
    const bool in = k < t.nnz;
    icol[interleaved_slot(t.data_begin, t.e_log2, lane, j, 4)] = in ? col[(long long)t.nnz_begin + k] : 0;
    ival[interleaved_slot(t.data_begin, t.e_log2, lane, j, (int)sizeof(T))] = in ? val[(long long)t.nnz_begin + k] : T(0);
  }
}
}  // namespace

void row_histogram(const int32_t* rp, int32_t r0, int32_t r1, float* h) {
  double w[kHistBins] = {};
  long long total = 0;
  for (int32_t r = r0; r < r1; ++r) {
    const long long len = (long long)rp[r + 1] - rp[r];
    if (len <= 0) continue;
    const int b = std::min(kHistBins - 1, 63 - __builtin_clzll((unsigned long long)len));  // floor(log2 len)
    w[b] += (double)len;
    total += len;
  }
  for (int b = 0; b < kHistBins; ++b) h[b] = total ? (float)(w[b] / (double)total) : 0.0f;
  h[kHistBins] = total ? (float)(std::log2((double)total) / 32.0) : 0.0f;
}

template <class T>
TileConfig default_tile_config() {
  return TileConfig{TileTraits<T>::kNnz, TileTraits<T>::kEMax, kTilesPerCtaMax};
}

namespace {
std::mutex g_override_mutex;
bool g_override_set[2][2] = {};
TileConfig g_override[2][2];
int precision_slot(int precision) { return precision == GPDHG_PRECISION_FP64 ? 0 : 1; }
}  // namespace

void set_tile_override(int precision, int side, const TileConfig* cfg) {
  if (side != kTileSideAt && side != kTileSideA) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "side must be 0 or 1");
  std::lock_guard<std::mutex> lk(g_override_mutex);
  const int q = precision_slot(precision);
  g_override_set[q][side] = cfg != nullptr;
  if (cfg) g_override[q][side] = *cfg;
}

template <class T>
TileConfig choose_tile_config(const int32_t* rp, int32_t r0, int32_t r1, int side) {
  const int q = sizeof(T) == 8 ? 0 : 1;
  auto clamp = [](TileConfig c) {
    c.tile_nnz = std::max(32, std::min(c.tile_nnz, TileTraits<T>::kNnz));
    c.e_floor = std::max(1, std::min(c.e_floor, TileTraits<T>::kEMax));
    c.tpc_max = std::max(kTilesPerCtaMin, std::min(c.tpc_max, kTilesPerCtaMax));
    return c;
  };
  {
    std::lock_guard<std::mutex> lk(g_override_mutex);
    if (g_override_set[q][side]) return clamp(g_override[q][side]);
  }
  float h[kHistLen];
  row_histogram(rp, r0, r1, h);
  // the table was measured on lone solves of large matrices; smaller instances (latency
  // bound alone, and run side by side with others in a batch, where the lone optimum did not
  // carry over) keep the default parameters
  if (h[kHistBins] < kTileTableMinSize) return default_tile_config<T>();
  const TileTableEntry* best = nullptr;
  double best_d = 0.0;
  for (const TileTableEntry& e : kTileTable) {
    if (e.fp64 != (q == 0) || e.side != side || e.hist[kHistBins] < kTileTableMinSize) continue;
    double d = 0.0;
    for (int b = 0; b < kHistLen; ++b) d += std::fabs((double)e.hist[b] - (double)h[b]);
    if (!best || d < best_d) {
      best = &e;
      best_d = d;
    }
  }
  if (!best) return default_tile_config<T>();
  return clamp(TileConfig{best->tile_nnz, best->e_floor, best->tpc_max});
}

template TileConfig default_tile_config<float>();
template TileConfig default_tile_config<double>();
template TileConfig choose_tile_config<float>(const int32_t*, int32_t, int32_t, int);
template TileConfig choose_tile_config<double>(const int32_t*, int32_t, int32_t, int);

void list_tiles(const int32_t* rp, int32_t r0, int32_t r1, int32_t inst, int32_t aux, int tile_nnz, int e_max,
                std::vector<Tile>& out, int32_t& splits, int32_t& carries) {
  auto len = [&](int32_t r) { return (long long)rp[r + 1] - rp[r]; };
  auto push = [&](int32_t rb, int32_t rows, long long nb, long long nnz, int32_t split, int32_t piece,
                  int32_t pieces, int32_t carry) {
    Tile t{};
    t.row_begin = rb;
    t.rows = rows;
    t.nnz_begin = (int32_t)nb;
    t.nnz = (int32_t)nnz;
    // nonzeros per lane: enough for the tile, and about one row per lane when rows are
    // short (fewer rows crossing lanes), at most e_max
    long long e = std::max<long long>(1, (nnz + 31) / 32);
    if (rows > 0) e = std::max<long long>(e, std::min<long long>((nnz + rows - 1) / rows, e_max));
    t.e_log2 = ceil_log2(e);
    t.split = split;
    t.piece = piece;
    t.pieces = pieces;
    t.carry = carry;
    t.aux = aux;
    out.push_back(t);
  };
  const size_t first = out.size();
  int32_t r = r0;
  while (r < r1) {
    const long long lr = len(r);
    if (lr > tile_nnz) {
      if (lr <= kWarpShare) {
        push(r, 1, rp[r], lr, -1, 0, 1, 0);
        out.back().e_log2 = kWarpLong;
        ++r;
        continue;
      }
      int g = 1;  // 2^g warps, about kWarpShare nonzeros each, at most 8
      while (g < 3 && ((long long)kWarpShare << g) < lr) ++g;
      const int32_t pieces = (int32_t)((lr + kCtaNnz - 1) / kCtaNnz);
      int32_t sid = -1, cb = 0;
      if (pieces > 1) {
        sid = splits++;
        cb = carries;
        carries += pieces;
      }
      for (int32_t q = 0; q < pieces; ++q) {
        push(r, 1, (long long)rp[r] + (long long)q * kCtaNnz,
             std::min<long long>(kCtaNnz, lr - (long long)q * kCtaNnz), sid, q, pieces, cb);
        out.back().e_log2 = group_code(g);
      }
      ++r;
      continue;
    }
    const int32_t start = r;
    long long nnz = 0;
    while (r < r1 && r - start < kTileRows && len(r) <= tile_nnz && nnz + len(r) <= tile_nnz) {
      nnz += len(r);
      ++r;
    }
    push(start, r - start, rp[start], nnz, -1, 0, 1, 0);
  }
  if (out.size() == first) push(r0, 0, rp[r0], 0, -1, 0, 1, 0);
}

template <class T>
void build_tile_plan(TilePlan<T>& plan, const DeviceMatrix& M, const std::vector<int32_t>& bounds,
                     const std::vector<int32_t>& aux, int ctas_per_sm, int side, cudaStream_t s) {
  if ((int32_t)M.host_rp.size() != M.nrows + 1) throw Error(GPDHG_ERR_INTERNAL, "matrix has no host row pointer");
  PhaseTrace tr;
  const int K = (int)bounds.size() - 1;
  // each instance's tiles and CTAs on their own (on host threads for a batch: the rows of a
  // packed A' run to tens of millions), then concatenated in instance order with the split
  // rows and carry slots renumbered after those of the instances before
  struct Part {
    std::vector<Tile> tiles;
    std::vector<int32_t> cta_begin;   // first tile of each CTA, within the instance
    int32_t splits = 0, carries = 0;
  };
  std::vector<Part> parts(K);
  auto plan_instance = [&](int k) {
    Part& P = parts[k];
    const TileConfig cfg = choose_tile_config<T>(M.host_rp.data(), bounds[k], bounds[k + 1], side);
    list_tiles(M.host_rp.data(), bounds[k], bounds[k + 1], k, aux.empty() ? 0 : aux[k], cfg.tile_nnz,
               cfg.e_floor, P.tiles, P.splits, P.carries);
    // warp-streamed rows first, in row order, then the other tiles in row order: CTAs then
    // hold one kind of work (a power-law A' scatters thousands of such rows among short ones)
    std::stable_partition(P.tiles.begin(), P.tiles.end(), [](const Tile& t) { return t.e_log2 == kWarpLong; });
    // CTAs: 8 / W group tiles of one width W together; warp-streamed rows, and the other
    // tiles, in groups of tpc: 8 while the instance has fewer tiles than one per warp of
    // every resident CTA slot (152 SMs x ctas_per_sm), then as many as make the instance's
    // CTAs one wave, up to kTilesPerCtaMax
    const long long nt = (long long)P.tiles.size();
    const long long slots = 152LL * ctas_per_sm;
    const long long tpc = std::min<long long>(cfg.tpc_max, std::max<long long>(kTilesPerCtaMin, (nt + slots - 1) / slots));
    long long open = 0;   // tiles in the CTA being filled
    int open_code = 0;    // its tiles' kind: 0 normal, kWarpLong, else the group code
    for (size_t q = 0; q < P.tiles.size(); ++q) {
      const int e = P.tiles[q].e_log2;
      const int code = e < 0 ? e : 0;
      const long long cap = code <= group_code(1) ? (8 >> group_log2(code)) : tpc;
      if (open == 0 || code != open_code || open == cap) {
        P.cta_begin.push_back((int32_t)q);
        open = 0;
        open_code = code;
      }
      ++open;
    }
  };
  const int threads = std::max(1, std::min<int>(K, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
  if (threads == 1) {
    for (int k = 0; k < K; ++k) plan_instance(k);
  } else {
    std::vector<std::exception_ptr> err(K);
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
      th.emplace_back([&] {
        for (int k = next++; k < K; k = next++) {
          try {
            plan_instance(k);
          } catch (...) {
            err[k] = std::current_exception();
          }
        }
      });
    for (auto& x : th) x.join();
    for (int k = 0; k < K; ++k)
      if (err[k]) std::rethrow_exception(err[k]);
  }
  tr.mark(side == kTileSideAt ? "    plan A': tiles" : "    plan A: tiles");
  std::vector<Tile> tiles;
  std::vector<int32_t> cta_begin, cta_inst, inst_cta(K + 1), inst_split(K + 1);
  int32_t splits = 0, carries = 0;
  {
    size_t total_tiles = 0, total_ctas = 0;
    for (const Part& P : parts) {
      total_tiles += P.tiles.size();
      total_ctas += P.cta_begin.size();
    }
    tiles.reserve(total_tiles);
    cta_begin.reserve(total_ctas + 1);
    cta_inst.reserve(total_ctas);
  }
  for (int k = 0; k < K; ++k) {
    Part& P = parts[k];
    inst_cta[k] = (int32_t)cta_inst.size();
    inst_split[k] = splits;
    const int32_t t0 = (int32_t)tiles.size();
    for (Tile t : P.tiles) {
      if (t.split >= 0) {
        t.split += splits;
        t.carry += carries;
      }
      tiles.push_back(t);
    }
    for (int32_t b : P.cta_begin) {
      cta_begin.push_back(t0 + b);
      cta_inst.push_back(k);
    }
    splits += P.splits;
    carries += P.carries;
    std::vector<Tile>().swap(P.tiles);
  }
  inst_cta[K] = (int32_t)cta_inst.size();
  inst_split[K] = splits;
  cta_begin.push_back((int32_t)tiles.size());
  // slots of the lane-interleaved copy: 32 E per warp tile, in plan order
  long long slots = 0;
  for (Tile& t : tiles) {
    if (t.e_log2 < 0) {
      t.data_begin = 0;
      continue;
    }
    t.data_begin = (int32_t)slots;
    slots += 32LL << t.e_log2;
    if (slots > 0x7fffffffLL) throw Error(GPDHG_ERR_NOT_SUPPORTED, "tile plan exceeds 2^31 interleaved slots");
  }
  plan.num_tiles = (int32_t)tiles.size();
  plan.num_ctas = (int32_t)cta_inst.size();
  plan.num_splits = splits;
  auto up = [&](DBuf<int32_t>& d, const std::vector<int32_t>& v) {
    d.alloc(std::max<size_t>(v.size(), 1));
    CK(cudaMemcpyAsync(d.get(), v.data(), sizeof(int32_t) * v.size(), cudaMemcpyHostToDevice, s));
  };
  plan.tiles.alloc(tiles.size());
  CK(cudaMemcpyAsync(plan.tiles.get(), tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, s));
  up(plan.cta_tile_begin, cta_begin);
  up(plan.cta_inst, cta_inst);
  up(plan.inst_cta_begin, inst_cta);
  up(plan.inst_split_begin, inst_split);
  plan.carry.alloc(std::max(carries, 1));
  plan.counter.alloc(std::max(splits, 1));
  CK(cudaMemsetAsync(plan.counter.get(), 0, sizeof(unsigned) * std::max(splits, 1), s));
  plan.interleaved_slots = slots;
  plan.icol.alloc(std::max<long long>(slots, 1));
  plan.ival.alloc(std::max<long long>(slots, 1));
  const CsrView<T> mv = M.view<T>();
  if (M.nnz > 0 && !mv.val) throw Error(GPDHG_ERR_INTERNAL, "matrix values of the plan's precision are missing");
  if (slots > 0) {
    const int nt = plan.num_tiles;
    const long long threads = 32LL * nt;
    interleave_tiles_kernel<T><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        plan.tiles.get(), nt, mv.col, mv.val, plan.icol.get(), plan.ival.get());
    CK_LAUNCH();
  }
  // the host vectors die at return: wait for the copies before they do
  CK(cudaStreamSynchronize(s));
  tr.mark(side == kTileSideAt ? "    plan A': copies, interleave" : "    plan A: copies, interleave");
}

template void build_tile_plan<float>(TilePlan<float>&, const DeviceMatrix&, const std::vector<int32_t>&,
                                     const std::vector<int32_t>&, int, int, cudaStream_t);
template void build_tile_plan<double>(TilePlan<double>&, const DeviceMatrix&, const std::vector<int32_t>&,
                                      const std::vector<int32_t>&, int, int, cudaStream_t);

}  // namespace gpdhg
