// chunks.h — chunk plans of the step kernels (see pipe.cuh for the layout).
#pragma once

#include <vector>

#include "pipe.cuh"
#include "problem.h"

namespace gpdhg {

// The chunks of one matrix for one value type, their blobs, and the split-row scratch.
template <class T>
struct ChunkPlan {
  DBuf<Chunk> chunks;
  DBuf<uint8_t> blob;
  DBuf<T> carry;
  DBuf<unsigned> counter;
  DBuf<int32_t> inst_begin;  // first chunk of each instance (instances + 1 entries)
  int32_t num = 0;
  int32_t splits = 0;
  long long blob_bytes = 0;
  ChunkView<T> view() const { return ChunkView<T>{chunks.get(), num, blob.get(), carry.get(), counter.get()}; }
};

// Appends the chunks of rows [r0, r1) of a CSR with row pointer rp (instance `inst`):
// consecutive rows while they hold at most s_cap nonzeros and r_cap rows; a row longer
// than s_cap becomes ceil(len / s_cap) pieces. An empty range still gets one empty chunk
// (the instance's step decision runs in it).
void list_chunks(const int32_t* rp, int32_t r0, int32_t r1, int32_t inst, int32_t aux, int s_cap, int r_cap,
                 int e_max, std::vector<Chunk>& out, int32_t& splits, int32_t& carries);

// Plan of rows [bounds[k], bounds[k + 1]) for every instance k of matrix M (Chunk::aux =
// aux[k], or 0 when aux is empty); blobs are filled on the device from M's CSR.
template <class T>
void build_chunk_plan(ChunkPlan<T>& plan, const DeviceMatrix& M, const std::vector<int32_t>& bounds,
                      const std::vector<int32_t>& aux, cudaStream_t s);

// Launch shape of a persistent step kernel: dynamic shared memory attribute set, grid =
// resident CTAs per SM x SMs (at most the chunk count).
int persistent_grid(const void* kernel, int dyn_smem, int num_chunks);

}  // namespace gpdhg
