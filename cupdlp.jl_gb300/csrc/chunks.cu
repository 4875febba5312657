// chunks.cu — host builder of the chunk plans and the device blob fill.
#include <algorithm>

#include "chunks.h"

namespace gpdhg {

namespace {

int ceil_log2(long long v) {
  int l = 0;
  while ((1LL << l) < v) ++l;
  return l;
}

// One CTA per chunk: local row offsets (clamped to the chunk, so a piece of a split row
// sees [0, nnz]), column indices, values converted to T at their padded positions.
template <class T>
__global__ void __launch_bounds__(kBlock) fill_blob_kernel(const Chunk* chunks, int num, const int32_t* row_ptr,
                                                           const int32_t* col, const double* val, uint8_t* blob) {
  constexpr int SH = PipeTraits<T>::kPadShift;
  for (int c = blockIdx.x; c < num; c += gridDim.x) {
    const Chunk ch = chunks[c];
    uint8_t* base = blob + ch.blob;
    int32_t* rp = reinterpret_cast<int32_t*>(base);
    int32_t* cb = reinterpret_cast<int32_t*>(base + blob_rp_bytes<T>(ch.rows));
    T* vb = reinterpret_cast<T*>(base + blob_rp_bytes<T>(ch.rows) + blob_col_bytes<T>(ch.nnz));
    const int rpn = blob_rp_bytes<T>(ch.rows) / 4;
    for (int j = threadIdx.x; j < rpn; j += kBlock) {
      const long long v = j <= ch.rows ? (long long)row_ptr[ch.row_begin + j] - ch.nnz_begin : ch.nnz;
      rp[j] = (int32_t)(v < 0 ? 0 : (v > ch.nnz ? ch.nnz : v));
    }
    const int cn = blob_col_bytes<T>(ch.nnz) / 4;
    for (int k = threadIdx.x; k < cn; k += kBlock) cb[k] = k < ch.nnz ? col[ch.nnz_begin + k] : 0;
    const int vn = blob_val_bytes<T>(ch.nnz) / (int)sizeof(T);
    for (int q = threadIdx.x; q < vn; q += kBlock) vb[q] = T(0);
    __syncthreads();
    for (int k = threadIdx.x; k < ch.nnz; k += kBlock) vb[pad_index(k, SH)] = (T)val[ch.nnz_begin + k];
    __syncthreads();
  }
}

}  // namespace

void list_chunks(const int32_t* rp, int32_t r0, int32_t r1, int32_t inst, int32_t aux, int s_cap, int r_cap,
                 int e_max, std::vector<Chunk>& out, int32_t& splits, int32_t& carries) {
  auto len = [&](int32_t r) { return (long long)rp[r + 1] - rp[r]; };
  auto push = [&](int32_t rb, int32_t rows, long long nb, long long nnz, int32_t split, int32_t piece,
                  int32_t pieces, int32_t carry) {
    Chunk ch{};
    ch.row_begin = rb;
    ch.rows = rows;
    ch.nnz_begin = (int32_t)nb;
    ch.nnz = (int32_t)nnz;
    ch.inst = inst;
    // nonzeros per thread: enough for the chunk, and about one row per run when rows are
    // short (fewer cross-run rows to complete), at most e_max
    long long e = std::max<long long>(1, (nnz + kBlock - 1) / kBlock);
    if (rows > 0) e = std::max<long long>(e, std::min<long long>((nnz + rows - 1) / rows, e_max));
    ch.e_log2 = ceil_log2(e);
    ch.split = split;
    ch.piece = piece;
    ch.pieces = pieces;
    ch.carry = carry;
    ch.aux = aux;
    out.push_back(ch);
  };
  const size_t first = out.size();
  int32_t r = r0;
  while (r < r1) {
    const long long lr = len(r);
    if (lr > s_cap) {
      const int32_t pieces = (int32_t)((lr + s_cap - 1) / s_cap);
      const int32_t sid = splits++;
      const int32_t cb = carries;
      carries += pieces;
      for (int32_t q = 0; q < pieces; ++q)
        push(r, 1, (long long)rp[r] + (long long)q * s_cap, std::min<long long>(s_cap, lr - (long long)q * s_cap), sid,
             q, pieces, cb);
      ++r;
      continue;
    }
    const int32_t start = r;
    long long nnz = 0;
    while (r < r1 && r - start < r_cap && len(r) <= s_cap && nnz + len(r) <= s_cap) {
      nnz += len(r);
      ++r;
    }
    push(start, r - start, rp[start], nnz, -1, 0, 1, 0);
  }
  if (out.size() == first) push(r0, 0, rp[r0], 0, -1, 0, 1, 0);
}

template <class T>
void build_chunk_plan(ChunkPlan<T>& plan, const DeviceMatrix& M, const std::vector<int32_t>& bounds,
                      const std::vector<int32_t>& aux, cudaStream_t s) {
  if ((int32_t)M.host_rp.size() != M.nrows + 1) throw Error(GPDHG_ERR_INTERNAL, "matrix has no host row pointer");
  const int K = (int)bounds.size() - 1;
  std::vector<Chunk> list;
  std::vector<int32_t> begin(K + 1);
  int32_t splits = 0, carries = 0;
  for (int k = 0; k < K; ++k) {
    begin[k] = (int32_t)list.size();
    list_chunks(M.host_rp.data(), bounds[k], bounds[k + 1], k, aux.empty() ? 0 : aux[k], PipeTraits<T>::kS,
                PipeTraits<T>::kR, PipeTraits<T>::kEMax, list, splits, carries);
  }
  begin[K] = (int32_t)list.size();
  long long off = 0;
  for (Chunk& ch : list) {
    ch.blob = off;
    off += blob_bytes<T>(ch.rows, ch.nnz);
  }
  plan.num = (int32_t)list.size();
  plan.splits = splits;
  plan.blob_bytes = off;
  plan.chunks.alloc(list.size());
  plan.blob.alloc((size_t)std::max<long long>(off, 16));
  plan.carry.alloc(std::max(carries, 1));
  plan.counter.alloc(std::max(splits, 1));
  plan.inst_begin.alloc(begin.size());
  CK(cudaMemcpyAsync(plan.chunks.get(), list.data(), sizeof(Chunk) * list.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(plan.inst_begin.get(), begin.data(), sizeof(int32_t) * begin.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(plan.counter.get(), 0, sizeof(unsigned) * std::max(splits, 1), s));
  const int grid = std::max(1, std::min(plan.num, 8192));
  fill_blob_kernel<T><<<grid, kBlock, 0, s>>>(plan.chunks.get(), plan.num, M.row_ptr.get(), M.col.get(),
                                              M.val64.get(), plan.blob.get());
  CK_LAUNCH();
  // the host list dies at return: wait for the copies before it does
  CK(cudaStreamSynchronize(s));
}

template void build_chunk_plan<float>(ChunkPlan<float>&, const DeviceMatrix&, const std::vector<int32_t>&,
                                      const std::vector<int32_t>&, cudaStream_t);
template void build_chunk_plan<double>(ChunkPlan<double>&, const DeviceMatrix&, const std::vector<int32_t>&,
                                       const std::vector<int32_t>&, cudaStream_t);

int persistent_grid(const void* kernel, int dyn_smem, int num_chunks) {
  int dev = 0, sms = 0, per_sm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, dyn_smem));
  if (per_sm < 1) throw Error(GPDHG_ERR_CUDA, "step kernel does not fit on an SM");
  return std::max(1, std::min(num_chunks, per_sm * sms));
}

}  // namespace gpdhg
