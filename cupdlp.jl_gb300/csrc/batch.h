// batch.h — the packed multi-LP layout behind gpdhg_batch.
#pragma once

#include <functional>

#include <memory>
#include <string>
#include <vector>

#include "host_logic.h"
#include "problem.h"

namespace gpdhg {

constexpr int kSegLen = 1024;   // elements per segmented-reduction item (one CTA each)

template <class T>
struct BatchWorkspace;
struct BatchWorkspaceDeleter {
  void operator()(BatchWorkspace<double>* w) const;
  void operator()(BatchWorkspace<float>* w) const;
};

// Splits [off[k], off[k+1]) of every instance into kSegLen-element items.
void build_seg_items(const std::vector<int32_t>& off, std::vector<SegItem>& items, std::vector<int32_t>& begin);

}  // namespace gpdhg

struct gpdhg_batch {
  int32_t count = 0;
  int32_t M = 0, N = 0;                        // packed rows / columns
  std::vector<int32_t> row_off, col_off, neq;  // per instance (offsets: count + 1)
  std::vector<gpdhg::InstanceInfo> info;
  std::vector<double> amax, norm_b, norm_c;
  std::vector<std::vector<int32_t>> col_perm;  // per instance: choose_column_order's order
  gpdhg::DeviceMatrix A, At;                   // block-diagonal CSR of A and A'
  gpdhg::DBuf<int32_t> row_off_d, neq_d;
  gpdhg::DBuf<double> l, u, c, b, ol, ou, oc, ob, con, var;
  gpdhg::DBuf<uint8_t> ineq_flag;              // per packed row: a '>=' row
  gpdhg::DBuf<int32_t> col_inst, row_inst;     // instance of each packed column / row
  gpdhg::DBuf<gpdhg::SegItem> seg_n, seg_m;
  gpdhg::DBuf<int32_t> seg_n_begin, seg_m_begin;
  int nseg_n = 0, nseg_m = 0;
  cudaStream_t stream = nullptr;
  std::unique_ptr<gpdhg::BatchWorkspace<double>, gpdhg::BatchWorkspaceDeleter> ws64;
  std::unique_ptr<gpdhg::BatchWorkspace<float>, gpdhg::BatchWorkspaceDeleter> ws32;
  ~gpdhg_batch();
};

namespace gpdhg {
void batch_init(gpdhg_batch* B, int32_t count, const gpdhg_lp_desc* descs);
// on_retire (optional) is called with an instance's index right after that instance has
// terminated and its result and solution have been written (from the calling thread).
void batch_solve(gpdhg_batch* B, const gpdhg_params& prm, gpdhg_result* results, double* const* primal_out,
                 double* const* dual_out, const std::function<void(int)>* on_retire = nullptr);

// Serving loop (server.cu).
double footprint_bytes(const gpdhg_lp_desc& d, const gpdhg_params& p);
gpdhg_server* server_create(const gpdhg_server_config& cfg);
void server_destroy(gpdhg_server* s);
uint64_t server_submit(gpdhg_server* s, const gpdhg_lp_desc& d, const gpdhg_params& p);
// OK (outputs copied, ticket released), NOT_READY, or the request's error (err set).
gpdhg_status server_take(gpdhg_server* s, uint64_t ticket, double timeout_sec, gpdhg_result* r, double* x,
                         double* y, std::string& err);
}  // namespace gpdhg
