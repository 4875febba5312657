// server.cu — the serving loop: continuous batching of arriving LPs on one GPU.
//
// Requests wait in a FIFO queue. Each worker thread owns its CUDA stream (through the
// gpdhg_batch it builds) and repeatedly forms a cohort: the waiting requests that share the
// head request's parameters, as many as the admission limits allow (device footprint within
// the HBM budget, resident request count, cohort size), after lingering briefly for more.
// The cohort is packed into one segmented batch and solved; every instance retires from the
// device work the moment it terminates, and its result is handed out at that moment (a
// small request does not wait for the large ones it was packed with). Once at most a quarter
// of a cohort's instances still run, the cohort gives up its worker slot: another worker (the
// server keeps twice `workers` threads) may start a new cohort beside its stragglers, so
// arriving requests back-fill the device while the stragglers finish. The cohort's memory
// returns to the budget when its last instance is done: the packed buffers are freed
// together. Cohorts of different workers run concurrently, so a request that arrives while
// others are on the GPU starts as soon as a worker and memory are free and its kernels
// overlap with theirs. Each result is the lone solve's result bit for bit. Requests whose
// parameters a batch does not take (the FP64 hand-off of FP32_REFINE, the constant step
// size) are solved one after another as lone problems by the worker that picked them.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "batch.h"
#include "problem.h"

namespace gpdhg {

namespace {

// Deep copy of a request's LP descriptor.
struct HostLp {
  gpdhg_lp_desc d{};
  std::vector<int32_t> rp, col;
  std::vector<double> val, l, u, c, b, ol, ou, oc, ob, con, var;

  void copy_from(const gpdhg_lp_desc& s) {
    d = s;
    const int32_t n = s.num_variables, m = s.num_constraints;
    auto cp = [](auto& dst, const auto* src, size_t len) -> decltype(dst.data()) {
      if (!src) return nullptr;
      dst.assign(src, src + len);
      return dst.data();
    };
    d.row_ptr = cp(rp, s.row_ptr, (size_t)m + 1);
    d.col_idx = cp(col, s.col_idx, (size_t)s.nnz);
    d.values = cp(val, s.values, (size_t)s.nnz);
    d.variable_lower_bound = cp(l, s.variable_lower_bound, n);
    d.variable_upper_bound = cp(u, s.variable_upper_bound, n);
    d.objective_vector = cp(c, s.objective_vector, n);
    d.right_hand_side = cp(b, s.right_hand_side, m);
    d.original_variable_lower_bound = cp(ol, s.original_variable_lower_bound, n);
    d.original_variable_upper_bound = cp(ou, s.original_variable_upper_bound, n);
    d.original_objective_vector = cp(oc, s.original_objective_vector, n);
    d.original_right_hand_side = cp(ob, s.original_right_hand_side, m);
    d.constraint_rescaling = cp(con, s.constraint_rescaling, m);
    d.variable_rescaling = cp(var, s.variable_rescaling, n);
  }
};

struct Request {
  uint64_t ticket = 0;
  HostLp lp;
  gpdhg_params params{};
  double footprint = 0.0;
  bool done = false;
  gpdhg_status status = GPDHG_OK;
  std::string error;
  gpdhg_result result{};
  std::vector<double> x, y;
};

bool same_params(const gpdhg_params& a, const gpdhg_params& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

}  // namespace

// Device bytes one request holds while resident in a batch: the packed CSR of A and A'
// (int32 indices, FP64 values, FP32 values in FP32 runs), the tile plans, the FP64 problem
// vectors (scaled and original, rescaling) and the workspace iterates.
double footprint_bytes(const gpdhg_lp_desc& d, const gpdhg_params& p) {
  const double n = d.num_variables, m = d.num_constraints, z = (double)d.nnz;
  const bool fp64 = p.precision == GPDHG_PRECISION_FP64, refine = p.precision == GPDHG_PRECISION_FP32_REFINE;
  const double t = fp64 ? 8.0 : 4.0;
  double bytes = 2.0 * (z * 12.0 + 4.0 * (n + m + 2.0));  // A and A' CSR
  if (!fp64) bytes += 2.0 * z * 4.0;                      // FP32 values
  const double plans = refine ? 2.0 : 1.0;                // FP32_REFINE: an FP64 plan too
  bytes += plans * 2.0 * 44.0 * (z / 32.0 + (n + m) / 16.0 + 2.0);  // tiles (generous)
  bytes += plans * 2.0 * z * (t + 4.0) * 1.5;              // lane-interleaved tile copies
  bytes += 8.0 * (7.0 * n + 3.0 * m) + m + 4.0 * (n + m);  // FP64 vectors, flags, instance maps
  bytes += t * (13.0 * n + 11.0 * m);                      // workspace iterates
  if (refine) bytes += 8.0 * (13.0 * n + 11.0 * m);        // the FP64 phase's workspace
  return 1.1 * bytes + (1 << 20);
}

// Parameters a batch takes (the rest is served by lone solves).
bool batch_takes(const gpdhg_params& p) {
  return p.precision != GPDHG_PRECISION_FP32_REFINE && p.step_size_policy == GPDHG_STEPSIZE_ADAPTIVE;
}

class Server {
 public:
  explicit Server(const gpdhg_server_config& cfg) : cfg_(cfg) {
    CK(cudaGetDevice(&device_));
    if (cfg_.hbm_budget_bytes <= 0.0) {
      size_t free_b = 0, total_b = 0;
      CK(cudaMemGetInfo(&free_b, &total_b));
      cfg_.hbm_budget_bytes = 0.5 * (double)free_b;
    }
    if (cfg_.max_resident <= 0) cfg_.max_resident = 4096;
    if (cfg_.max_cohort <= 0) cfg_.max_cohort = 256;
    if (cfg_.workers <= 0) cfg_.workers = 2;
    if (cfg_.linger_sec < 0.0) cfg_.linger_sec = 0.0;
    else if (cfg_.linger_sec == 0.0) cfg_.linger_sec = 0.002;
    // twice the cohort slots in threads: a straggling cohort's slot goes to a new cohort
    for (int w = 0; w < 2 * cfg_.workers; ++w) workers_.emplace_back([this] { worker_main(); });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      // requests never started are cancelled; running cohorts finish
      for (auto& r : queue_) {
        r->done = true;
        r->status = GPDHG_ERR_INTERNAL;
        r->error = "server destroyed before the request started";
      }
      queue_.clear();
    }
    cv_work_.notify_all();
    cv_done_.notify_all();
    for (std::thread& t : workers_) t.join();
  }

  uint64_t submit(const gpdhg_lp_desc& d, const gpdhg_params& p) {
    validate_lp_desc(&d, true);
    auto r = std::make_shared<Request>();
    r->params = p;
    r->footprint = footprint_bytes(d, p);
    if (r->footprint > cfg_.hbm_budget_bytes)
      throw Error(GPDHG_ERR_ADMISSION, "request needs about " + std::to_string((long long)r->footprint) +
                                           " device bytes, more than the server's HBM budget");
    r->lp.copy_from(d);
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (stop_) throw Error(GPDHG_ERR_INTERNAL, "server is shutting down");
      r->ticket = next_ticket_++;
      all_[r->ticket] = r;
      queue_.push_back(r);
    }
    cv_work_.notify_one();
    return r->ticket;
  }

  gpdhg_status take(uint64_t ticket, double timeout_sec, gpdhg_result* res, double* x, double* y,
                    std::string& err) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = all_.find(ticket);
    if (it == all_.end()) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "unknown or already collected ticket");
    std::shared_ptr<Request> r = it->second;
    if (!r->done && timeout_sec > 0.0)
      cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_sec), [&] { return r->done; });
    if (!r->done) return GPDHG_ERR_NOT_READY;
    all_.erase(it);
    lk.unlock();
    if (r->status != GPDHG_OK) {
      err = r->error;
      return r->status;
    }
    if (res) *res = r->result;
    if (x && !r->x.empty()) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
    if (y && !r->y.empty()) std::memcpy(y, r->y.data(), sizeof(double) * r->y.size());
    return GPDHG_OK;
  }

 private:
  // Takes the next cohort off the queue (lock held); empty when there is nothing to do.
  std::vector<std::shared_ptr<Request>> pick_cohort(double& fp) {
    std::vector<std::shared_ptr<Request>> cohort;
    fp = 0.0;
    if (queue_.empty()) return cohort;
    const gpdhg_params head = queue_.front()->params;
    for (auto it = queue_.begin(); it != queue_.end() && (int)cohort.size() < cfg_.max_cohort;) {
      const bool fits = in_use_ + fp + (*it)->footprint <= cfg_.hbm_budget_bytes &&
                        resident_ + (int)cohort.size() < cfg_.max_resident;
      if (same_params((*it)->params, head) && fits) {
        fp += (*it)->footprint;
        cohort.push_back(*it);
        it = queue_.erase(it);
      } else if (cohort.empty() && same_params((*it)->params, head)) {
        break;  // the head itself does not fit yet: wait for memory
      } else {
        ++it;
      }
    }
    in_use_ += fp;
    resident_ += (int)cohort.size();
    return cohort;
  }

  // A cohort slot is free: fewer cohorts hold one than `workers` (stragglers hold none).
  bool slot_free() const { return active_cohorts_ - straggling_cohorts_ < cfg_.workers; }

  void worker_main() {
    cudaSetDevice(device_);
    while (true) {
      std::vector<std::shared_ptr<Request>> cohort;
      double fp = 0.0;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] { return stop_ || (!queue_.empty() && slot_free()); });
        if (stop_) return;
        if ((int)queue_.size() < cfg_.max_cohort && cfg_.linger_sec > 0.0)
          cv_work_.wait_for(lk, std::chrono::duration<double>(cfg_.linger_sec),
                            [&] { return stop_ || (int)queue_.size() >= cfg_.max_cohort; });
        if (stop_) return;
        if (!slot_free()) continue;
        cohort = pick_cohort(fp);
        if (cohort.empty()) {
          // the head waits for memory held by running cohorts (their end notifies)
          if (!queue_.empty() && resident_ > 0) cv_work_.wait(lk);
          continue;
        }
        ++active_cohorts_;
      }
      bool straggling = false;
      if (batch_takes(cohort.front()->params)) solve(cohort, straggling);
      else solve_alone(cohort);
      {
        std::lock_guard<std::mutex> lk(mu_);
        in_use_ -= fp;
        resident_ -= (int)cohort.size();
        for (auto& r : cohort) r->done = true;
        --active_cohorts_;
        if (straggling) --straggling_cohorts_;
      }
      cv_done_.notify_all();
      cv_work_.notify_all();
    }
  }

  // `straggling` is set (under the lock, with straggling_cohorts_) when at most a quarter of
  // the cohort's instances are still running.
  void solve(std::vector<std::shared_ptr<Request>>& cohort, bool& straggling) {
    const int k = (int)cohort.size();
    std::vector<gpdhg_lp_desc> descs(k);
    std::vector<gpdhg_result> results(k);
    std::vector<double*> xs(k), ys(k);
    for (int q = 0; q < k; ++q) {
      Request& r = *cohort[q];
      descs[q] = r.lp.d;
      r.x.assign((size_t)r.lp.d.num_variables, 0.0);
      r.y.assign((size_t)r.lp.d.num_constraints, 0.0);
      xs[q] = r.x.data();
      ys[q] = r.y.empty() ? nullptr : r.y.data();
    }
    gpdhg_status status = GPDHG_OK;
    std::string error;
    gpdhg_batch* b = nullptr;
    // an instance's result is handed out as soon as it has terminated
    int running = k;
    const std::function<void(int)> retire = [&](int q) {
      bool freed_slot = false;
      {
        std::lock_guard<std::mutex> lk(mu_);
        Request& r = *cohort[q];
        r.status = GPDHG_OK;
        r.result = results[q];
        r.done = true;
        --running;
        if (!straggling && k > 1 && 4 * running <= k && running > 0) {
          straggling = true;
          ++straggling_cohorts_;
          freed_slot = true;
        }
      }
      cv_done_.notify_all();
      if (freed_slot) cv_work_.notify_all();
    };
    try {
      b = new gpdhg_batch();
      batch_init(b, k, descs.data());
      for (int q = 0; q < k; ++q) cohort[q]->lp = HostLp();   // packed on the device: the copy can go
      batch_solve(b, cohort.front()->params, results.data(), xs.data(), ys.data(), &retire);
    } catch (const Error& e) {
      status = e.status;
      error = e.what();
    } catch (const std::bad_alloc&) {
      status = GPDHG_ERR_OUT_OF_MEMORY;
      error = "host allocation failed";
    } catch (const std::exception& e) {
      status = GPDHG_ERR_INTERNAL;
      error = e.what();
    }
    delete b;
    std::lock_guard<std::mutex> lk(mu_);
    for (int q = 0; q < k; ++q) {
      Request& r = *cohort[q];
      if (r.done) continue;   // handed out at its retirement
      r.status = status == GPDHG_OK ? GPDHG_ERR_INTERNAL : status;
      r.error = status == GPDHG_OK ? "the batch ended before this instance terminated" : error;
      r.lp = HostLp();
    }
  }

  // Requests a batch does not take: each solved as a lone problem, its result handed out
  // when it is done.
  void solve_alone(std::vector<std::shared_ptr<Request>>& cohort) {
    for (auto& rp : cohort) {
      Request& r = *rp;
      r.x.assign((size_t)r.lp.d.num_variables, 0.0);
      r.y.assign((size_t)r.lp.d.num_constraints, 0.0);
      gpdhg_status status = GPDHG_OK;
      std::string error;
      gpdhg_result result{};
      gpdhg_problem* p = nullptr;
      try {
        p = new gpdhg_problem();
        problem_init(p, &r.lp.d);
        gpdhg::solve(p, r.params, &result, r.x.data(), r.y.empty() ? nullptr : r.y.data());
        to_caller_columns(p->col_perm, r.x.data());
      } catch (const Error& e) {
        status = e.status;
        error = e.what();
      } catch (const std::bad_alloc&) {
        status = GPDHG_ERR_OUT_OF_MEMORY;
        error = "host allocation failed";
      } catch (const std::exception& e) {
        status = GPDHG_ERR_INTERNAL;
        error = e.what();
      }
      delete p;
      {
        std::lock_guard<std::mutex> lk(mu_);
        r.status = status;
        r.error = error;
        r.result = result;
        r.lp = HostLp();
        r.done = true;
      }
      cv_done_.notify_all();
    }
  }

  gpdhg_server_config cfg_;
  int device_ = 0;
  std::mutex mu_;
  std::condition_variable cv_work_;  // queue, memory or shutdown changed
  std::condition_variable cv_done_;  // a request finished
  std::deque<std::shared_ptr<Request>> queue_;
  std::map<uint64_t, std::shared_ptr<Request>> all_;  // submitted and not collected
  double in_use_ = 0.0;
  int resident_ = 0;
  int active_cohorts_ = 0;       // cohorts being solved
  int straggling_cohorts_ = 0;   // of those, the ones that gave up their slot
  uint64_t next_ticket_ = 1;
  bool stop_ = false;
  std::vector<std::thread> workers_;
};

}  // namespace gpdhg

struct gpdhg_server {
  std::unique_ptr<gpdhg::Server> impl;
};

namespace gpdhg {
gpdhg_server* server_create(const gpdhg_server_config& cfg) {
  auto* s = new gpdhg_server();
  try {
    s->impl.reset(new Server(cfg));
  } catch (...) {
    delete s;
    throw;
  }
  return s;
}
void server_destroy(gpdhg_server* s) { delete s; }
uint64_t server_submit(gpdhg_server* s, const gpdhg_lp_desc& d, const gpdhg_params& p) {
  return s->impl->submit(d, p);
}
gpdhg_status server_take(gpdhg_server* s, uint64_t ticket, double timeout_sec, gpdhg_result* r, double* x,
                         double* y, std::string& err) {
  return s->impl->take(ticket, timeout_sec, r, x, y, err);
}
}  // namespace gpdhg
