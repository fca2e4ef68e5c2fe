// Batched and served proving: a pool of host workers, each driving its own CUDA stream, that
// takes whole-proof jobs from a queue. Many proofs in flight keep the GPU busy while each
// proof's host-side transcript steps (channel draws, decommitment reads) wait on their own
// stream, and small proofs that cannot fill 152 SMs alone overlap with one another.
//
// Admission: a job starts only when the device bytes it is estimated to need fit in the budget
// next to the jobs already running (a job larger than the whole budget runs alone). Among the
// queued jobs the first one, in submission order, that fits is started next.
//
// Stream priorities: a small proof is a chain of about a hundred short launches, and behind the
// wide kernels of a large proof each of them waits for whole waves of blocks, so that a 1 ms
// proof took 50 ms next to two 2^20-row proofs. Each worker therefore owns one stream per
// priority level and starts a job on the level of its size: jobs under 256 MB of device bytes on
// the highest, jobs under 2 GB on the next, and larger jobs on the levels below in the order they
// start (each below every large job still running), so that large proofs that overlap finish one
// after another instead of all late. Priorities only order the dispatch of waiting blocks; a
// lower-priority proof still takes every SM the others leave idle. A batch (stwo_prove_batch)
// is judged by its total time, not by the latency of each proof, and runs without priorities.
//
// The reference proves one statement per call (crates/prover/src/core/prover/mod.rs:27-79) and
// has no scheduler; this runtime only multiplexes calls of stwo_prove_wide_fib,
// stwo_prove_poseidon and stwo_prove_blake_round, whose results are unchanged by it.
#include "common.cuh"
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <algorithm>
#include <unordered_map>

namespace stwo {
namespace {

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Pending {
  uint64_t ticket;
  stwo_proof_job job;
  size_t bytes;
  Clock::time_point submitted;
};

struct Done {
  stwo_proof_result r;
};

constexpr uint32_t PRIO_LEVELS = 6;
constexpr size_t SMALL_JOB_BYTES = (size_t)256 << 20;
constexpr size_t LARGE_JOB_BYTES = (size_t)2 << 30;

}  // namespace

// Device bytes a job is expected to hold at its peak: evaluations on the blowup domain, the
// extended composition domain, coefficients and Merkle layers of every committed column.
size_t job_hbm_bytes(const stwo_proof_job& j) {
  const size_t n = (size_t)1 << j.log_n_rows;
  const size_t blow = (size_t)1 << j.cfg.log_blowup_factor;
  if (j.air == STWO_AIR_POSEIDON) {
    const size_t cols = 1264 + 32 + 8;
    return cols * n * 4 * (1 + blow + 4) + 64 * n * blow + (64u << 20);
  }
  if (j.air == STWO_AIR_BLAKE_ROUND) {
    const size_t cols = 384 + 260 + 8;
    return cols * n * 4 * (1 + blow + 2) + 64 * n * blow + (64u << 20);
  }
  const size_t cols = j.n_cols + 4;
  return cols * n * 4 * (2 + blow + 2) + 64 * n * blow + (64u << 20);
}

int32_t run_job(const stwo_proof_job& j, cudaStream_t s, stwo_proof_result& r) {
  r.len = 0;
  if (j.air == STWO_AIR_POSEIDON) {
    return stwo_prove_poseidon(j.log_n_rows, j.d_init, j.cfg, j.h_proof, j.capacity, &r.len, &r.claimed_sum, s);
  }
  if (j.air == STWO_AIR_BLAKE_ROUND) {
    return stwo_prove_blake_round(j.log_n_rows, j.d_init, j.cfg, j.h_proof, j.capacity, &r.len, &r.claimed_sum, s);
  }
  STWO_REQUIRE(j.air == STWO_AIR_WIDE_FIB, "unknown AIR %u", j.air);
  STWO_REQUIRE(j.d_a && j.d_b, "wide-Fibonacci job without its first two columns");
  STWO_REQUIRE(j.n_cols >= 3 && j.n_cols <= MAX_PARAM_COLS && j.log_n_rows <= 28, "bad wide-Fibonacci shape");
  const size_t n = (size_t)1 << j.log_n_rows;
  uint32_t* block = nullptr;
  int32_t st = scratch_alloc((void**)&block, (size_t)j.n_cols * n * 4, s);
  if (st) return st;
  std::vector<uint32_t*> cols(j.n_cols);
  for (uint32_t c = 0; c < j.n_cols; c++) cols[c] = block + (size_t)c * n;
  st = stwo_gen_wide_fib_trace(j.log_n_rows, j.n_cols, j.d_a, j.d_b, cols.data(), s);
  if (!st) st = stwo_prove_wide_fib(j.log_n_rows, j.n_cols, cols.data(), j.cfg, j.h_proof, j.capacity, &r.len, s);
  scratch_free(block, s);
  std::memset(&r.claimed_sum, 0, sizeof(r.claimed_sum));
  return st;
}

}  // namespace stwo

using namespace stwo;

struct stwo_server_s {
  int device = 0;
  size_t budget = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::unordered_map<uint64_t, Done> done;
  size_t in_flight_bytes = 0;
  uint32_t running = 0;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::vector<std::thread> workers;
  std::vector<cudaStream_t> streams;  // `levels` per worker, highest priority first
  uint32_t levels = 1;                 // PRIO_LEVELS, or 1 without priorities
  uint32_t level_use[PRIO_LEVELS] = {};

  // Priority level of a job that starts now (called with mu held).
  uint32_t level_for(size_t bytes) const {
    if (levels == 1 || bytes < SMALL_JOB_BYTES) return 0;
    if (bytes < LARGE_JOB_BYTES) return 1;
    uint32_t lv = 2;
    for (uint32_t k = 2; k < PRIO_LEVELS; k++)
      if (level_use[k]) lv = k + 1;
    return std::min(lv, PRIO_LEVELS - 1);
  }

  // The first queued job that fits next to the running ones (any job when nothing runs).
  bool pick(Pending& out) {
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      if (running == 0 || in_flight_bytes + it->bytes <= budget) {
        out = *it;
        queue.erase(it);
        return true;
      }
    }
    return false;
  }

  void work(const cudaStream_t* level_streams) {
    cudaSetDevice(device);
    for (;;) {
      Pending p{};
      bool got = false;
      uint32_t level = 0;
      {
        // After stop the queue is drained before the workers leave.
        std::unique_lock<std::mutex> g(mu);
        cv_work.wait(g, [&] {
          got = pick(p);
          return got || (stop && queue.empty());
        });
        if (!got) break;
        running++;
        in_flight_bytes += p.bytes;
        level = level_for(p.bytes);
        level_use[level]++;
      }
      stwo_proof_result r{};
      const Clock::time_point t0 = Clock::now();
      r.status = run_job(p.job, level_streams[level], r);
      if (r.status != STWO_OK) {
        std::snprintf(r.error, sizeof(r.error), "%s", stwo_last_error());
      }
      const Clock::time_point t1 = Clock::now();
      r.queue_ms = ms_between(p.submitted, t0);
      r.run_ms = ms_between(t0, t1);
      r.latency_ms = ms_between(p.submitted, t1);
      {
        std::lock_guard<std::mutex> g(mu);
        running--;
        in_flight_bytes -= p.bytes;
        level_use[level]--;
        done[p.ticket] = Done{r};
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

namespace {

stwo_status server_create(uint32_t n_workers, size_t hbm_budget_bytes, int device, bool priorities,
                          stwo_server* out) {
  STWO_REQUIRE(out && n_workers >= 1 && n_workers <= 256, "server: 1..256 workers");
  STWO_CHECK_CUDA(cudaSetDevice(device));
  STWO_CHECK_CUDA(cudaFree(nullptr));
  if (hbm_budget_bytes == 0) {
    size_t free_b = 0, total = 0;
    STWO_CHECK_CUDA(cudaMemGetInfo(&free_b, &total));
    hbm_budget_bytes = free_b / 10 * 9;
  }
  int least = 0, greatest = 0;
  STWO_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  auto* srv = new stwo_server_s();
  srv->device = device;
  srv->budget = hbm_budget_bytes;
  srv->levels = priorities ? PRIO_LEVELS : 1;
  for (uint32_t i = 0; i < n_workers * srv->levels; i++) {
    cudaStream_t s = nullptr;
    const int prio = std::min(least, greatest + (int)(i % srv->levels));
    cudaError_t e = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio);
    if (e != cudaSuccess) {
      for (cudaStream_t t : srv->streams) cudaStreamDestroy(t);
      delete srv;
      set_error("server: stream creation failed: %s", cudaGetErrorString(e));
      return STWO_ERR_CUDA;
    }
    srv->streams.push_back(s);
  }
  for (uint32_t i = 0; i < n_workers; i++) {
    const cudaStream_t* level_streams = srv->streams.data() + (size_t)i * srv->levels;
    srv->workers.emplace_back([srv, level_streams] { srv->work(level_streams); });
  }
  *out = srv;
  return STWO_OK;
}

}  // namespace

extern "C" {

size_t stwo_job_hbm_bytes(const stwo_proof_job* job) { return job ? job_hbm_bytes(*job) : 0; }

stwo_status stwo_server_create(uint32_t n_workers, size_t hbm_budget_bytes, int device, stwo_server* out) {
  return server_create(n_workers, hbm_budget_bytes, device, true, out);
}

stwo_status stwo_server_submit(stwo_server srv, const stwo_proof_job* job, uint64_t* ticket) {
  STWO_REQUIRE(srv && job && ticket, "server: null argument");
  STWO_REQUIRE(job->h_proof, "server: job without a proof buffer");
  {
    std::lock_guard<std::mutex> g(srv->mu);
    STWO_REQUIRE(!srv->stop, "server: stopped");
    *ticket = srv->next_ticket++;
    srv->queue.push_back(Pending{*ticket, *job, job_hbm_bytes(*job), Clock::now()});
  }
  srv->cv_work.notify_one();
  return STWO_OK;
}

stwo_status stwo_server_wait(stwo_server srv, uint64_t ticket, stwo_proof_result* out) {
  STWO_REQUIRE(srv && out, "server: null argument");
  std::unique_lock<std::mutex> g(srv->mu);
  STWO_REQUIRE(ticket >= 1 && ticket < srv->next_ticket, "server: unknown ticket %llu", (unsigned long long)ticket);
  srv->cv_done.wait(g, [&] { return srv->done.count(ticket) > 0; });
  *out = srv->done[ticket].r;
  srv->done.erase(ticket);
  return STWO_OK;
}

stwo_status stwo_server_destroy(stwo_server srv) {
  if (!srv) return STWO_OK;
  {
    std::lock_guard<std::mutex> g(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (auto& t : srv->workers) t.join();
  for (cudaStream_t s : srv->streams) cudaStreamDestroy(s);
  delete srv;
  return STWO_OK;
}

stwo_status stwo_prove_batch(const stwo_proof_job* jobs, uint32_t n_jobs, uint32_t n_workers, size_t hbm_budget_bytes,
                             stwo_proof_result* results) {
  STWO_REQUIRE(n_jobs == 0 || (jobs && results), "prove_batch: null argument");
  int dev = 0;
  STWO_CHECK_CUDA(cudaGetDevice(&dev));
  stwo_server srv = nullptr;
  stwo_status st = server_create(n_workers, hbm_budget_bytes, dev, false, &srv);
  if (st) return st;
  // Largest jobs first (by their device-byte estimate, which grows with the work): a large proof
  // submitted last would otherwise run alone at the end of the batch. Results stay in job order.
  std::vector<uint32_t> order(n_jobs);
  for (uint32_t i = 0; i < n_jobs; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return job_hbm_bytes(jobs[a]) > job_hbm_bytes(jobs[b]); });
  std::vector<uint64_t> tickets(n_jobs);
  for (uint32_t k = 0; k < n_jobs && st == STWO_OK; k++) {
    const uint32_t i = order[k];
    st = stwo_server_submit(srv, &jobs[i], &tickets[i]);
  }
  for (uint32_t i = 0; i < n_jobs && st == STWO_OK; i++) st = stwo_server_wait(srv, tickets[i], &results[i]);
  stwo_server_destroy(srv);
  if (st) return st;
  for (uint32_t i = 0; i < n_jobs; i++)
    if (results[i].status != STWO_OK) {
      set_error("prove_batch: job %u failed: %s", i, results[i].error);
      return results[i].status;
    }
  return STWO_OK;
}

}  // extern "C"
