// Simulation-job server: continuous batching of whole simulations.
//
// Jobs (a model, its globals, a seed, an initial population and a number of
// timesteps) are submitted from any thread and queue for admission.  A job is
// admitted as soon as one of the server's slots is free AND its estimated
// device memory fits in what is left of the server's HBM budget; an admitted
// job runs in its own runtime context on its own CUDA stream, so the kernels
// of all running jobs overlap on the device, and the next queued job starts
// the moment a running one finishes and releases its slot and memory.  The
// state stays resident on the device for the whole run; the final population
// is copied back to host memory owned by the server until released.
//
// Small jobs are batched: when a worker admits a job of at most
// `batch_agents` agents whose model has an ensemble form, it also admits
// the queued jobs of the same model that are small too (up to
// `batch_jobs`, each as its memory fits), and runs them as the replicas of
// one ensemble in one slot: each phase of a timestep is one launch for all
// of them instead of one per job.  The ensemble runs to each job's
// timestep count in turn; a job's result is read back and the job
// completes when its count is reached.
//
// Each job keeps its submit, admission and completion times (steady clock)
// and the device time of its timesteps, so callers can report latency
// percentiles next to aggregate throughput.  A job computes exactly what the
// same job computes alone: contexts share nothing but the device, and an
// ensemble replica's results equal its own context's bit for bit.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "abl_model.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

size_t member_size(const abl_member_desc &m) { return (size_t) m.components * m.scalar_bytes; }

struct Job {
  long id = 0;
  const abl_model_desc *model = nullptr;
  std::vector<unsigned char> globals;
  uint64_t seed = 0;
  int timesteps = 0;
  // population per type: counts and one host column per member
  std::vector<size_t> counts;
  std::vector<std::vector<std::vector<unsigned char>>> cols;
  size_t reserve = 0;  // bytes of budget held while running
  int status = 0;      // 0 queued, 1 running, 2 done, < 0 error code
  double t_submit = 0, t_admit = 0, t_done = 0, exec_s = 0;
};

}  // namespace

struct abl_server {
  int device = 0;
  size_t budget = 0, in_use = 0;
  int slots = 0, running = 0;
  int batch_jobs = 64;       // replicas of one batch (1: no batching)
  long batch_agents = 65536; // largest job (agents of all types) that is batched
  bool stop = false;
  long next_id = 1;
  std::mutex mu;
  std::condition_variable cv;       // queue, budget and stop changes
  std::condition_variable done_cv;  // job completions
  std::deque<std::shared_ptr<Job>> queue;
  std::map<long, std::shared_ptr<Job>> jobs;
  std::vector<std::thread> workers;
};

namespace {

// Device memory a job needs: both buffers of every column, the binning
// arrays (cell index, rank, slot order, float positions, gathered members,
// neighbourhood lists of up to 27 slots per agent) and spare capacity for
// types whose population changes, plus a fixed allowance for grid arrays.
size_t estimate_bytes(const abl_model_desc *m, const std::vector<size_t> &counts) {
  size_t total = 64u << 20;
  for (int t = 0; t < m->num_agent_types; t++) {
    size_t rec = 0;
    for (int k = 0; k < m->agents[t].num_members; k++) rec += member_size(m->agents[t].members[k]);
    bool dynamic = false;
    for (int s = 0; s < m->num_steps; s++) {
      if (m->steps[s].agent_type == t && m->steps[s].uses_remove) dynamic = true;
      if (m->steps[s].add_type == t) dynamic = true;
    }
    size_t n = counts[t] * (dynamic ? 2 : 1) + (dynamic ? 1024 : 1);
    size_t per = 2 * rec + 4 * 4 + 12 + rec + 27 * 4 + (dynamic ? 2 * rec + 24 : 0);
    total += n * per;
  }
  return total;
}

// Runs one job in a context of its own: its results replace its columns,
// *exec receives the device time of its timesteps.  Returns the status.
int run_alone(Job *job, double *exec) {
  abl_ctx *ctx = nullptr;
  int r = abl_create(job->model, job->reserve, &ctx);
  if (r == ABL_OK) r = abl_set_globals(ctx, job->globals.data(), job->globals.size());
  if (r == ABL_OK) r = abl_set_seed(ctx, job->seed);
  for (int t = 0; r == ABL_OK && t < job->model->num_agent_types; t++) {
    std::vector<const void *> cols;
    for (auto &c : job->cols[t]) cols.push_back(c.data());
    r = abl_upload(ctx, t, cols.data(), job->counts[t]);
  }
  if (r == ABL_OK) r = abl_run(ctx, job->timesteps);
  *exec = 0;
  if (r == ABL_OK) abl_last_exec_time(ctx, exec);
  for (int t = 0; r == ABL_OK && t < job->model->num_agent_types; t++) {
    size_t n = 0;
    r = abl_count(ctx, t, &n);
    if (r != ABL_OK) break;
    std::vector<void *> cols;
    for (int k = 0; k < job->model->agents[t].num_members; k++) {
      job->cols[t][k].resize(std::max<size_t>(1, n * member_size(job->model->agents[t].members[k])));
      cols.push_back(job->cols[t][k].data());
    }
    size_t cap = n;
    r = abl_download(ctx, t, cols.data(), &cap);
    job->counts[t] = n;
  }
  if (ctx) abl_destroy(ctx);
  return r;
}

void run_job(abl_server *S, const std::shared_ptr<Job> &job) {
  double exec = 0;
  const int r = run_alone(job.get(), &exec);
  std::lock_guard<std::mutex> lock(S->mu);
  job->exec_s = exec;
  job->t_done = now_s();
  job->status = r == ABL_OK ? 2 : r;
  S->in_use -= job->reserve;
  S->running--;
  S->cv.notify_all();
  S->done_cv.notify_all();
}

// Every step function has an ensemble form and there is no sequential step.
bool batchable(const abl_model_desc *m) {
  if (m->seq_step || m->num_steps == 0) return false;
  for (int k = 0; k < m->num_steps; k++)
    if (!m->steps[k].launch_ens) return false;
  return true;
}

long job_agents(const Job &j) {
  long n = 0;
  for (size_t c : j.counts) n += (long) c;
  return n;
}

// Runs `jobs` (one model, all admitted) as the replicas of one ensemble.
void run_batch(abl_server *S, const std::vector<std::shared_ptr<Job>> &jobs) {
  const abl_model_desc *m = jobs[0]->model;
  const int R = (int) jobs.size();
  size_t reserve = 0;
  std::vector<unsigned char> globals;
  std::vector<uint64_t> seeds;
  for (auto &j : jobs) {
    reserve += j->reserve;
    globals.insert(globals.end(), j->globals.begin(), j->globals.end());
    seeds.push_back(j->seed);
  }
  // Per-phase launches (graph replay), not the persistent kernel: a
  // persistent launch holds every SM for its whole run, so the kernels of
  // the other running jobs could not interleave with it.
  abl_ensemble *e = nullptr;
  int r = abl_ensemble_create(m, R, globals.data(), seeds.data(), reserve, &e);
  for (int t = 0; r == ABL_OK && t < m->num_agent_types; t++) {
    std::vector<size_t> counts(R);
    std::vector<std::vector<unsigned char>> cat(m->agents[t].num_members);
    for (int q = 0; q < R; q++) {
      counts[q] = jobs[q]->counts[t];
      for (int k = 0; k < m->agents[t].num_members; k++) {
        const auto &c = jobs[q]->cols[t][k];
        cat[k].insert(cat[k].end(), c.begin(), c.end());
      }
    }
    std::vector<const void *> cols;
    for (auto &c : cat) cols.push_back(c.data());
    r = abl_ensemble_upload(e, t, counts.data(), cols.data());
  }
  if (r != ABL_OK) {
    // The ensemble could not be set up (e.g. its memory): the jobs run one
    // after another in this slot instead, each alone.
    if (e) abl_ensemble_destroy(e);
    for (auto &j : jobs) {
      double exec = 0;
      const int rj = run_alone(j.get(), &exec);
      std::lock_guard<std::mutex> lock(S->mu);
      j->exec_s = exec;
      j->t_done = now_s();
      j->status = rj == ABL_OK ? 2 : rj;
      S->done_cv.notify_all();
    }
    std::lock_guard<std::mutex> lock(S->mu);
    S->in_use -= reserve;
    S->running--;
    S->cv.notify_all();
    S->done_cv.notify_all();
    return;
  }
  // Segments: up to each distinct timestep count in turn.
  std::vector<int> order(R);
  for (int q = 0; q < R; q++) order[q] = q;
  std::sort(order.begin(), order.end(),
            [&](int a, int b) { return jobs[a]->timesteps < jobs[b]->timesteps; });
  int done = 0;
  double exec = 0;
  size_t pos = 0;
  while (pos < order.size()) {
    const int target = jobs[order[pos]]->timesteps;
    if (r == ABL_OK && target > done) {
      r = abl_ensemble_run(e, target - done);
      double seg = 0;
      if (r == ABL_OK) abl_ensemble_last_exec_time(e, &seg);
      exec += seg;
      done = target;
    }
    // Read back every replica, keep those finishing here.
    for (int t = 0; r == ABL_OK && t < m->num_agent_types; t++) {
      std::vector<size_t> counts(R);
      r = abl_ensemble_download(e, t, counts.data(), nullptr);
      if (r != ABL_OK) break;
      size_t total = 0;
      for (size_t c : counts) total += c;
      std::vector<std::vector<unsigned char>> cat(m->agents[t].num_members);
      std::vector<void *> cols;
      for (int k = 0; k < m->agents[t].num_members; k++) {
        cat[k].resize(std::max<size_t>(1, total * member_size(m->agents[t].members[k])));
        cols.push_back(cat[k].data());
      }
      r = abl_ensemble_download(e, t, nullptr, cols.data());
      size_t base = 0;
      for (int q = 0; r == ABL_OK && q < R; q++) {
        if (jobs[q]->timesteps == target) {
          jobs[q]->counts[t] = counts[q];
          for (int k = 0; k < m->agents[t].num_members; k++) {
            const size_t b = member_size(m->agents[t].members[k]);
            auto &dst = jobs[q]->cols[t][k];
            dst.assign(cat[k].begin() + base * b, cat[k].begin() + (base + counts[q]) * b);
          }
        }
        base += counts[q];
      }
    }
    std::lock_guard<std::mutex> lock(S->mu);
    for (; pos < order.size() && jobs[order[pos]]->timesteps == target; pos++) {
      Job &j = *jobs[order[pos]];
      j.exec_s = exec;
      j.t_done = now_s();
      j.status = r == ABL_OK ? 2 : r;
    }
    S->done_cv.notify_all();
  }
  if (e) abl_ensemble_destroy(e);
  std::lock_guard<std::mutex> lock(S->mu);
  S->in_use -= reserve;
  S->running--;
  S->cv.notify_all();
  S->done_cv.notify_all();
}

void worker(abl_server *S) {
  cudaSetDevice(S->device);
  for (;;) {
    std::shared_ptr<Job> job;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      // Admit the oldest queued job once it fits in the remaining budget
      // (jobs larger than the whole budget are rejected at submission).
      S->cv.wait(lock, [&] {
        return S->stop || (!S->queue.empty()
                           && S->in_use + S->queue.front()->reserve <= S->budget);
      });
      if (S->stop && S->queue.empty()) return;
      if (S->queue.empty()) continue;
      job = S->queue.front();
      S->queue.pop_front();
      S->in_use += job->reserve;
      S->running++;
      job->status = 1;
      job->t_admit = now_s();
      if (S->batch_jobs > 1 && job_agents(*job) <= S->batch_agents && batchable(job->model)) {
        // Admit the small queued jobs of the same model with it, in queue
        // order, as long as their memory fits.
        std::vector<std::shared_ptr<Job>> batch{job};
        for (auto it = S->queue.begin();
             it != S->queue.end() && (int) batch.size() < S->batch_jobs;) {
          Job &q = **it;
          if (q.model == job->model && job_agents(q) <= S->batch_agents &&
              S->in_use + q.reserve <= S->budget) {
            S->in_use += q.reserve;
            q.status = 1;
            q.t_admit = job->t_admit;
            batch.push_back(*it);
            it = S->queue.erase(it);
          } else {
            ++it;
          }
        }
        if (batch.size() > 1) {
          lock.unlock();
          run_batch(S, batch);
          continue;
        }
      }
    }
    run_job(S, job);
  }
}

}  // namespace

extern "C" {

int abl_server_create(int slots, size_t hbm_budget, abl_server **out) {
  if (slots <= 0 || !out) return ABL_E_INVALID;
  abl_server *S = new abl_server;
  cudaGetDevice(&S->device);
  S->slots = slots;
  if (hbm_budget == 0) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    hbm_budget = free_b / 10 * 9;
  }
  S->budget = hbm_budget;
  for (int k = 0; k < slots; k++) S->workers.emplace_back(worker, S);
  *out = S;
  return ABL_OK;
}

int abl_server_submit(abl_server *S, const abl_job_desc *jd, long *job_id) {
  if (!S || !jd || !jd->model || !jd->counts || jd->timesteps < 0) return ABL_E_INVALID;
  const abl_model_desc *m = jd->model;
  auto job = std::make_shared<Job>();
  job->model = m;
  const unsigned char *g = (const unsigned char *) (jd->globals ? jd->globals
                                                                : m->globals_default);
  job->globals.assign(g, g + m->globals_size);
  job->seed = jd->seed;
  job->timesteps = jd->timesteps;
  job->counts.assign(jd->counts, jd->counts + m->num_agent_types);
  job->cols.resize(m->num_agent_types);
  for (int t = 0; t < m->num_agent_types; t++) {
    for (int k = 0; k < m->agents[t].num_members; k++) {
      size_t bytes = job->counts[t] * member_size(m->agents[t].members[k]);
      const unsigned char *src = bytes ? (const unsigned char *) jd->cols[t][k] : nullptr;
      job->cols[t].emplace_back(src, src + bytes);
    }
  }
  job->reserve = estimate_bytes(m, job->counts);
  std::lock_guard<std::mutex> lock(S->mu);
  if (job->reserve > S->budget) return ABL_E_BUDGET;
  job->id = S->next_id++;
  job->t_submit = now_s();
  S->jobs[job->id] = job;
  S->queue.push_back(job);
  S->cv.notify_all();
  if (job_id) *job_id = job->id;
  return ABL_OK;
}

int abl_server_wait(abl_server *S, long job_id, double timeout_s) {
  if (!S) return ABL_E_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return ABL_E_INVALID;
  auto job = it->second;
  bool ok = S->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_s),
                                [&] { return job->status == 2 || job->status < 0; });
  if (!ok) return ABL_E_TIMEOUT;
  return job->status < 0 ? job->status : ABL_OK;
}

int abl_server_job_info(abl_server *S, long job_id, int *status, double *times) {
  if (!S) return ABL_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return ABL_E_INVALID;
  const Job &j = *it->second;
  if (status) *status = j.status;
  if (times) {
    times[0] = j.t_submit;
    times[1] = j.t_admit;
    times[2] = j.t_done;
    times[3] = j.exec_s;
  }
  return ABL_OK;
}

int abl_server_result(abl_server *S, long job_id, int type_id, void *const *cols, size_t *n) {
  if (!S || !n) return ABL_E_INVALID;
  std::shared_ptr<Job> job;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->jobs.find(job_id);
    if (it == S->jobs.end()) return ABL_E_INVALID;
    job = it->second;
    if (job->status != 2) return job->status < 0 ? job->status : ABL_E_INVALID;
  }
  if (type_id < 0 || type_id >= job->model->num_agent_types) return ABL_E_INVALID;
  size_t cnt = job->counts[type_id];
  if (!cols || *n < cnt) {
    *n = cnt;
    return cols ? ABL_E_INVALID : ABL_OK;
  }
  for (int k = 0; k < job->model->agents[type_id].num_members; k++) {
    size_t bytes = cnt * member_size(job->model->agents[type_id].members[k]);
    if (bytes) std::memcpy(cols[k], job->cols[type_id][k].data(), bytes);
  }
  *n = cnt;
  return ABL_OK;
}

int abl_server_release(abl_server *S, long job_id) {
  if (!S) return ABL_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->jobs.find(job_id);
  if (it == S->jobs.end()) return ABL_E_INVALID;
  if (it->second->status == 0 || it->second->status == 1) return ABL_E_INVALID;
  S->jobs.erase(it);
  return ABL_OK;
}

int abl_server_set_batching(abl_server *S, int max_jobs, long max_agents) {
  if (!S || max_jobs < 1 || max_agents < 0) return ABL_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  S->batch_jobs = max_jobs;
  S->batch_agents = max_agents;
  return ABL_OK;
}

int abl_server_stats(abl_server *S, int *queued, int *running, size_t *bytes_in_use) {
  if (!S) return ABL_E_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  if (queued) *queued = (int) S->queue.size();
  if (running) *running = S->running;
  if (bytes_in_use) *bytes_in_use = S->in_use;
  return ABL_OK;
}

int abl_server_destroy(abl_server *S) {
  if (!S) return ABL_E_INVALID;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  for (auto &w : S->workers) w.join();
  delete S;
  return ABL_OK;
}

}  // extern "C"
