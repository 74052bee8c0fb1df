// gpv_serve.cu -- continuous-batching voxelization server.
//
// Requests (host triangles in caller-owned memory that stays valid until completion, plus a
// grid) arrive at any time.  Worker threads, each with its own context and stream, repeatedly
// take every request that is waiting and fits the HBM budget (FIFO, by a predicted device
// footprint), copy their triangles into one device buffer, and voxelize them with one batched
// launch sequence (run_batch).  Requests that arrive while batches are on the GPU are admitted
// into the next batch as soon as a worker and budget free up; with two workers, two batches are
// in flight on the device at once.  Results stay on the device until the client releases them,
// and their bytes count against the budget until then.
//
// Meshes can also be made resident: gpv_server_add_mesh uploads a mesh once into the server's
// device pool (its bytes count against the budget while it stays), and gpv_server_submit_mesh
// requests it by id, so a batch reads it in place with no host-to-device copy.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gpv_ctx.h"

namespace gpv {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  const float *h_tris = nullptr;
  const float *d_tris = nullptr;  // a resident mesh's device triangles (no copy), else null
  uint64_t mesh_id = 0;           // the resident mesh, 0 for host triangles
  int64_t T = 0;
  gpv_grid_spec spec{};
  Clock::time_point t_submit, t_start, t_done;
  int64_t pred = 0;        // predicted device bytes (workspace + results)
  int64_t res_bytes = 0;   // predicted result bytes, held until release
  int status = GPV_ERR_PENDING;
  gpv_result res{};
  int worker = -1;
};

// Predicted device footprint of one voxelization: inputs, per-triangle workspace, planes,
// pairs (from a candidate-count estimate) and the outputs (from a boundary-voxel estimate).
void predict(Request &r) {
  int64_t N1 = 1, surf = 0;
  const int *n = r.spec.ndiv;
  for (int a = 0; a < 3; ++a) N1 *= std::max(n[a], 1);
  surf = 2 * ((int64_t)n[0] * n[1] + (int64_t)n[1] * n[2] + (int64_t)n[0] * n[2]);
  const int64_t cells = (int64_t)r.spec.ndiv2[0] * r.spec.ndiv2[1] * r.spec.ndiv2[2];
  const int64_t B = std::min(N1, 2 * surf);
  const int64_t pairs = 8 * r.T + 4 * B;
  const int64_t work = (r.d_tris ? 0 : 36 * r.T) + 80 * r.T + N1 / 2 + 40 * pairs + 24 * B;
  r.res_bytes = 5 * N1 + B * (4 + cells);
  r.pred = work + r.res_bytes + (1 << 20);
}

// A mesh kept in the server's device pool (gpv_server_add_mesh).
struct ResidentMesh {
  float *d_tris = nullptr;
  int64_t T = 0, bytes = 0;
  int64_t refs = 0;  // pending or running requests that read it
};

}  // namespace
}  // namespace gpv

using namespace gpv;

struct gpv_server {
  std::unordered_map<uint64_t, ResidentMesh> meshes;
  uint64_t next_mesh = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> all;
  int64_t budget = 0, in_use = 0;
  int max_batch = 256;
  int64_t max_pending = 1 << 20;
  uint64_t next = 1;
  bool stop = false;
  int device = 0;
  std::vector<std::thread> workers;
  std::vector<gpv_ctx *> ctxs;
  std::vector<cudaStream_t> streams;
  // results released by clients, freed by their worker between batches: a worker's stream is
  // recorded into CUDA graphs while it runs a batch, so no other thread may enqueue on it
  std::vector<std::vector<gpv_result>> to_free;
  uint64_t batches = 0, served = 0;
};

namespace {

void worker_loop(gpv_server *srv, int w) {
  cudaSetDevice(srv->device);
  gpv_ctx *ctx = srv->ctxs[w];
  cudaStream_t s = srv->streams[w];
  std::vector<gpv_result> frees;
  for (;;) {
    std::vector<Request *> batch;
    int64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->cv_work.wait(lk, [&] {
        return srv->stop || !srv->to_free[w].empty() ||
               (!srv->pending.empty() && srv->in_use + srv->pending.front()->pred <= srv->budget);
      });
      if (srv->stop) return;  // the destroy call frees what is left
      frees.swap(srv->to_free[w]);
      if (!frees.empty()) {
        lk.unlock();
        for (gpv_result &r : frees) gpv_result_release(ctx, &r);
        frees.clear();
        continue;
      }
      while (!srv->pending.empty() && (int)batch.size() < srv->max_batch) {
        Request *r = srv->pending.front();
        if (srv->in_use + bytes + r->pred > srv->budget) break;
        bytes += r->pred;
        batch.push_back(r);
        srv->pending.pop_front();
      }
      srv->in_use += bytes;
    }
    const auto t0 = Clock::now();
    const int n = (int)batch.size();
    std::vector<int64_t> off(n + 1, 0), T(n);
    std::vector<gpv_grid_spec> specs(n);
    for (int i = 0; i < n; ++i) {
      T[i] = batch[i]->T;
      specs[i] = batch[i]->spec;
      // host triangles get 16-byte aligned slots of one device buffer; resident ones none
      off[i + 1] = off[i] + (batch[i]->d_tris ? 0 : ((T[i] * 9 + 3) / 4) * 4);
      batch[i]->t_start = t0;
      batch[i]->worker = w;
    }
    float *d = nullptr;
    int rc = GPV_OK;
    if (off[n] > 0)
      rc = (cudaMallocAsync((void **)&d, off[n] * sizeof(float), s) == cudaSuccess) ? GPV_OK : GPV_ERR_OOM;
    std::vector<const float *> ptrs(n);
    for (int i = 0; i < n && rc == GPV_OK; ++i) {
      if (batch[i]->d_tris) {  // resident: read in place
        ptrs[i] = batch[i]->d_tris;
        continue;
      }
      ptrs[i] = d + off[i];
      if (T[i] > 0 &&
          cudaMemcpyAsync(d + off[i], batch[i]->h_tris, T[i] * 9 * sizeof(float),
                          cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = GPV_ERR_CUDA;
    }
    std::vector<gpv_result> res(n);
    if (rc == GPV_OK) rc = run_batch(ctx, n, ptrs.data(), T.data(), specs.data(), res.data(), s);
    if (d) cudaFreeAsync(d, s);
    cudaStreamSynchronize(s);
    const auto t1 = Clock::now();
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      for (int i = 0; i < n; ++i) {
        Request *r = batch[i];
        r->t_done = t1;
        r->status = rc;
        if (r->mesh_id) {
          auto mt = srv->meshes.find(r->mesh_id);
          if (mt != srv->meshes.end()) mt->second.refs--;
        }
        if (rc == GPV_OK) {
          r->res = res[i];
          srv->in_use -= r->pred - r->res_bytes;  // workspace returns now, results on release
        } else {
          srv->in_use -= r->pred;
        }
      }
      srv->batches++;
      srv->served += n;
    }
    srv->cv_done.notify_all();
    srv->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int gpv_server_create(int device, int64_t budget_bytes, int32_t workers, int32_t max_batch,
                      gpv_server **out) {
  if (!out || budget_bytes <= 0 || workers < 1 || workers > 8 || max_batch < 1) return GPV_ERR_INVALID;
  *out = nullptr;
  auto *srv = new gpv_server();
  srv->device = device;
  srv->budget = budget_bytes;
  srv->max_batch = max_batch;
  for (int w = 0; w < workers; ++w) {
    gpv_ctx *ctx = nullptr;
    int rc = gpv_init(device, &ctx);
    cudaStream_t s = nullptr;
    if (rc == GPV_OK && cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      rc = GPV_ERR_CUDA;
    if (rc != GPV_OK) {
      if (ctx) gpv_destroy(ctx);
      for (size_t k = 0; k < srv->ctxs.size(); ++k) {
        gpv_destroy(srv->ctxs[k]);
        cudaStreamDestroy(srv->streams[k]);
      }
      delete srv;
      return rc;
    }
    srv->ctxs.push_back(ctx);
    srv->streams.push_back(s);
  }
  srv->to_free.resize(workers);
  for (int w = 0; w < workers; ++w) srv->workers.emplace_back(worker_loop, srv, w);
  *out = srv;
  return GPV_OK;
}

int gpv_server_set_tunables(gpv_server *srv, int32_t tile, int32_t level2_chunk) {
  if (!srv) return GPV_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  for (gpv_ctx *c : srv->ctxs) {
    if (gpv_set_tile(c, tile) != GPV_OK || gpv_set_level2_chunk(c, level2_chunk) != GPV_OK)
      return GPV_ERR_INVALID;
  }
  return GPV_OK;
}

int gpv_server_submit(gpv_server *srv, const float *h_tris, int64_t num_triangles,
                      const gpv_grid_spec *spec, uint64_t *ticket) {
  if (!srv || !spec || !ticket || num_triangles < 0 || (num_triangles > 0 && !h_tris))
    return GPV_ERR_INVALID;
  auto r = std::make_unique<Request>();
  r->h_tris = h_tris;
  r->T = num_triangles;
  r->spec = *spec;
  predict(*r);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (r->pred > srv->budget || (int64_t)srv->pending.size() >= srv->max_pending)
      return GPV_ERR_BUDGET;
    r->ticket = srv->next++;
    *ticket = r->ticket;
    srv->pending.push_back(r.get());
    srv->all.emplace(r->ticket, std::move(r));
  }
  srv->cv_work.notify_one();
  return GPV_OK;
}

int gpv_server_add_mesh(gpv_server *srv, const float *h_tris, int64_t num_triangles,
                        uint64_t *mesh_id) {
  if (!srv || !mesh_id || num_triangles <= 0 || !h_tris || num_triangles >= ((int64_t)1 << 31))
    return GPV_ERR_INVALID;
  const int64_t bytes = num_triangles * 9 * (int64_t)sizeof(float);
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->in_use + bytes > srv->budget) return GPV_ERR_BUDGET;
    srv->in_use += bytes;  // reserved while the upload runs
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(srv->device);
  float *d = nullptr;
  int rc = GPV_OK;
  if (cudaMalloc(&d, bytes) != cudaSuccess) {
    cudaGetLastError();
    rc = GPV_ERR_OOM;
  } else if (cudaMemcpy(d, h_tris, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    rc = GPV_ERR_CUDA;
  }
  cudaSetDevice(prev);
  std::lock_guard<std::mutex> lk(srv->mu);
  if (rc != GPV_OK) {
    srv->in_use -= bytes;
    return rc;
  }
  ResidentMesh m;
  m.d_tris = d;
  m.T = num_triangles;
  m.bytes = bytes;
  *mesh_id = srv->next_mesh++;
  srv->meshes.emplace(*mesh_id, m);
  return GPV_OK;
}

int gpv_server_submit_mesh(gpv_server *srv, uint64_t mesh_id, const gpv_grid_spec *spec,
                           uint64_t *ticket) {
  if (!srv || !spec || !ticket) return GPV_ERR_INVALID;
  auto r = std::make_unique<Request>();
  r->spec = *spec;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto mt = srv->meshes.find(mesh_id);
    if (mt == srv->meshes.end()) return GPV_ERR_NOTFOUND;
    r->d_tris = mt->second.d_tris;
    r->T = mt->second.T;
    r->mesh_id = mesh_id;
    predict(*r);
    if (r->pred > srv->budget || (int64_t)srv->pending.size() >= srv->max_pending)
      return GPV_ERR_BUDGET;
    mt->second.refs++;
    r->ticket = srv->next++;
    *ticket = r->ticket;
    srv->pending.push_back(r.get());
    srv->all.emplace(r->ticket, std::move(r));
  }
  srv->cv_work.notify_one();
  return GPV_OK;
}

int gpv_server_remove_mesh(gpv_server *srv, uint64_t mesh_id) {
  if (!srv) return GPV_ERR_INVALID;
  ResidentMesh m;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto mt = srv->meshes.find(mesh_id);
    if (mt == srv->meshes.end()) return GPV_ERR_NOTFOUND;
    if (mt->second.refs > 0) return GPV_ERR_PENDING;  // requests still read it
    m = mt->second;
    srv->meshes.erase(mt);
    srv->in_use -= m.bytes;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(srv->device);
  cudaFree(m.d_tris);  // waits for any work still reading it
  cudaSetDevice(prev);
  srv->cv_work.notify_all();
  return GPV_OK;
}

// Waits up to timeout_ms (0: do not wait, <0: forever) for a request; on completion fills the
// result (device arrays owned by the server until gpv_server_release) and the latency.
int gpv_server_poll(gpv_server *srv, uint64_t ticket, int32_t timeout_ms, gpv_result *out,
                    double *latency_ms, double *queue_ms) {
  if (!srv) return GPV_ERR_INVALID;
  std::unique_lock<std::mutex> lk(srv->mu);
  auto it = srv->all.find(ticket);
  if (it == srv->all.end()) return GPV_ERR_NOTFOUND;
  Request *r = it->second.get();
  auto ready = [&] { return r->status != GPV_ERR_PENDING; };
  if (!ready()) {
    if (timeout_ms == 0) return GPV_ERR_PENDING;
    if (timeout_ms < 0) srv->cv_done.wait(lk, ready);
    else if (!srv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
      return GPV_ERR_PENDING;
  }
  if (out) *out = r->res;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
  return r->status;
}

int gpv_server_release(gpv_server *srv, uint64_t ticket) {
  if (!srv) return GPV_ERR_INVALID;
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->all.find(ticket);
    if (it == srv->all.end()) return GPV_ERR_NOTFOUND;
    if (it->second->status == GPV_ERR_PENDING) return GPV_ERR_PENDING;
    r = std::move(it->second);
    srv->all.erase(it);
    if (r->status == GPV_OK) srv->in_use -= r->res_bytes;
    if (r->status == GPV_OK && r->worker >= 0) srv->to_free[r->worker].push_back(r->res);
  }
  srv->cv_work.notify_all();
  return GPV_OK;
}

int gpv_server_stats(gpv_server *srv, int64_t *in_use_bytes, int64_t *pending, uint64_t *batches,
                     uint64_t *served) {
  if (!srv) return GPV_ERR_INVALID;
  std::lock_guard<std::mutex> lk(srv->mu);
  if (in_use_bytes) *in_use_bytes = srv->in_use;
  if (pending) *pending = (int64_t)srv->pending.size();
  if (batches) *batches = srv->batches;
  if (served) *served = srv->served;
  return GPV_OK;
}

void gpv_server_destroy(gpv_server *srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->cv_work.notify_all();
  for (auto &t : srv->workers) t.join();
  for (size_t k = 0; k < srv->ctxs.size(); ++k) {
    for (gpv_result &r : srv->to_free[k]) gpv_result_release(srv->ctxs[k], &r);
    cudaStreamSynchronize(srv->streams[k]);
    gpv_destroy(srv->ctxs[k]);
    cudaStreamDestroy(srv->streams[k]);
  }
  if (!srv->meshes.empty()) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(srv->device);
    for (auto &kv : srv->meshes) cudaFree(kv.second.d_tris);
    cudaSetDevice(prev);
  }
  delete srv;
}

}  // extern "C"
