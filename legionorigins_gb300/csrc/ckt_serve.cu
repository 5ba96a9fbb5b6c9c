// ckt_serve.cu -- serving loop: circuit-solve requests arrive over time, are
// admitted under an HBM budget, stay resident on the device, and advance
// together -- every "round" is one persistent launch that runs one outer loop
// of every resident circuit.  Requests join at the next round after their
// upload finishes and leave after their last loop (continuous batching);
// uploads and result downloads run on their own stream, overlapping the
// rounds.
//
// Threads: `prep_threads` workers build each request's circuit and graph on
// the host; one IO thread allocates device memory (stream-ordered pool),
// uploads, downloads results and frees; one scheduler thread admits and runs
// rounds.  No request blocks another: a failing request completes with an
// error status and the others carry on.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "ckt_gen.h"
#include "ckt_round.h"

using namespace ckt;

namespace {

enum JobState { kQueued, kPreparing, kPrepared, kUploading, kResident, kDraining, kDone };

struct Job {
  ckt_request req;
  int64_t W = 0, N = 0;
  JobState state = kQueued;
  int status = CKT_OK;
  bool cancel = false;
  double submit_s = 0, admit_s = 0, start_s = -1, finish_s = 0;
  int32_t loops_done = 0;      // rounds completed
  int32_t loops_enqueued = 0;  // rounds launched (completed or in flight)
  int fail = CKT_OK;           // status of a failed round this job was in
  // host data (prep output)
  std::vector<uint32_t> in_ptr, out_ptr, slot_in, slot_out, ent, off, gstart;
  std::vector<uint8_t> in_loc, out_loc;
  std::vector<float> L, R, C, charge, nvolt, cap, leak;
  // device block and descriptor
  size_t bytes = 0;
  char *dmem = nullptr;
  int32_t *dlocator = nullptr;  // device locator (device generation only)
  RoundCircuit rc;
  cudaEvent_t uploaded = nullptr;
  // results (host)
  std::vector<float> res_cur, res_vol, res_charge, res_nvolt;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Device bytes of a circuit: wires (statics, state, graph, contributions)
// and nodes (state, constants, locator, offsets).
size_t device_bytes_for(int64_t W, int64_t N) {
  size_t b = 0;
  b += align256(W * 4) * 4;      // in_ptr, out_ptr, slot_in, slot_out
  b += align256(W) * 2;          // in_loc, out_loc
  b += align256(W * 4) * 3;      // L, R, C
  b += align256(10 * W * 4);     // current
  b += align256(9 * W * 4);      // voltage
  b += align256(2 * W * 4) * 2;  // ent, contrib
  b += align256(gstart_words(W) * 4);
  b += align256(N * 4) * 5;      // charge, voltage, cap, leak, locator
  b += align256((N + 1) * 4);    // off
  return b;
}

}  // namespace

struct ckt_server {
  ckt_server_config cfg;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_prep, cv_sched, cv_io, cv_done;
  std::deque<std::shared_ptr<Job>> queued, prepared, io_up, io_down;
  std::vector<std::shared_ptr<Job>> resident;  // uploading or resident
  std::map<uint64_t, std::shared_ptr<Job>> jobs;
  std::deque<ckt_completion> completions;
  std::atomic<bool> stop{false};
  uint64_t bytes_in_use = 0, bytes_peak = 0;
  int64_t submitted = 0, completed = 0, rounds = 0, resident_peak = 0;
  double busy_s = 0;
  int device = 0, sm_count = 0, grid = 0;
  cudaStream_t compute = nullptr, io = nullptr;
  // round buffers (device), grown on demand
  BatchItem *d_items = nullptr;
  size_t items_cap = 0;
  RoundCircuit *d_circ = nullptr;
  size_t circ_cap = 0;
  uint32_t *d_sync = nullptr;
  size_t sync_cap = 0;
  // Two rounds may be in flight on the compute stream; each has its own
  // pinned host copy of its tables and error word, and timing events.
  struct Stage {
    BatchItem *items = nullptr;
    size_t items_cap = 0;
    RoundCircuit *circ = nullptr;
    size_t circ_cap = 0;
    uint32_t *err = nullptr;
    cudaEvent_t start = nullptr, end = nullptr;
  } stage[2];
  std::vector<std::thread> prep_threads;
  std::thread io_thread, sched_thread;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

void complete(ckt_server *s, Job &j, int status) {
  // called with s->mu held
  j.status = status;
  j.state = kDone;
  j.finish_s = s->now();
  ckt_completion c;
  memset(&c, 0, sizeof(c));
  c.request_id = j.req.request_id;
  c.status = status;
  c.loops = j.loops_done;
  c.submit_s = j.submit_s;
  c.admit_s = j.admit_s;
  c.start_s = j.start_s;
  c.finish_s = j.finish_s;
  c.wires = j.W;
  c.nodes = j.N;
  c.segment_updates = (double)j.W * CKT_SEGMENTS * j.req.steps * j.loops_done;
  s->completions.push_back(c);
  s->completed++;
  // drop host inputs; keep results only if asked
  std::vector<uint32_t>().swap(j.in_ptr); std::vector<uint32_t>().swap(j.out_ptr);
  std::vector<uint32_t>().swap(j.slot_in); std::vector<uint32_t>().swap(j.slot_out);
  std::vector<uint32_t>().swap(j.ent); std::vector<uint32_t>().swap(j.off);
  std::vector<uint32_t>().swap(j.gstart);
  std::vector<uint8_t>().swap(j.in_loc); std::vector<uint8_t>().swap(j.out_loc);
  std::vector<float>().swap(j.L); std::vector<float>().swap(j.R); std::vector<float>().swap(j.C);
  std::vector<float>().swap(j.charge); std::vector<float>().swap(j.nvolt);
  std::vector<float>().swap(j.cap); std::vector<float>().swap(j.leak);
  if (!s->cfg.keep_results || status != CKT_OK) s->jobs.erase(j.req.request_id);
  s->cv_done.notify_all();
}

int prepare(Job &j) {
  const ckt_gen_params &p = j.req.shape;
  const int64_t W = j.W, N = j.N;
  j.in_ptr.resize(W); j.out_ptr.resize(W); j.in_loc.resize(W); j.out_loc.resize(W);
  j.L.resize(W); j.R.resize(W); j.C.resize(W);
  j.charge.resize(N); j.nvolt.resize(N); j.cap.resize(N); j.leak.resize(N);
  std::vector<int32_t> locator(N);
  float unused = 0.f;
  ckt_host_circuit h = {j.in_ptr.data(), j.out_ptr.data(), j.in_loc.data(), j.out_loc.data(),
                        j.L.data(), j.R.data(), j.C.data(), &unused, &unused, j.charge.data(),
                        j.nvolt.data(), j.cap.data(), j.leak.data(), locator.data()};
  int rc = generate_into(&p, &h, 0);
  if (rc) return rc;
  HostGraph g;
  if ((rc = build_circuit_graph(p, j.in_ptr.data(), j.out_ptr.data(), j.in_loc.data(),
                                j.out_loc.data(), g)))
    return rc;
  j.ent.swap(g.ent); j.off.swap(g.off); j.slot_in.swap(g.slot_in);
  j.slot_out.swap(g.slot_out); j.gstart.swap(g.gstart);
  return CKT_OK;
}

void prep_loop(ckt_server *s) {
  cudaSetDevice(s->device);
  while (true) {
    std::shared_ptr<Job> j;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_prep.wait(lk, [&] { return s->stop || !s->queued.empty(); });
      if (s->stop) return;
      j = s->queued.front();
      s->queued.pop_front();
      if (j->cancel) {
        complete(s, *j, CKT_ECANCELLED);
        continue;
      }
      j->state = kPreparing;
    }
    const int rc = s->cfg.device_generate ? CKT_OK : prepare(*j);
    std::string err = rc ? ckt_last_error() : "";
    std::lock_guard<std::mutex> lk(s->mu);
    if (rc) {
      complete(s, *j, rc);
    } else if (j->cancel) {
      complete(s, *j, CKT_ECANCELLED);
    } else {
      j->state = kPrepared;
      s->prepared.push_back(j);
      s->cv_sched.notify_all();
    }
  }
}

// Carves the circuit's arrays out of its device block.
void layout_device(Job &j) {
  char *p = j.dmem;
  const int64_t W = j.W, N = j.N;
  auto take = [&p](size_t bytes) {
    char *q = p;
    p += align256(bytes);
    return q;
  };
  RoundCircuit &rc = j.rc;
  memset(&rc, 0, sizeof(rc));
  rc.in_ptr = (const uint32_t *)take(W * 4);
  rc.out_ptr = (const uint32_t *)take(W * 4);
  rc.slot_in = (const uint32_t *)take(W * 4);
  rc.slot_out = (const uint32_t *)take(W * 4);
  rc.in_loc = (const uint8_t *)take(W);
  rc.out_loc = (const uint8_t *)take(W);
  rc.L = (const float *)take(W * 4);
  rc.R = (const float *)take(W * 4);
  rc.C = (const float *)take(W * 4);
  rc.cur = (float *)take(10 * W * 4);
  rc.vol = (float *)take(9 * W * 4);
  rc.ent = (const uint32_t *)take(2 * W * 4);
  rc.contrib = (float *)take(2 * W * 4);
  rc.gstart = (const uint32_t *)take(gstart_words(W) * 4);
  rc.charge = (float *)take(N * 4);
  rc.nvolt = (float *)take(N * 4);
  rc.cap = (const float *)take(N * 4);
  rc.leak = (const float *)take(N * 4);
  rc.off = (const uint32_t *)take((N + 1) * 4);
  j.dlocator = (int32_t *)take(N * 4);
  rc.W = (uint32_t)W;
  rc.N = (uint32_t)N;
  rc.steps = j.req.steps;
}

int upload(ckt_server *s, Job &j) {
  const cudaStream_t st = s->io;
  CKT_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&j.dmem), j.bytes, st));
  layout_device(j);
  if (s->cfg.device_generate) {
    RoundCircuit &rc = j.rc;
    ckt_device_circuit d = {const_cast<uint32_t *>(rc.in_ptr), const_cast<uint32_t *>(rc.out_ptr),
                            const_cast<uint8_t *>(rc.in_loc), const_cast<uint8_t *>(rc.out_loc),
                            const_cast<float *>(rc.L), const_cast<float *>(rc.R),
                            const_cast<float *>(rc.C), rc.cur, rc.vol, rc.charge, rc.nvolt,
                            const_cast<float *>(rc.cap), const_cast<float *>(rc.leak), j.dlocator,
                            const_cast<uint32_t *>(rc.off), const_cast<uint32_t *>(rc.ent),
                            const_cast<uint32_t *>(rc.slot_in), const_cast<uint32_t *>(rc.slot_out),
                            const_cast<uint32_t *>(rc.gstart)};
    int r = ckt_generate_device(&j.req.shape, &d, st);
    if (r) return r;
    CKT_CUDA(cudaEventCreateWithFlags(&j.uploaded, cudaEventDisableTiming));
    CKT_CUDA(cudaEventRecord(j.uploaded, st));
    return CKT_OK;
  }
  const RoundCircuit &rc = j.rc;
  const int64_t W = j.W, N = j.N;
  auto h2d = [st](const void *d, const void *h, size_t bytes) {
    return bytes ? cudaMemcpyAsync(const_cast<void *>(d), h, bytes, cudaMemcpyHostToDevice, st)
                 : cudaSuccess;
  };
  CKT_CUDA(h2d(rc.in_ptr, j.in_ptr.data(), W * 4));
  CKT_CUDA(h2d(rc.out_ptr, j.out_ptr.data(), W * 4));
  CKT_CUDA(h2d(rc.slot_in, j.slot_in.data(), W * 4));
  CKT_CUDA(h2d(rc.slot_out, j.slot_out.data(), W * 4));
  CKT_CUDA(h2d(rc.in_loc, j.in_loc.data(), W));
  CKT_CUDA(h2d(rc.out_loc, j.out_loc.data(), W));
  CKT_CUDA(h2d(rc.L, j.L.data(), W * 4));
  CKT_CUDA(h2d(rc.R, j.R.data(), W * 4));
  CKT_CUDA(h2d(rc.C, j.C.data(), W * 4));
  CKT_CUDA(h2d(rc.ent, j.ent.data(), 2 * W * 4));
  CKT_CUDA(h2d(rc.gstart, j.gstart.data(), j.gstart.size() * 4));
  CKT_CUDA(h2d(rc.charge, j.charge.data(), N * 4));
  CKT_CUDA(h2d(rc.nvolt, j.nvolt.data(), N * 4));
  CKT_CUDA(h2d(rc.cap, j.cap.data(), N * 4));
  CKT_CUDA(h2d(rc.leak, j.leak.data(), N * 4));
  CKT_CUDA(h2d(rc.off, j.off.data(), (N + 1) * 4));
  if (W) {
    CKT_CUDA(cudaMemsetAsync(rc.cur, 0, 10 * W * 4, st));
    CKT_CUDA(cudaMemsetAsync(rc.vol, 0, 9 * W * 4, st));
  }
  CKT_CUDA(cudaEventCreateWithFlags(&j.uploaded, cudaEventDisableTiming));
  CKT_CUDA(cudaEventRecord(j.uploaded, st));
  return CKT_OK;
}

int download(ckt_server *s, Job &j) {
  const cudaStream_t st = s->io;
  const RoundCircuit &rc = j.rc;
  const int64_t W = j.W, N = j.N;
  j.res_cur.resize(10 * W);
  j.res_vol.resize(9 * W);
  j.res_charge.resize(N);
  j.res_nvolt.resize(N);
  if (W) {
    CKT_CUDA(cudaMemcpyAsync(j.res_cur.data(), rc.cur, 10 * W * 4, cudaMemcpyDeviceToHost, st));
    CKT_CUDA(cudaMemcpyAsync(j.res_vol.data(), rc.vol, 9 * W * 4, cudaMemcpyDeviceToHost, st));
  }
  CKT_CUDA(cudaMemcpyAsync(j.res_charge.data(), rc.charge, N * 4, cudaMemcpyDeviceToHost, st));
  CKT_CUDA(cudaMemcpyAsync(j.res_nvolt.data(), rc.nvolt, N * 4, cudaMemcpyDeviceToHost, st));
  CKT_CUDA(cudaStreamSynchronize(st));
  return CKT_OK;
}

void release(ckt_server *s, Job &j) {
  // called without s->mu
  if (j.dmem) cudaFreeAsync(j.dmem, s->io);
  j.dmem = nullptr;
  if (j.uploaded) cudaEventDestroy(j.uploaded);
  j.uploaded = nullptr;
}

void io_loop(ckt_server *s) {
  cudaSetDevice(s->device);
  while (true) {
    std::shared_ptr<Job> j;
    bool up = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_io.wait(lk, [&] { return s->stop || !s->io_up.empty() || !s->io_down.empty(); });
      if (s->stop) return;
      // results first: they free memory for admissions
      if (!s->io_down.empty()) {
        j = s->io_down.front();
        s->io_down.pop_front();
      } else {
        j = s->io_up.front();
        s->io_up.pop_front();
        up = true;
      }
    }
    int rc = up ? upload(s, *j)
                : ((s->cfg.keep_results && j->status == CKT_OK) ? download(s, *j) : CKT_OK);
    if (!up && j->status != CKT_OK) rc = j->status;  // the round failed
    if (!up || rc) {
      release(s, *j);
      cudaStreamSynchronize(s->io);
    } else {
      // Pageable uploads are staged before cudaMemcpyAsync returns: the host
      // inputs are no longer needed.
      std::vector<uint32_t>().swap(j->in_ptr); std::vector<uint32_t>().swap(j->out_ptr);
      std::vector<uint32_t>().swap(j->slot_in); std::vector<uint32_t>().swap(j->slot_out);
      std::vector<uint32_t>().swap(j->ent); std::vector<uint32_t>().swap(j->off);
      std::vector<uint32_t>().swap(j->gstart);
      std::vector<uint8_t>().swap(j->in_loc); std::vector<uint8_t>().swap(j->out_loc);
      std::vector<float>().swap(j->L); std::vector<float>().swap(j->R);
      std::vector<float>().swap(j->C); std::vector<float>().swap(j->charge);
      std::vector<float>().swap(j->nvolt); std::vector<float>().swap(j->cap);
      std::vector<float>().swap(j->leak);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (up && rc == CKT_OK) {
      j->state = kResident;  // joins a round once its upload event completes
    } else {
      s->bytes_in_use -= j->bytes;
      s->resident.erase(std::remove(s->resident.begin(), s->resident.end(), j), s->resident.end());
      complete(s, *j, rc);
      s->cv_sched.notify_all();
    }
  }
}

template <typename T>
int ensure_cap(T **p, size_t *cap, size_t need) {
  if (*cap >= need) return CKT_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  const size_t n = std::max<size_t>(need * 2, 64);
  CKT_CUDA(cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T)));
  *cap = n;
  return CKT_OK;
}

template <typename T>
int ensure_host_cap(T **p, size_t *cap, size_t need) {
  if (*cap >= need) return CKT_OK;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  const size_t n = std::max<size_t>(need * 2, 64);
  CKT_CUDA(cudaMallocHost(reinterpret_cast<void **>(p), n * sizeof(T)));
  *cap = n;
  return CKT_OK;
}

// A round launched on the compute stream and not yet retired.
struct InFlight {
  int slot;
  std::vector<std::shared_ptr<Job>> jobs;
};

// Sends a job whose rounds are all retired to the IO thread (download,
// release) when it is finished, cancelled or failed.  Called with s->mu held.
void maybe_drain(ckt_server *s, const std::shared_ptr<Job> &j) {
  if (j->state != kResident || j->loops_enqueued != j->loops_done) return;
  if (!(j->fail || j->cancel || j->loops_done >= j->req.loops)) return;
  s->resident.erase(std::remove(s->resident.begin(), s->resident.end(), j), s->resident.end());
  if (j->fail) j->status = j->fail;
  else if (j->loops_done < j->req.loops) j->status = CKT_ECANCELLED;
  j->state = kDraining;
  s->io_down.push_back(j);
}

// Retires the oldest round: waits for its end event, reads its error word,
// advances its jobs.
void retire_round(ckt_server *s, InFlight &f) {
  ckt_server::Stage &st = s->stage[f.slot];
  int rc = cudaEventSynchronize(st.end) == cudaSuccess ? CKT_OK : CKT_ECUDA;
  if (rc) set_error(CKT_ECUDA, "round failed: %s", cudaGetErrorString(cudaGetLastError()));
  else if (*st.err) rc = set_error(CKT_ETIMEOUT, "a round's bounded wait ran out");
  float ms = 0.f;
  if (!rc) cudaEventElapsedTime(&ms, st.start, st.end);
  std::lock_guard<std::mutex> lk(s->mu);
  s->rounds++;
  s->busy_s += 1e-3 * ms;
  for (auto &j : f.jobs) {
    j->loops_done++;
    if (rc && !j->fail) j->fail = rc;
    maybe_drain(s, j);
  }
  s->cv_io.notify_all();
}

// Builds and launches one round over `jobs` into stage `slot`.  Buffers that
// must grow are grown only with no round in flight (the caller retires them
// first when grow_needed says so).
bool grow_needed(const ckt_server *s, int slot, size_t nitems, size_t ncirc) {
  const ckt_server::Stage &st = s->stage[slot];
  return nitems > s->items_cap || ncirc > s->circ_cap || 2 + 2 * ncirc > s->sync_cap ||
         nitems > st.items_cap || ncirc > st.circ_cap || st.err == nullptr;
}

int launch_staged_round(ckt_server *s, int slot, const std::vector<RoundCircuit> &circ,
                        const std::vector<BatchItem> &items) {
  ckt_server::Stage &st = s->stage[slot];
  int rc;
  if ((rc = ensure_cap(&s->d_items, &s->items_cap, std::max<size_t>(items.size(), 1))) ||
      (rc = ensure_cap(&s->d_circ, &s->circ_cap, circ.size())) ||
      (rc = ensure_cap(&s->d_sync, &s->sync_cap, 2 + 2 * circ.size())) ||
      (rc = ensure_host_cap(&st.items, &st.items_cap, std::max<size_t>(items.size(), 1))) ||
      (rc = ensure_host_cap(&st.circ, &st.circ_cap, circ.size())))
    return rc;
  if (!st.err) CKT_CUDA(cudaMallocHost(reinterpret_cast<void **>(&st.err), sizeof(uint32_t)));
  memcpy(st.items, items.data(), items.size() * sizeof(BatchItem));
  memcpy(st.circ, circ.data(), circ.size() * sizeof(RoundCircuit));
  *st.err = 0;
  CKT_CUDA(cudaEventRecord(st.start, s->compute));
  CKT_CUDA(cudaMemcpyAsync(s->d_items, st.items, items.size() * sizeof(BatchItem),
                           cudaMemcpyHostToDevice, s->compute));
  CKT_CUDA(cudaMemcpyAsync(s->d_circ, st.circ, circ.size() * sizeof(RoundCircuit),
                           cudaMemcpyHostToDevice, s->compute));
  if ((rc = launch_round(s->cfg.mode, s->cfg.launch, s->grid, s->d_items, (uint32_t)items.size(),
                         s->d_circ, (uint32_t)circ.size(), s->d_sync, s->cfg.round_timeout_ns,
                         s->compute)))
    return rc;
  CKT_CUDA(cudaMemcpyAsync(st.err, s->d_sync + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           s->compute));
  CKT_CUDA(cudaEventRecord(st.end, s->compute));
  return CKT_OK;
}

// The scheduler keeps up to two rounds in flight: the next round's members
// are known before the current one ends (every resident circuit with loops
// left, plus circuits whose upload has finished), so it is launched right
// behind it on the stream and the GPU does not wait for the host between
// rounds.  Circuits join and leave at round boundaries.
void sched_loop(ckt_server *s) {
  cudaSetDevice(s->device);
  std::deque<InFlight> inflight;
  std::vector<RoundCircuit> circ;
  std::vector<BatchItem> items;
  int slot = 0;
  while (true) {
    std::vector<std::shared_ptr<Job>> next;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->stop) break;
      // Admission: prepared requests, first come first served, while slots
      // and the HBM budget allow.  A request larger than the whole budget
      // can never run: it completes with CKT_ENOMEM.
      while (!s->prepared.empty()) {
        std::shared_ptr<Job> j = s->prepared.front();
        if (j->cancel) {
          s->prepared.pop_front();
          complete(s, *j, CKT_ECANCELLED);
          continue;
        }
        if (j->bytes > s->cfg.hbm_budget_bytes) {
          s->prepared.pop_front();
          complete(s, *j, CKT_ENOMEM);
          continue;
        }
        if ((int64_t)s->resident.size() >= s->cfg.max_circuits ||
            s->bytes_in_use + j->bytes > s->cfg.hbm_budget_bytes)
          break;
        s->prepared.pop_front();
        s->bytes_in_use += j->bytes;
        s->bytes_peak = std::max(s->bytes_peak, s->bytes_in_use);
        j->admit_s = s->now();
        j->state = kUploading;
        s->resident.push_back(j);
        s->resident_peak = std::max<int64_t>(s->resident_peak, (int64_t)s->resident.size());
        s->io_up.push_back(j);
        s->cv_io.notify_all();
      }
      const std::vector<std::shared_ptr<Job>> res = s->resident;
      for (auto &j : res) {
        if (j->state != kResident || !j->uploaded) continue;
        if (j->loops_enqueued == 0 && cudaEventQuery(j->uploaded) != cudaSuccess) continue;
        maybe_drain(s, j);  // cancelled or failed with nothing in flight
        if (j->state == kResident && !j->fail && !j->cancel && j->loops_enqueued < j->req.loops)
          next.push_back(j);
      }
      s->cv_io.notify_all();
      if (next.empty() && inflight.empty()) {
        s->cv_sched.wait_for(lk, std::chrono::microseconds(200));
        continue;
      }
    }
    if (next.empty() || inflight.size() >= 2) {
      retire_round(s, inflight.front());
      inflight.pop_front();
      continue;
    }
    circ.resize(next.size());
    for (size_t k = 0; k < next.size(); k++) circ[k] = next[k]->rc;
    build_round_table(circ, s->cfg.launch, items);
    if (grow_needed(s, slot, items.size(), circ.size()) && !inflight.empty()) {
      // buffers are reallocated only with nothing in flight
      while (!inflight.empty()) {
        retire_round(s, inflight.front());
        inflight.pop_front();
      }
      continue;  // membership may have changed
    }
    NvtxRange range("ckt_server_round");
    const int rc = items.empty() ? CKT_OK : launch_staged_round(s, slot, circ, items);
    std::lock_guard<std::mutex> lk(s->mu);
    const double t = s->now();
    for (auto &j : next) {
      if (rc) {
        j->fail = rc;
        maybe_drain(s, j);
        continue;
      }
      if (j->start_s < 0) j->start_s = t;
      j->loops_enqueued++;
      if (items.empty()) {  // nothing to run: the round is done already
        j->loops_done++;
        maybe_drain(s, j);
      }
    }
    if (!rc && !items.empty()) {
      inflight.push_back({slot, next});
      slot ^= 1;
    }
    s->cv_io.notify_all();
  }
}

}  // namespace

extern "C" {

void ckt_server_default_config(ckt_server_config *c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->hbm_budget_bytes = 80ull << 30;
  c->max_circuits = 4096;
  c->prep_threads = (int32_t)std::max(1u, std::thread::hardware_concurrency());
  c->mode = CKT_MODE_EXACT;
  c->keep_results = 0;
  c->round_timeout_ns = 5000000000ull;
  c->launch.block = 128;
  c->launch.wires_per_thread = 2;
  c->launch.dc_schedule = 0;
  c->device_generate = 1;
}

int ckt_server_create(const ckt_server_config *cfg, ckt_server **out) {
  CKT_REQUIRE(cfg != nullptr && out != nullptr, "NULL argument");
  *out = nullptr;
  CKT_REQUIRE(cfg->mode == CKT_MODE_EXACT || cfg->mode == CKT_MODE_FAST, "unknown mode %d", cfg->mode);
  CKT_REQUIRE(cfg->max_circuits >= 1 && cfg->prep_threads >= 1 && cfg->hbm_budget_bytes > 0,
              "bad server configuration");
  int rc = check_batch_config(&cfg->launch);
  if (rc) return rc;
  std::unique_ptr<ckt_server> s(new ckt_server());
  s->cfg = *cfg;
  if (s->cfg.round_timeout_ns == 0) s->cfg.round_timeout_ns = 5000000000ull;
  s->t0 = std::chrono::steady_clock::now();
  CKT_CUDA(cudaGetDevice(&s->device));
  CKT_CUDA(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
  int per_sm = 1;
  if ((rc = round_blocks_per_sm(s->cfg.launch, &per_sm))) return rc;
  s->cfg.launch.blocks_per_sm = per_sm;
  s->grid = s->sm_count * per_sm;
  // Rounds outrank circuit building and copies: when a round ends, the next
  // round's blocks are dispatched before the generator's and the copies'.
  int least = 0, greatest = 0;
  CKT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CKT_CUDA(cudaStreamCreateWithPriority(&s->compute, cudaStreamNonBlocking, greatest));
  CKT_CUDA(cudaStreamCreateWithPriority(&s->io, cudaStreamNonBlocking, least));
  for (auto &st : s->stage) {
    CKT_CUDA(cudaEventCreate(&st.start));
    CKT_CUDA(cudaEventCreate(&st.end));
  }
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  ckt_server *p = s.release();
  for (int t = 0; t < p->cfg.prep_threads; t++) p->prep_threads.emplace_back(prep_loop, p);
  p->io_thread = std::thread(io_loop, p);
  p->sched_thread = std::thread(sched_loop, p);
  *out = p;
  return CKT_OK;
}

int ckt_server_submit(ckt_server *s, const ckt_request *r) {
  CKT_REQUIRE(s != nullptr && r != nullptr, "NULL argument");
  const ckt_gen_params &p = r->shape;
  CKT_REQUIRE(p.num_pieces >= 1 && p.nodes_per_piece >= 1 && p.wires_per_piece >= 0,
              "request %llu has a bad shape", (unsigned long long)r->request_id);
  CKT_REQUIRE(r->steps >= 0 && r->loops >= 1, "request %llu: steps >= 0 and loops >= 1",
              (unsigned long long)r->request_id);
  const int64_t W = (int64_t)p.num_pieces * p.wires_per_piece;
  const int64_t N = (int64_t)p.num_pieces * p.nodes_per_piece;
  CKT_REQUIRE(W <= kMaxWires && N < 0x7fffffffLL, "request %llu is too large",
              (unsigned long long)r->request_id);
  auto j = std::make_shared<Job>();
  j->req = *r;
  j->W = W;
  j->N = N;
  j->bytes = device_bytes_for(W, N);
  std::lock_guard<std::mutex> lk(s->mu);
  CKT_REQUIRE(s->jobs.find(r->request_id) == s->jobs.end(), "request id %llu is in use",
              (unsigned long long)r->request_id);
  j->submit_s = s->now();
  s->jobs[r->request_id] = j;
  s->queued.push_back(j);
  s->submitted++;
  s->cv_prep.notify_one();
  return CKT_OK;
}

int ckt_server_cancel(ckt_server *s, uint64_t request_id) {
  CKT_REQUIRE(s != nullptr, "server is NULL");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(request_id);
  CKT_REQUIRE(it != s->jobs.end(), "unknown request %llu", (unsigned long long)request_id);
  it->second->cancel = true;
  return CKT_OK;
}

int ckt_server_poll(ckt_server *s, ckt_completion *out, int32_t capacity, int32_t *count) {
  CKT_REQUIRE(s != nullptr && count != nullptr && (capacity == 0 || out != nullptr),
              "bad arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  int32_t n = 0;
  while (n < capacity && !s->completions.empty()) {
    out[n++] = s->completions.front();
    s->completions.pop_front();
  }
  *count = n;
  return CKT_OK;
}

int ckt_server_wait(ckt_server *s, double timeout_s) {
  CKT_REQUIRE(s != nullptr, "server is NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                      [&] { return s->completed >= s->submitted; });
  if (!ok)
    return set_error(CKT_ETIMEOUT, "%lld of %lld requests still open after %.3f s",
                     (long long)(s->submitted - s->completed), (long long)s->submitted, timeout_s);
  return CKT_OK;
}

int ckt_server_take_result(ckt_server *s, uint64_t request_id, float *current, float *voltage,
                           float *charge, float *node_voltage) {
  CKT_REQUIRE(s != nullptr, "server is NULL");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(request_id);
  CKT_REQUIRE(it != s->jobs.end() && it->second->state == kDone,
              "no finished result for request %llu (keep_results must be set)",
              (unsigned long long)request_id);
  Job &j = *it->second;
  if (current) memcpy(current, j.res_cur.data(), j.res_cur.size() * 4);
  if (voltage) memcpy(voltage, j.res_vol.data(), j.res_vol.size() * 4);
  if (charge) memcpy(charge, j.res_charge.data(), j.res_charge.size() * 4);
  if (node_voltage) memcpy(node_voltage, j.res_nvolt.data(), j.res_nvolt.size() * 4);
  s->jobs.erase(it);
  return CKT_OK;
}

int ckt_server_get_stats(ckt_server *s, ckt_server_stats *out) {
  CKT_REQUIRE(s != nullptr && out != nullptr, "NULL argument");
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rounds = s->rounds;
  out->resident_peak = s->resident_peak;
  out->bytes_in_use = s->bytes_in_use;
  out->bytes_peak = s->bytes_peak;
  out->busy_s = s->busy_s;
  out->clock_s = s->now();
  return CKT_OK;
}

double ckt_server_clock(const ckt_server *s) { return s ? s->now() : 0.0; }

int ckt_server_destroy(ckt_server *s) {
  if (!s) return CKT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_prep.notify_all();
  s->cv_io.notify_all();
  s->cv_sched.notify_all();
  for (auto &t : s->prep_threads) t.join();
  if (s->sched_thread.joinable()) s->sched_thread.join();
  if (s->io_thread.joinable()) s->io_thread.join();
  cudaStreamSynchronize(s->compute);
  cudaStreamSynchronize(s->io);
  for (auto &kv : s->jobs) release(s, *kv.second);
  for (auto &j : s->resident) release(s, *j);
  cudaStreamSynchronize(s->io);
  cudaFree(s->d_items);
  cudaFree(s->d_circ);
  cudaFree(s->d_sync);
  for (auto &st : s->stage) {
    if (st.items) cudaFreeHost(st.items);
    if (st.circ) cudaFreeHost(st.circ);
    if (st.err) cudaFreeHost(st.err);
    if (st.start) cudaEventDestroy(st.start);
    if (st.end) cudaEventDestroy(st.end);
  }
  cudaStreamDestroy(s->compute);
  cudaStreamDestroy(s->io);
  delete s;
  return CKT_OK;
}

}  // extern "C"
