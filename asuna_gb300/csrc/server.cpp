// server.cpp — continuous-batching render server.
//
// Requests (a resident scene + a shot: camera, resolution, spp) arrive at any
// time.  `slots` worker threads each own a context (CUDA stream + wavefront
// buffers), so the work of several requests overlaps on the device.  A slot
// keeps an active set of requests on the same scene and renders them as one
// multi-shot wavefront per chunk of frames; after each chunk, finished
// requests leave the set and pending requests of that scene join it (as long
// as the memory budget admits their films), so new work enters as soon as
// slots and memory free up.  Requests whose footprint can never fit, or that
// arrive while the pending queue is full, are rejected.  Scene BVHs stay
// resident on the device for the lifetime of the server.
//
// Each path's sample stream depends only on (pixel, frame, shot seed), so a
// request renders the same film alone or in any mix (tested).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/asuna_rt.h"
#include "common.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  uint64_t id = 0;
  uint32_t scene = 0;
  asuna_shot shot{};
  double arrival = 0, start = -1, finish = -1;
  uint32_t done = 0;  // frames rendered
  int status = ASUNA_OK;
  uint64_t filmBytes = 0;
  asuna_film* film = nullptr;
  asuna_ctx* filmCtx = nullptr;
};

}  // namespace

struct asuna_server {
  asuna_server_opts opts{};
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<Req>> pending;
  std::vector<std::shared_ptr<Req>> finished;  // not yet polled
  std::unordered_map<uint64_t, std::shared_ptr<Req>> byId;
  std::vector<asuna_scene*> scenes;
  std::vector<uint64_t> sceneBytes;
  std::vector<asuna_ctx*> ctxs;
  std::vector<std::thread> workers;
  uint64_t memUsed = 0;  // films held + scenes
  uint64_t nextId = 1;
  int inFlight = 0;
  bool stop = false;
  uint64_t rejected = 0, admitted = 0, samples = 0;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

uint64_t filmFootprint(const asuna_shot& s) { return uint64_t(s.width) * s.height * 16ull * 9ull; }

// Takes pending requests of `scene` (any scene if scene < 0) that the memory
// budget admits, up to `room`, oldest first.  Caller holds the lock.
void admit(asuna_server* S, int scene, size_t room, std::vector<std::shared_ptr<Req>>& out) {
  for (auto it = S->pending.begin(); it != S->pending.end() && room > 0;) {
    auto& r = *it;
    if (scene >= 0 && int(r->scene) != scene) {
      ++it;
      continue;
    }
    if (S->memUsed + r->filmBytes > S->opts.memory_budget) {
      if (scene < 0) break;  // keep arrival order for new sets
      ++it;
      continue;
    }
    S->memUsed += r->filmBytes;
    r->start = S->now();
    out.push_back(r);
    if (scene < 0) scene = int(r->scene);
    it = S->pending.erase(it);
    --room;
  }
}

void worker(asuna_server* S, int slot) {
  asuna_ctx* ctx = S->ctxs[slot];
  std::vector<std::shared_ptr<Req>> active;
  const size_t maxSet = std::max(1u, S->opts.max_batch);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && !active.empty()) {
        // shutting down: abandon the active set
        for (auto& r : active) {
          r->status = ASUNA_ERR_TIMEOUT;
          r->finish = S->now();
        }
        active.clear();
        S->inFlight--;
        return;
      }
      if (active.empty()) {
        S->cv.wait(lk, [&] { return S->stop || !S->pending.empty(); });
        if (S->stop && S->pending.empty()) return;
        admit(S, -1, maxSet, active);
        if (active.empty()) {
          // nothing fits right now: wait for memory to be released
          S->cv.wait_for(lk, std::chrono::milliseconds(2));
          continue;
        }
        S->inFlight++;
      } else {
        admit(S, int(active[0]->scene), maxSet - active.size(), active);
      }
    }
    // films for newly admitted requests
    for (auto& r : active) {
      if (r->film) continue;
      if (asuna_film_create(ctx, r->shot.width, r->shot.height, &r->film) != ASUNA_OK) {
        r->status = ASUNA_ERR_OOM;
        r->done = r->shot.frames;
      }
      r->filmCtx = ctx;
    }
    // one chunk: every active request advances by up to frames_per_chunk frames
    std::vector<asuna_shot> shots;
    std::vector<asuna_film*> films;
    std::vector<Req*> owners;
    for (auto& r : active) {
      if (r->status != ASUNA_OK || r->done >= r->shot.frames) continue;
      asuna_shot s = r->shot;
      s.frame0 = r->shot.frame0 + r->done;
      s.frames = std::min(S->opts.frames_per_chunk, r->shot.frames - r->done);
      shots.push_back(s);
      films.push_back(r->film);
      owners.push_back(r.get());
    }
    int rc = ASUNA_OK;
    if (!shots.empty()) {
      rc = asuna_render_batch(ctx, S->scenes[active[0]->scene], shots.data(), films.data(), uint32_t(shots.size()),
                              nullptr);
      if (rc == ASUNA_OK) rc = asuna_ctx_sync(ctx);
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const double t = S->now();
      for (size_t k = 0; k < owners.size(); ++k) {
        if (rc != ASUNA_OK) {
          owners[k]->status = rc;
          owners[k]->done = owners[k]->shot.frames;
        } else {
          owners[k]->done += shots[k].frames;
          S->samples += uint64_t(shots[k].frames) * shots[k].width * shots[k].height;
        }
      }
      for (auto it = active.begin(); it != active.end();) {
        auto& r = *it;
        if (r->done >= r->shot.frames) {
          r->finish = t;
          S->finished.push_back(r);
          it = active.erase(it);
        } else {
          ++it;
        }
      }
      if (active.empty()) S->inFlight--;
    }
    S->cv.notify_all();
  }
}

}  // namespace

extern "C" {

int asuna_server_create(const asuna_server_opts* opts, asuna_server** out) {
  asuna::clearError();
  if (!opts || !out) return asuna::fail(ASUNA_ERR_INVALID, "asuna_server_create: null argument");
  if (opts->slots == 0 || opts->slots > 64 || opts->frames_per_chunk == 0)
    return asuna::fail(ASUNA_ERR_INVALID, "asuna_server_create: slots in [1, 64], frames_per_chunk >= 1");
  auto* S = new (std::nothrow) asuna_server;
  if (!S) return asuna::fail(ASUNA_ERR_OOM, "host allocation failed");
  S->opts = *opts;
  if (!S->opts.memory_budget) S->opts.memory_budget = 150ull << 30;
  if (!S->opts.max_queue) S->opts.max_queue = 1u << 20;
  if (!S->opts.max_batch) S->opts.max_batch = 8;
  S->t0 = Clock::now();
  for (uint32_t i = 0; i < opts->slots; ++i) {
    asuna_ctx* c = nullptr;
    int rc = asuna_ctx_create(opts->device, &c);
    if (rc) {
      for (auto* x : S->ctxs) asuna_ctx_destroy(x);
      delete S;
      return rc;
    }
    if (opts->path_budget) asuna_ctx_set_path_budget(c, opts->path_budget);
    S->ctxs.push_back(c);
  }
  for (uint32_t i = 0; i < opts->slots; ++i) S->workers.emplace_back(worker, S, int(i));
  *out = S;
  return ASUNA_OK;
}

int asuna_server_add_scene(asuna_server* S, const asuna_scene_desc* desc, uint32_t* scene_id) {
  asuna::clearError();
  if (!S || !desc || !scene_id) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  asuna_scene* sc = nullptr;
  int rc = asuna_scene_create(S->ctxs[0], desc, &sc);
  if (rc) return rc;
  asuna_scene_stats st;
  asuna_scene_get_stats(sc, &st);
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->memUsed + st.device_bytes > S->opts.memory_budget) {
    asuna_scene_destroy(sc);
    return asuna::fail(ASUNA_ERR_OOM, "scene of %llu bytes exceeds the server memory budget",
                       (unsigned long long)st.device_bytes);
  }
  S->memUsed += st.device_bytes;
  S->scenes.push_back(sc);
  S->sceneBytes.push_back(st.device_bytes);
  *scene_id = uint32_t(S->scenes.size() - 1);
  return ASUNA_OK;
}

int asuna_server_submit(asuna_server* S, const asuna_request* req, uint64_t* id) {
  asuna::clearError();
  if (!S || !req || !id) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  auto r = std::make_shared<Req>();
  r->scene = req->scene;
  r->shot = req->shot;
  r->filmBytes = filmFootprint(req->shot);
  std::lock_guard<std::mutex> lk(S->mu);
  r->id = S->nextId++;
  r->arrival = S->now();
  *id = r->id;
  S->byId[r->id] = r;
  int reason = ASUNA_OK;
  if (req->scene >= S->scenes.size())
    reason = ASUNA_ERR_INVALID;
  else if (req->shot.width == 0 || req->shot.height == 0 || req->shot.frames == 0 ||
           req->shot.state.max_path_depth < 1 || req->shot.state.max_path_depth > 32)
    reason = ASUNA_ERR_INVALID;
  else if (r->filmBytes > S->opts.memory_budget)
    reason = ASUNA_ERR_OOM;  // can never be admitted
  else if (S->pending.size() >= S->opts.max_queue)
    reason = ASUNA_ERR_BUSY;
  if (reason != ASUNA_OK) {
    r->status = reason;
    r->start = r->finish = r->arrival;
    S->finished.push_back(r);
    S->rejected++;
    return ASUNA_OK;  // the rejection is reported through asuna_server_poll
  }
  S->admitted++;
  S->pending.push_back(r);
  S->cv.notify_all();
  return ASUNA_OK;
}

int asuna_server_poll(asuna_server* S, asuna_request_result* out, uint32_t max, uint32_t* n) {
  if (!S || !n || (max && !out)) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  uint32_t k = 0;
  while (k < max && !S->finished.empty()) {
    auto r = S->finished.front();
    S->finished.erase(S->finished.begin());
    asuna_request_result& o = out[k++];
    o.id = r->id;
    o.status = r->status;
    o.scene = r->scene;
    o.arrival_s = r->arrival;
    o.start_s = r->start;
    o.finish_s = r->finish;
    o.samples = uint64_t(r->shot.frames) * r->shot.width * r->shot.height;
  }
  *n = k;
  return ASUNA_OK;
}

int asuna_server_read(asuna_server* S, uint64_t id, int image, float* host_rgba) {
  if (!S) return asuna::fail(ASUNA_ERR_INVALID, "null server");
  std::shared_ptr<Req> r;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->byId.find(id);
    if (it == S->byId.end()) return asuna::fail(ASUNA_ERR_INVALID, "unknown request %llu", (unsigned long long)id);
    r = it->second;
  }
  if (r->status != ASUNA_OK || !r->film) return asuna::fail(ASUNA_ERR_INVALID, "request %llu has no film",
                                                            (unsigned long long)id);
  if (r->finish < 0) return asuna::fail(ASUNA_ERR_INVALID, "request %llu is not finished", (unsigned long long)id);
  return asuna_film_read(r->filmCtx, r->film, image, host_rgba);
}

int asuna_server_release(asuna_server* S, uint64_t id) {
  if (!S) return asuna::fail(ASUNA_ERR_INVALID, "null server");
  std::shared_ptr<Req> r;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->byId.find(id);
    if (it == S->byId.end()) return ASUNA_OK;
    r = it->second;
    if (r->finish < 0) return asuna::fail(ASUNA_ERR_INVALID, "request %llu is not finished", (unsigned long long)id);
    S->byId.erase(it);
    if (r->film) S->memUsed -= r->filmBytes;
  }
  if (r->film) asuna_film_destroy(r->film);
  r->film = nullptr;
  S->cv.notify_all();
  return ASUNA_OK;
}

int asuna_server_drain(asuna_server* S, double timeout_s) {
  if (!S) return asuna::fail(ASUNA_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  bool ok = S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                           [&] { return S->pending.empty() && S->inFlight == 0; });
  return ok ? ASUNA_OK : asuna::fail(ASUNA_ERR_TIMEOUT, "server did not drain within %.1f s", timeout_s);
}

int asuna_server_get_stats(asuna_server* S, asuna_server_stats* out) {
  if (!S || !out) return asuna::fail(ASUNA_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  out->admitted = S->admitted;
  out->rejected = S->rejected;
  out->pending = S->pending.size();
  out->samples = S->samples;
  out->memory_used = S->memUsed;
  out->elapsed_s = S->now();
  return ASUNA_OK;
}

int asuna_server_destroy(asuna_server* S) {
  if (!S) return ASUNA_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->pending.clear();
  }
  S->cv.notify_all();
  for (auto& t : S->workers) t.join();
  for (auto& kv : S->byId)
    if (kv.second->film) asuna_film_destroy(kv.second->film);
  for (auto* sc : S->scenes) asuna_scene_destroy(sc);
  for (auto* c : S->ctxs) asuna_ctx_destroy(c);
  delete S;
  return ASUNA_OK;
}

}  // extern "C"
